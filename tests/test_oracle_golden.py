"""The CPU oracle against golden vectors produced by the reference's own
kernels on a GB300 (tests/golden/make_golden.py).  No GPU needed."""
import hashlib
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kernels.npz")


@pytest.fixture(scope="module")
def g():
    if not os.path.exists(GOLDEN):
        pytest.skip("golden fixture not generated")
    return dict(np.load(GOLDEN))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def bits(a):
    a = np.asarray(a)
    return a.view(np.int32) if a.dtype == np.float32 else a


@pytest.mark.parametrize("site", ["s1", "s2"])
def test_search_kernels_restatement(g, site):
    F, R = g[site + "_F"], g[site + "_R"]
    chunks = sorted({k.split("_")[1] for k in g if k.startswith(site + "_c")})
    assert chunks
    for c in chunks:
        key = "%s_%s" % (site, c)
        IBB, NBB, vn = g[key + "_IBB"], g[key + "_NBB"], g[key + "_vn"]
        D, I = O.search_min_drift(F, IBB, NBB, vn, 1024)
        assert [sha(D), sha(I)] == list(g[key + "_min_sha"]), key
        v, m = O.post_sort_knn(D, I, 30)
        assert np.array_equal(bits(v), bits(g[key + "_min_vrKnn"])) and np.array_equal(m, g[key + "_min_miKnn"])
        D, I = O.search_delta_drift(F, R, IBB, NBB, vn, 512)
        assert [sha(D), sha(I)] == list(g[key + "_delta_sha"]), key
        v, m = O.post_min(D, I)
        assert np.array_equal(bits(v), bits(g[key + "_delta_min"])) and np.array_equal(m, g[key + "_delta_idx"])


def test_cuda_knn_index_restatement(g):
    K, I = O.cuda_knn_index(g["knn_B"], g["knn_A"], 30)
    assert np.array_equal(bits(K), bits(g["knn_K"])) and np.array_equal(I, g["knn_I"])


def test_cuda_delta_knn_restatement(g):
    D, N = O.cuda_delta_knn(g["knn_B"], g["knn_A"], g["dknn_RB"], g["dknn_RA"])
    assert np.array_equal(bits(D), bits(g["dknn_D"]))
    assert np.array_equal(N.view(np.int32), g["dknn_N"])


def test_rho_drift_restatement(g):
    site = np.stack([g["rho_s1"], g["rho_s2"]], 1)
    rho = O.rho_drift(site, g["rho_f1"], g["rho_f2"], 200, float(g["rho_dc2"]))
    assert np.array_equal(bits(rho), bits(g["rho_out"]))


def test_delta_drift_restatement(g):
    site = np.stack([g["rho_s1"], g["rho_s2"]], 1)
    de, nn = O.delta_drift(site, g["rho_f1"], g["rho_f2"], g["ddrift_rho"], 200, float(g["rho_dc2"]))
    assert np.array_equal(bits(de), bits(g["ddrift_delta"]))
    assert np.array_equal(nn.view(np.int32), g["ddrift_nn"])


def test_cuda_knn_variants_restatement(g):
    B, A = g["knn_B"], g["knn_A"]
    assert np.array_equal(bits(O.cuda_knn(B, A, 30)), bits(g["cknn_K"]))
    K, I = O.cuda_knn_full(B, A, 30)
    assert np.array_equal(bits(K), bits(g["cknnf_K"])) and np.array_equal(I, g["cknnf_I"])
    K, I = O.cuda_knn_ib(B, A, g["cknnib_IB"], 30)
    assert np.array_equal(bits(K), bits(g["cknnib_K"])) and np.array_equal(I, g["cknnib_I"])


@pytest.mark.parametrize("fdc", [0, 1])
def test_spacetime_rho_delta_restatement(g, fdc):
    F, ordr, rr = g["st_F"], g["st_ord"], g["st_rr"]
    dc2 = g["st%d_dc2" % fdc]
    rho = O.cuda_rho(F, ordr, 300, 60, dc2, fdc)
    assert np.array_equal(bits(rho), bits(g["st%d_rho" % fdc]))
    de, nn = O.cuda_delta(F, ordr, rr, 300, 60, dc2, fdc)
    assert np.array_equal(bits(de), bits(g["st%d_delta" % fdc]))
    assert np.array_equal(nn.view(np.int32), g["st%d_nn" % fdc])


def test_planted_mistake_is_caught(g):
    """A one-ulp change in one feature must change the restated output."""
    F = g["s1_F"].copy()
    key = "s1_c0"
    q = int(g[key + "_vn"][3])
    F[q, 0] = np.nextafter(F[q, 0], np.float32(np.inf))
    D, I = O.search_min_drift(F, g[key + "_IBB"], g[key + "_NBB"], g[key + "_vn"], 1024)
    assert [sha(D), sha(I)] != list(g[key + "_min_sha"])
