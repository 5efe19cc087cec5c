"""The clustering step after the path on the GPU (irc_sort_rho,
irc_assign_cluster_knn) against the C oracle, bit for bit.

Labels, centres, counts and the order are integers and must be identical;
the normalised rho must match bit for bit (one IEEE single division)."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import _lib, irc, synth
from oracle import oracle as O
from tests.cases import small_site
from tests.cluster_cases import geometric_case, random_case
from tests.test_oracle_cluster import CASES

pytestmark = pytest.mark.gpu


def _same_f32(a, b):
    """Bit-identical floats; NaN matches NaN whatever its payload (the GPU
    returns the canonical NaN, the CPU propagates the input's)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(a)
    np.testing.assert_array_equal(a[ok].view(np.uint32), b[ok].view(np.uint32))


def _cmp(gpu_out, ref):
    for k in ("nClu", "nClu_pre", "nClu_post"):
        assert gpu_out[k] == ref[k], (k, gpu_out[k], ref[k])
    for k in ("viClu", "icl", "vnSpk_clu"):
        np.testing.assert_array_equal(gpu_out[k].cpu().numpy(), ref[k], err_msg=k)


@pytest.mark.parametrize("n,nan", [(1, False), (777, False), (5000, True), (1_000_000, True)])
def test_sort_rho_matches_oracle(gpu, n, nan):
    rng = np.random.default_rng(n)
    rho = rng.gamma(2.0, 1.0, n).astype(np.float32)
    rho[::7] = rho[0]                                # ties (also after the division)
    rho[1::11] = np.round(rho[1::11], 1)
    if nan:
        rho[rng.random(n) < 0.01] = np.nan
    r_ref, o_ref = O.sort_rho(rho)
    r, o = irc.sort_rho(rho)
    _same_f32(r.cpu().numpy(), r_ref)
    np.testing.assert_array_equal(o.cpu().numpy(), o_ref)


def test_sort_rho_all_nan(gpu):
    rho = np.full(100, np.nan, np.float32)
    r, o = irc.sort_rho(rho)
    r_ref, o_ref = O.sort_rho(rho)
    assert np.isnan(r.cpu().numpy()).all()
    np.testing.assert_array_equal(o.cpu().numpy(), o_ref)


@pytest.mark.parametrize("case", CASES, ids=[str(c["seed"]) for c in CASES])
@pytest.mark.parametrize("min_count", [0, 5])
def test_assign_matches_oracle(gpu, case, min_count):
    rho, delta, ordrho, nneigh, mk = random_case(**case)
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, min_count)
    _cmp(irc.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, min_count), ref)


@pytest.mark.parametrize("cut", [1.0, 1e30, 0.0])
def test_assign_peak_count_edges(gpu, cut):
    rho, delta, ordrho, nneigh, mk = random_case(11, n=200)
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, cut, 3)
    _cmp(irc.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, cut, 3), ref)


def test_assign_single_spike(gpu):
    one = np.ones(1, np.float32)
    ref = O.assign_cluster_knn(one, one, [1], [1], [[1]], 1.0, 0)
    _cmp(irc.assign_cluster_knn(one, one, [1], [1], [[1]], 1.0, 0), ref)


def test_assign_many_peaks(gpu):
    """~19k peaks: a 19k x 19k bit matrix, sparse overlaps, many clusters."""
    rho, delta, ordrho, nneigh, mk = random_case(21, n=100000, knn=8, vocab=3_000_000, delta_scale=1.0)
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 2)
    assert ref["nClu_pre"] > 15000
    _cmp(irc.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 2), ref)


def test_assign_deep_chains(gpu):
    """nneigh chains thousands of spikes deep (every spike points to the one
    ranked just above it): the pointer jumping needs more than one batch of
    rounds."""
    n = 200_000
    rng = np.random.default_rng(5)
    rho = np.sort(rng.random(n).astype(np.float32))[::-1].copy()
    rho, ordrho = O.sort_rho(rho)
    nneigh = np.empty(n, np.int64)
    nneigh[ordrho[1:] - 1] = ordrho[:-1]
    nneigh[ordrho[0] - 1] = ordrho[0]
    delta = np.zeros(n, np.float32)
    delta[ordrho[[0, n // 3, 2 * n // 3]] - 1] = 5.0            # three peaks -> three long chains
    mk = np.arange(1, n + 1, dtype=np.int64)[:, None].repeat(3, 1)
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 0)
    assert ref["nClu"] == 3
    _cmp(irc.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 0), ref)


def test_assign_geometric(gpu):
    rho, delta, ordrho, nneigh, mk = geometric_case(3, n=1500)
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 10)
    _cmp(irc.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 10), ref)


def _site_clustering_inputs(F, plan, mode):
    """rho, delta, nneigh and kNN of one single-page site through the fused
    path, then sort_'s normalisation on the device."""
    Fd = torch.from_numpy(F).to("cuda")
    k = irc.knn_rho_delta_site(irc.Plan(plan), Fd, knn=30, mode=mode)
    n = F.shape[0]
    rho, mi = irc.rho_post(k["vrKnn"].cpu().numpy(), k["miKnn"].cpu().numpy(), np.arange(1, n + 1), 30)
    delta, nn = irc.delta_post(k["delta"].cpu().numpy(), k["nneigh"].cpu().numpy(), np.arange(1, n + 1))
    rn, order = irc.sort_rho(rho)
    return rn.cpu().numpy(), delta, order.cpu().numpy(), nn, mi


@pytest.mark.parametrize("mode", ["bf16", "ref"])
def test_assign_on_site_outputs(gpu, mode):
    F, plan, _ = small_site(n=20000, d=33, n_chunks=10, seed=12)
    rho, delta, ordrho, nneigh, mk = _site_clustering_inputs(F, plan, mode)
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 30)
    assert ref["nClu"] >= 2
    _cmp(irc.post_cluster(dict(rho=rho, delta=delta, ordrho=ordrho, nneigh=nneigh, miKnn=mk),
                          dict(delta_cut=1.0, min_count=30)), ref)


def test_assign_full_size_drift400k(gpu):
    """The 400,000-spike drift workload end to end (BF16 form), bit-exact
    against the oracle on the same inputs."""
    site = synth.make_workload("drift400k")
    plan = synth.site_plan(site)
    rho, delta, ordrho, nneigh, mk = _site_clustering_inputs(site["F"], plan, "bf16")
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 30)
    got = irc.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 30)
    _cmp(got, ref)
    assert ref["nClu"] >= 2


def test_assign_errors(gpu):
    rho, delta, ordrho, nneigh, mk = random_case(12, n=100, knn=2, vocab=5000)
    bad = nneigh.copy()
    bad[np.nonzero(delta < 1.0)[0][0]] = 0
    with pytest.raises(_lib.IrcError):
        irc.assign_cluster_knn(rho, delta, ordrho, bad, mk, 1.0, 0)
    dup = ordrho.copy()
    dup[1] = dup[0]
    with pytest.raises(_lib.IrcError):
        irc.assign_cluster_knn(rho, delta, dup, nneigh, mk, 1.0, 0)
    # the library still works after an error
    ref = O.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 0)
    _cmp(irc.assign_cluster_knn(rho, delta, ordrho, nneigh, mk, 1.0, 0), ref)


def test_assign_too_many_peaks(gpu):
    n = _lib.CLUSTER_MAX_PEAKS + 10
    z = np.zeros(n, np.float32)
    with pytest.raises(_lib.IrcError) as e:
        irc.assign_cluster_knn(z, np.full(n, 2.0, np.float32), np.arange(1, n + 1), np.arange(1, n + 1),
                               np.arange(1, n + 1)[:, None], 1.0, 0)
    assert e.value.status == _lib.IRC_E_UNSUPPORTED
