"""Fused per-site path vs the per-chunk MATLAB loop and the oracles."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import irc
from oracle import oracle as O
from tests.cases import rho_with_ties, small_site

pytestmark = pytest.mark.gpu


def bits(t):
    a = t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)
    return a.view(np.int32) if a.dtype == np.float32 else a


CASES = [
    dict(n=3000, d=24, n_chunks=5, seed=7),
    dict(n=2500, d=33, n_chunks=4, seed=8, secondary=True),
    dict(n=1203, d=45, n_chunks=3, seed=9, sizes=[1, 601, 601]),
    dict(n=4000, d=18, n_chunks=1, seed=10),
]


@pytest.mark.parametrize("case", CASES)
def test_site_knn_ref_equals_reference_loop(gpu, refk, case):
    """irc_site_knn(REF) == reference search_min_drift per chunk + MATLAB sort."""
    F, plan, _ = small_site(**case)
    Fd = torch.from_numpy(F).to(gpu)
    P = irc.Plan(plan)
    out = irc.site_knn(P, Fd, knn=30, mode="ref")
    n = plan["n_out"]
    vr = np.zeros(n, np.float32)
    mi = np.zeros((n, 30), np.int32)
    for i in range(len(plan["q0"])):
        r0, r1 = plan["roff"][i], plan["roff"][i + 1]
        IBB = torch.from_numpy(plan["rs"][r0:r1]).to(gpu)
        NBB = torch.from_numpy(plan["rn"][r0:r1]).to(gpu)
        q0, nq = int(plan["q0"][i]), int(plan["nq"][i])
        D, I = refk.search_min_drift(Fd, IBB, NBB, [F.shape[1], F.shape[0], int(r1 - r0), q0, nq])
        v, m = O.post_sort_knn(D.cpu().numpy(), I.cpu().numpy(), 30)
        vr[q0 - plan["q_base"]:q0 - plan["q_base"] + nq] = v
        mi[q0 - plan["q_base"]:q0 - plan["q_base"] + nq] = m
    assert np.array_equal(bits(out["vrKnn"]), bits(vr))
    assert np.array_equal(out["miKnn"].cpu().numpy(), mi)
    rho = (np.float32(1) / vr).astype(np.float32)
    assert np.array_equal(bits(out["rho"]), bits(rho))
    # the host loop over the drop-in (torch MATLAB-sort) agrees too
    v2, m2 = irc.search_knn_drift(plan, Fd, 30)
    assert np.array_equal(bits(v2), bits(vr)) and np.array_equal(m2.cpu().numpy(), mi)


@pytest.mark.parametrize("case", CASES)
def test_site_delta_ref_equals_reference_loop(gpu, refk, case):
    F, plan, _ = small_site(**case)
    R = rho_with_ties(F.shape[0], 11)
    Fd, Rd = torch.from_numpy(F).to(gpu), torch.from_numpy(R).to(gpu)
    P = irc.Plan(plan)
    delta, nneigh = irc.site_delta(P, Fd, Rd, mode="ref")
    n = plan["n_out"]
    de = np.zeros(n, np.float32)
    nn = np.zeros(n, np.int32)
    for i in range(len(plan["q0"])):
        r0, r1 = plan["roff"][i], plan["roff"][i + 1]
        IBB = torch.from_numpy(plan["rs"][r0:r1]).to(gpu)
        NBB = torch.from_numpy(plan["rn"][r0:r1]).to(gpu)
        q0, nq = int(plan["q0"][i]), int(plan["nq"][i])
        D, I = refk.search_delta_drift(Fd, Rd, IBB, NBB, [F.shape[1], F.shape[0], int(r1 - r0), q0, nq])
        v, m = O.post_min(D.cpu().numpy(), I.cpu().numpy())
        o = q0 - plan["q_base"]
        de[o:o + nq] = v * R[q0:q0 + nq]
        nn[o:o + nq] = m
    assert np.array_equal(bits(delta), bits(de))
    assert np.array_equal(nneigh.cpu().numpy(), nn)


@pytest.mark.parametrize("case", CASES)
def test_site_knn_exact_equals_fp32_oracle(gpu, case):
    F, plan, _ = small_site(**case)
    Fd = torch.from_numpy(F).to(gpu)
    P = irc.Plan(plan)
    out = irc.site_knn(P, Fd, knn=30, mode="exact")
    idx, d2 = O.exact_knn_f32(F, plan, 30)
    assert np.array_equal(out["miKnn"].cpu().numpy(), idx)
    assert np.array_equal(bits(out["d2Knn"]), bits(d2))
    vr = np.sqrt(d2[:, 29]).astype(np.float32)
    assert np.array_equal(bits(out["vrKnn"]), bits(vr))
    # and the FP64 ground truth agrees on the neighbour sets except at near-ties
    i64, _ = O.exact_knn_f64(F, plan, 30)
    agree = np.mean([len(set(a) & set(b)) / 30 for a, b in zip(idx, i64)])
    assert agree > 0.999


@pytest.mark.parametrize("case", CASES)
def test_site_delta_from_knn_list_is_exact(gpu, case):
    F, plan, _ = small_site(**case)
    Fd = torch.from_numpy(F).to(gpu)
    P = irc.Plan(plan)
    if plan["n_out"] != F.shape[0]:
        pytest.skip("kNN-list delta needs every column as a query")
    out = irc.knn_rho_delta_site(P, Fd, knn=30, mode="exact")
    R = out["rho"].cpu().numpy()
    nn, d2 = O.exact_delta_f32(F, R, plan)
    de = (np.sqrt(d2).astype(np.float32) * R).astype(np.float32)
    assert np.array_equal(out["nneigh"].cpu().numpy(), nn)
    assert np.array_equal(bits(out["delta"]), bits(de))
