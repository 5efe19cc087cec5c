"""Drop-in kernels vs the reference's own kernels (and the CPU oracle).

Every comparison is bit-exact: float outputs are compared as raw bits.
The reference kernels are the shipped .cu sources compiled to PTX and
launched with the MATLAB launch configuration (oracle/ref_harness.cu).
"""
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


def same(a, b):
    return np.array_equal(bits(a), bits(b))


CASES = [
    dict(n=3000, d=24, n_chunks=5, seed=7),
    dict(n=2500, d=33, n_chunks=4, seed=8, secondary=True),
    dict(n=1203, d=45, n_chunks=3, seed=9, sizes=[1, 601, 601]),
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("nT", [1024, 512])
def test_search_min_drift_bitexact(gpu, refk, case, nT):
    F, plan, _ = small_site(**case)
    Fd = torch.from_numpy(F).to(gpu)
    for i in range(len(plan["q0"])):
        r0, r1 = plan["roff"][i], plan["roff"][i + 1]
        IBB = torch.from_numpy(plan["rs"][r0:r1]).to(gpu)
        NBB = torch.from_numpy(plan["rn"][r0:r1]).to(gpu)
        vn = [F.shape[1], F.shape[0], int(r1 - r0), int(plan["q0"][i]), int(plan["nq"][i])]
        D, I = irc.search_min_drift(Fd, IBB, NBB, vn, nThreads=nT)
        Dr, Ir = refk.search_min_drift(Fd, IBB, NBB, vn, nT=nT)
        assert same(D, Dr) and same(I, Ir), "chunk %d differs from the reference kernel" % i
        if i == 0:
            Do, Io = O.search_min_drift(F, plan["rs"][r0:r1], plan["rn"][r0:r1], vn, nT)
            assert same(D, Do) and same(I, Io), "oracle differs"


@pytest.mark.parametrize("case", CASES)
def test_search_min_drift_exact_mode(gpu, case):
    """IRC_MODE_EXACT fills rows 0..knn-1 so that the unchanged MATLAB sort
    returns the exact kNN of the chunk."""
    F, plan, _ = small_site(**case)
    Fd = torch.from_numpy(F).to(gpu)
    idx, d2 = O.exact_knn_f32(F, plan, 30)
    for i in range(len(plan["q0"])):
        r0, r1 = plan["roff"][i], plan["roff"][i + 1]
        IBB = torch.from_numpy(plan["rs"][r0:r1]).to(gpu)
        NBB = torch.from_numpy(plan["rn"][r0:r1]).to(gpu)
        q0, nq = int(plan["q0"][i]), int(plan["nq"][i])
        D, I = irc.search_min_drift(Fd, IBB, NBB, [F.shape[1], F.shape[0], int(r1 - r0), q0, nq],
                                    nThreads=1024, mode="exact", knn=30)
        v, m = O.post_sort_knn(D.cpu().numpy(), I.cpu().numpy(), 30)
        o = q0 - plan["q_base"]
        assert np.array_equal(m, idx[o:o + nq]), i
        assert np.array_equal(bits(v), bits(np.sqrt(d2[o:o + nq, 29]).astype(np.float32))), i


@pytest.mark.parametrize("case", CASES)
def test_search_delta_drift_bitexact(gpu, refk, case):
    F, plan, _ = small_site(**case)
    R = rho_with_ties(F.shape[0])
    Fd, Rd = torch.from_numpy(F).to(gpu), torch.from_numpy(R).to(gpu)
    for i in range(len(plan["q0"])):
        r0, r1 = plan["roff"][i], plan["roff"][i + 1]
        IBB = torch.from_numpy(plan["rs"][r0:r1]).to(gpu)
        NBB = torch.from_numpy(plan["rn"][r0:r1]).to(gpu)
        vn = [F.shape[1], F.shape[0], int(r1 - r0), int(plan["q0"][i]), int(plan["nq"][i])]
        D, I = irc.search_delta_drift(Fd, Rd, IBB, NBB, vn)
        Dr, Ir = refk.search_delta_drift(Fd, Rd, IBB, NBB, vn)
        assert same(D, Dr) and same(I, Ir), "chunk %d differs" % i
        if i == 0:
            Do, Io = O.search_delta_drift(F, R, plan["rs"][r0:r1], plan["rn"][r0:r1], vn)
            assert same(D, Do) and same(I, Io)


@pytest.mark.parametrize("nB,nA,nC,knn", [(1500, 200, 33, 30), (300, 77, 24, 30), (40, 17, 18, 40),
                                          (5000, 33, 60, 30)])
def test_cuda_knn_index_bitexact(gpu, refk, nB, nA, nC, knn):
    rng = np.random.default_rng(nB + nA)
    B = rng.normal(0, 3, (nB, nC)).astype(np.float32)
    B[5] = B[4]                                                   # duplicate candidates
    A = np.concatenate([B[:nA // 2], rng.normal(0, 3, (nA - nA // 2, nC))]).astype(np.float32)
    knn = min(knn, nB)
    Bd, Ad = torch.from_numpy(B).to(gpu), torch.from_numpy(A).to(gpu)
    K, I = irc.cuda_knn_index(Bd, Ad, knn)
    Kr, Ir = refk.cuda_knn_index(Bd, Ad, knn)
    assert same(K, Kr) and same(I, Ir)
    Ko, Io = O.cuda_knn_index(B, A, knn)
    assert same(K, Ko) and same(I, Io)


@pytest.mark.parametrize("nB,nA,nC", [(1500, 200, 33), (100, 300, 24), (3000, 16, 45)])
def test_cuda_delta_knn_bitexact(gpu, refk, nB, nA, nC):
    rng = np.random.default_rng(nB * 3 + nA)
    B = rng.normal(0, 3, (nB, nC)).astype(np.float32)
    A = B[rng.choice(nB, nA)] if nA <= nB else rng.normal(0, 3, (nA, nC)).astype(np.float32)
    RB = rho_with_ties(nB, 5)
    RA = rho_with_ties(nA, 6)
    RA[0] = RB.max() + 1                     # a query with no higher-rho candidate
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(gpu)
    D, N = irc.cuda_delta_knn(t(B), t(A), t(RB), t(RA))
    Dr, Nr = refk.cuda_delta_knn(t(B), t(A), t(RB), t(RA))
    assert same(D, Dr) and same(N, Nr)
    Do, No = O.cuda_delta_knn(B, A, RB, RA)
    assert same(D, Do) and np.array_equal(N.cpu().numpy().view(np.uint32), No)


@pytest.mark.parametrize("n12,n1,nC", [(1500, 300, 33), (700, 700, 24), (2000, 17, 45)])
def test_delta_drift_bitexact(gpu, refk, n12, n1, nC):
    rng = np.random.default_rng(n12 * 7 + n1)
    f1 = rng.normal(0, 2, (n12, nC)).astype(np.float32)
    f2 = (f1 + rng.normal(0, 0.5, (n12, nC))).astype(np.float32)
    f1[3] = f1[2]                                             # a zero distance (kept by this kernel)
    s1 = rng.integers(1, 4, n12).astype(np.int32)
    s2 = rng.integers(1, 4, n12).astype(np.int32)
    rho = rho_with_ties(n12, 9)
    rho[0] = rho.max() + 1                                    # a query with no higher-rho candidate
    dc2 = float(np.float32(17.5))
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(gpu)
    site_cm = t(np.concatenate([s1, s2]))
    de, nn = irc.delta_drift(site_cm, t(f1), t(f2), t(rho), n1, dc2)
    dr, nr = refk.delta_drift(site_cm, t(f1), t(f2), t(rho), n1, dc2)
    assert same(de, dr) and same(nn, nr)
    do, no = O.delta_drift(np.stack([s1, s2], 1), f1, f2, rho, n1, dc2)
    assert same(de, do) and np.array_equal(nn.cpu().numpy().view(np.uint32), no)


@pytest.mark.parametrize("n12,n1,nC", [(1500, 300, 33), (700, 700, 24), (2000, 17, 45)])
def test_rho_drift_bitexact(gpu, refk, n12, n1, nC):
    rng = np.random.default_rng(n12 + n1)
    f1 = rng.normal(0, 2, (n12, nC)).astype(np.float32)
    f2 = (f1 + rng.normal(0, 0.5, (n12, nC))).astype(np.float32)
    s1 = rng.integers(1, 4, n12).astype(np.int32)
    s2 = rng.integers(1, 4, n12).astype(np.int32)
    site = np.stack([s1, s2], 1)
    d = ((f1[:50, None, :] - f1[None, :50, :]) ** 2).sum(-1)
    dc2 = float(np.float32(np.quantile(d[d > 0], 0.2)))
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(gpu)
    site_cm = t(np.concatenate([s1, s2]))
    rho = irc.rho_drift(site_cm, t(f1), t(f2), n1, dc2)
    rr = refk.rho_drift(site_cm, t(f1), t(f2), n1, dc2)
    assert same(rho, rr)
    ro = O.rho_drift(site, f1, f2, n1, dc2)
    assert same(rho, ro)


def _knn_inputs(nB, nA, nC, seed):
    rng = np.random.default_rng(seed)
    B = rng.normal(0, 3, (nB, nC)).astype(np.float32)
    B[5] = B[4]                                                   # duplicate candidates
    A = np.concatenate([B[:nA // 2], rng.normal(0, 3, (nA - nA // 2, nC))]).astype(np.float32)
    return B, A


@pytest.mark.parametrize("nB,nA,nC,knn", [(2000, 300, 33, 30), (200, 100, 24, 30), (5000, 33, 36, 16),
                                          (100, 50, 9, 120)])
def test_cuda_knn_bitexact(gpu, refk, nB, nA, nC, knn):
    """cuda_knn.cu: 256 bins, K only (nB < 256 leaves empty bins)."""
    B, A = _knn_inputs(nB, nA, nC, nB + 7)
    knn = min(knn, nB)
    Bd, Ad = torch.from_numpy(B).to(gpu), torch.from_numpy(A).to(gpu)
    K = irc.cuda_knn_kth(Bd, Ad, knn)
    assert same(K, refk.cuda_knn(Bd, Ad, knn))
    assert same(K, O.cuda_knn(B, A, knn))


@pytest.mark.parametrize("nB,nA,nC,knn", [(3000, 200, 33, 30), (300, 64, 60, 30), (1000, 9, 45, 200)])
def test_cuda_knn_full_bitexact(gpu, refk, nB, nA, nC, knn):
    B, A = _knn_inputs(nB, nA, nC, nB + 8)
    knn = min(knn, nB)
    Bd, Ad = torch.from_numpy(B).to(gpu), torch.from_numpy(A).to(gpu)
    K, I = irc.cuda_knn_full(Bd, Ad, knn)
    Kr, Ir = refk.cuda_knn_full(Bd, Ad, knn)
    assert same(K, Kr) and same(I, Ir)
    Ko, Io = O.cuda_knn_full(B, A, knn)
    assert same(K, Ko) and same(I, Io)


@pytest.mark.parametrize("nF,nB,nA,nC,knn", [(4000, 2500, 150, 33, 30), (600, 600, 40, 24, 30),
                                             (5000, 300, 20, 60, 50)])
def test_cuda_knn_ib_bitexact(gpu, refk, nF, nB, nA, nC, knn):
    """Candidates through an index list with repeats and an arbitrary order."""
    rng = np.random.default_rng(nF + nB)
    F, A = _knn_inputs(nF, nA, nC, nF + 9)
    IB = rng.integers(1, nF + 1, nB).astype(np.int32)
    IB[:10] = IB[10]                                              # repeated candidates
    Fd, Ad, IBd = (torch.from_numpy(x).to(gpu) for x in (F, A, IB))
    K, I = irc.cuda_knn_ib(Fd, Ad, IBd, knn)
    Kr, Ir = refk.cuda_knn_ib(Fd, Ad, IBd, knn)
    assert same(K, Kr) and same(I, Ir)
    Ko, Io = O.cuda_knn_ib(F, A, IB, knn)
    assert same(K, Ko) and same(I, Io)


def test_cuda_knn_ib_rejects_bad_index(gpu):
    from ironclust_gb300 import _lib
    F, A = _knn_inputs(100, 10, 8, 3)
    IB = np.arange(1, 51, dtype=np.int32)
    IB[7] = 101
    with pytest.raises(_lib.IrcError):
        irc.cuda_knn_ib(torch.from_numpy(F).to(gpu), torch.from_numpy(A).to(gpu), IB, 10)


def _spacetime_inputs(n12, n1, nC, seed):
    """Features with duplicates, a time order with ties, rho ranks."""
    rng = np.random.default_rng(seed)
    F = rng.normal(0, 2, (n12, nC)).astype(np.float32)
    F[3] = F[2]
    ordr = np.sort(rng.integers(0, n12 // 2, n12)).astype(np.int32)     # time order, with ties
    perm = rng.permutation(n12)
    F, ordr = F[perm], ordr[perm]
    rr = np.argsort(np.argsort(-rho_with_ties(n12, seed), kind="stable"), kind="stable").astype(np.int32) + 1
    return F, ordr, rr


@pytest.mark.parametrize("n12,n1,nC,dn,fdc", [(1500, 400, 33, 100, 0), (800, 800, 24, 40, 1), (2000, 17, 45, 5, 0),
                                              (300, 100, 12, 1000, 1)])
def test_cuda_rho_spacetime_bitexact(gpu, refk, n12, n1, nC, dn, fdc):
    F, ordr, _ = _spacetime_inputs(n12, n1, nC, n12 + dn)
    dc2 = np.float32(4.0) if fdc == 0 else np.float32(0.05)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(gpu)
    rho = irc.cuda_rho_st(t(F), t(ordr), n1, dn, float(dc2), fdc)
    assert same(rho, refk.cuda_rho(t(F), t(ordr), n1, dn, float(dc2), fdc))
    assert same(rho, O.cuda_rho(F, ordr, n1, dn, dc2, fdc))


@pytest.mark.parametrize("n12,n1,nC,dn,fdc,nT", [(1500, 400, 33, 100, 0, 128), (800, 800, 24, 40, 1, 128),
                                                 (2000, 17, 45, 5, 0, 64), (300, 100, 12, 1000, 1, 32)])
def test_cuda_delta_spacetime_bitexact(gpu, refk, n12, n1, nC, dn, fdc, nT):
    F, ordr, rr = _spacetime_inputs(n12, n1, nC, n12 + dn + 1)
    rr[0] = 0                                                     # a query ranked first: no candidate
    dc2 = np.float32(4.0) if fdc == 0 else np.float32(0.05)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(gpu)
    de, nn = irc.cuda_delta_st(t(F), t(ordr), t(rr), n1, dn, float(dc2), fdc, nT)
    der, nnr = refk.cuda_delta(t(F), t(ordr), t(rr), n1, dn, float(dc2), fdc, nT)
    assert same(de, der) and same(nn, nnr)
    deo, nno = O.cuda_delta(F, ordr, rr, n1, dn, dc2, fdc, nT)
    assert same(de, deo) and np.array_equal(nn.cpu().numpy().view(np.uint32), nno)
