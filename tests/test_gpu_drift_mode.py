"""The irc.m clustering modes built on the drop-in kernels, end to end.

* calc_dc2_drift_ (matlab/irc.m:24582-24608) on the device equals its C
  restatement bit for bit (dc2 and every site's value);
* cluster_drift_ (matlab/irc.m:24041-24180, GPU branch: dc2 from the first
  window, rho then delta window by window) equals the same loop over the
  reference's own jrc3_cuda_rho_drift / jrc3_cuda_delta_drift kernels;
* rho_drift_knn_ / delta_drift_knn_ (matlab/irc.m:24336-24361, :24477-24515)
  equal their per-chunk loops over the reference's cuda_knn_index /
  cuda_delta_knn with MATLAB's index mapping, padding and NaN rule.
"""
import numpy as np
import pytest
import torch

from ironclust_gb300 import irc
from oracle import oracle as O
from tests.dc2_cases import window

pytestmark = pytest.mark.gpu

SQRT_INF = np.float32(np.sqrt(3.402e38))


def bits(a):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return a.view(np.int32) if a.dtype == np.float32 else a


@pytest.mark.parametrize("n12,n1,nC,n_sites,sub,pct,seed,dup", [(3000, 600, 12, 4, 100, 2.0, 1, 0),
                                                                (5000, 900, 24, 7, 150, 5.0, 2, 0),
                                                                (1200, 1200, 33, 3, 1000, 2.0, 3, 30),
                                                                (9000, 2000, 33, 16, 1000, 2.0, 4, 0)])
def test_dc2_device_equals_oracle(gpu, n12, n1, nC, n_sites, sub, pct, seed, dup):
    F1, F2, s1, s2 = window(n12, n1, nC, n_sites, seed, dup)
    d, site = irc.calc_dc2_drift(n1, s1, s2, torch.from_numpy(F1).to(gpu), torch.from_numpy(F2).to(gpu), n_sites,
                                 sub, pct)
    do, so = O.calc_dc2_drift(n1, s1, s2, F1, F2, n_sites, sub, pct)
    assert bits(np.float32(d)) == bits(np.float32(do))
    assert np.array_equal(bits(site), bits(so))


def drift_recording(n_chunks=5, per=900, nC=16, n_sites=4, seed=11):
    rng = np.random.default_rng(seed)
    n = n_chunks * per
    centres = rng.normal(0, 5, (n_sites, nC))
    s1 = rng.integers(1, n_sites + 1, n).astype(np.int32)
    s2 = np.where(rng.random(n) < 0.7, rng.integers(1, n_sites + 1, n), 0).astype(np.int32)
    drift = np.repeat(rng.normal(0, 0.3, (n_chunks, nC)).cumsum(0), per, 0)
    F1 = (centres[s1 - 1] + drift + rng.normal(0, 1.2, (n, nC))).astype(np.float32)
    F2 = (F1 + rng.normal(0, 0.6, (n, nC))).astype(np.float32)
    cvi = [np.arange(i * per, (i + 1) * per) for i in range(n_chunks)]
    miSort = np.array([[0, 1, 2] if i == 0 else [i, i - 1, i - 2] if i == n_chunks - 1 else [i, i - 1, i + 1]
                       for i in range(n_chunks)]).T          # own chunk first, then two neighbours
    return F1, F2, s1, s2, cvi, miSort


def test_cluster_drift_equals_reference_kernel_loop(gpu, refk):
    F1, F2, s1, s2, cvi, miSort = drift_recording()
    n_sites = 4
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(gpu)
    out = irc.cluster_drift(s1, s2, t(F1), t(F2), cvi, miSort, n_sites, dc_subsample=200, dc_percent=2.0)
    # the same loop over the reference's kernels, dc2 from the oracle
    wins = irc.drift_windows(cvi, miSort)
    own0, w0 = wins[0]
    dc2, _ = O.calc_dc2_drift(len(own0), s1[w0], s2[w0], F1[w0], F2[w0], n_sites, 200, 2.0)
    assert bits(np.float32(out["dc2"])) == bits(dc2)
    n = F1.shape[0]
    rho = np.zeros(n, np.float32)
    for own, w in wins:
        site_cm = t(np.concatenate([s1[w], s2[w]]))
        rho[own] = refk.rho_drift(site_cm, t(F1[w]), t(F2[w]), len(own), float(dc2)).cpu().numpy()
    delta = np.zeros(n, np.float32)
    nneigh = np.zeros(n, np.int64)
    for own, w in wins:
        site_cm = t(np.concatenate([s1[w], s2[w]]))
        d, nn = refk.delta_drift(site_cm, t(F1[w]), t(F2[w]), t(rho[w]), len(own), float(dc2))
        delta[own] = d.cpu().numpy()
        nneigh[own] = w[nn.cpu().numpy().astype(np.int64) - 1]
    bad = np.isnan(delta)
    delta[bad] = delta[~bad].max()
    assert np.array_equal(bits(out["rho"]), bits(rho))
    assert np.array_equal(bits(out["delta"]), bits(delta))
    assert np.array_equal(out["nneigh"].cpu().numpy(), nneigh)


def knn_site(n12=4000, n1=3000, nC=24, n_chunks=6, seed=21):
    """One site's feature matrix: its own n1 spikes first, then neighbouring
    sites' copies; 1-based chunk ids; banded chunk linkage (mlDrift[i, j]:
    chunk i's spikes are candidates of chunk j)."""
    rng = np.random.default_rng(seed)
    F = rng.normal(0, 2, (n12, nC)).astype(np.float32)
    F[7] = F[6]                                               # an exact duplicate
    vd = np.concatenate([np.repeat(np.arange(1, n_chunks + 1), n1 // n_chunks + 1)[:n1],
                         rng.integers(1, n_chunks + 1, n12 - n1)]).astype(np.int64)
    ml = np.zeros((n_chunks, n_chunks), bool)
    for j in range(n_chunks):
        ml[max(0, j - 1):j + 2, j] = True
    ml[:, n_chunks - 1] = False
    ml[n_chunks - 1, n_chunks - 1] = True                    # a chunk linked to itself only
    return F, vd, ml


def test_rho_drift_knn_equals_reference_loop(gpu, refk):
    F, vd, ml = knn_site()
    n1, knn = 3000, 30
    Fd = torch.from_numpy(F).to(gpu)
    rho, mi = irc.rho_drift_knn(Fd, vd, ml, n1, knn)
    want_rho = np.zeros(n1, np.float32)
    want_mi = np.zeros((n1, knn), np.int64)
    for d in range(1, ml.shape[0] + 1):
        vi1 = np.flatnonzero(vd[:n1] == d)
        if not vi1.size:
            continue
        vi2 = np.flatnonzero(ml[vd - 1, d - 1])
        k = min(knn, vi2.size)
        K, I = refk.cuda_knn_index(Fd[vi2].contiguous(), Fd[vi1].contiguous(), k)
        want_rho[vi1] = (np.float32(1) / K.cpu().numpy()).astype(np.float32)
        m = vi2[I.cpu().numpy().astype(np.int64) - 1]
        if k < knn:
            m = np.concatenate([m, np.repeat(m[:, -1:], knn - k, 1)], 1)
        want_mi[vi1] = m
    assert np.array_equal(bits(rho), bits(want_rho))
    assert np.array_equal(mi.cpu().numpy(), want_mi)


def test_delta_drift_knn_equals_reference_loop(gpu, refk):
    F, vd, ml = knn_site(seed=22)
    n1 = 3000
    rng = np.random.default_rng(5)
    R = rng.uniform(0.1, 1, F.shape[0]).astype(np.float32)
    # local peaks: no higher-rho candidate, so the kernel's distance is
    # sqrt(SINGLE_INF) and delta .* rho overflows -- the NaN/Inf rule
    R[np.flatnonzero(vd[:n1] == 2)[:3]] = 1e20
    Fd, Rd = torch.from_numpy(F).to(gpu), torch.from_numpy(R).to(gpu)
    delta, nneigh = irc.delta_drift_knn(Fd, vd, ml, Rd, n1)
    want_d = np.zeros(n1, np.float32)
    want_n = np.zeros(n1, np.int64)
    for d in range(1, ml.shape[0] + 1):
        vi1 = np.flatnonzero(vd[:n1] == d)
        if not vi1.size:
            continue
        vi2 = np.flatnonzero(ml[vd - 1, d - 1])
        D, N = refk.cuda_delta_knn(Fd[vi2].contiguous(), Fd[vi1].contiguous(), Rd[vi2].contiguous(),
                                   Rd[vi1].contiguous())
        want_d[vi1] = D.cpu().numpy()
        want_n[vi1] = vi2[N.cpu().numpy().view(np.uint32).astype(np.int64) - 1]
    with np.errstate(over="ignore"):                          # the peaks' products overflow on purpose
        want_d = (want_d * R[:n1]).astype(np.float32)
    bad = ~np.isfinite(want_d)
    want_n[bad] = np.flatnonzero(bad)
    want_d[bad] = SQRT_INF
    assert bad.any()                                          # the local peaks take the NaN/Inf rule
    assert np.array_equal(bits(delta), bits(want_d))
    assert np.array_equal(nneigh.cpu().numpy(), want_n)
