"""Parity at the full benchmark configurations.

static20k  20,000 spikes, D = 24, one chunk: REF equals the reference's own
           search_min_drift / search_delta_drift (PTX compiled from its
           sources, MATLAB launch configuration) + MATLAB sort / min, bit for
           bit; EXACT equals the FP32 oracle bit for bit; BF16 against FP64.
drift400k  400,000 spikes, D = 33, 200 drift chunks x 15 links: REF equals
           the reference kernels chunk by chunk over all 200 chunks; EXACT
           equals the FP32 oracle (kNN and delta); BF16 and EXACT against the
           FP64 oracle on every spike.
probe10m   384 sites, 10 M spikes, one batch plan: BF16 against FP64 on whole
           sites drawn (seeded) until they hold at least 1 M spikes.

FP64 bars (the precision targets of the tensor-core form), every spike:
  * kNN recall >= 0.999 (set overlap of the k lists);
  * rho = 1/d_knn within 1e-4 relative;
  * delta within 1e-4 relative, with the nearest higher-rho neighbour taken
    from the FP64 rho; a different neighbour is an error unless the two
    candidates are ordered differently by FP32 and FP64 rho (a rho-order
    flip, below FP32 resolution: the exact FP32 form meets the same ones);
    such flips stay below 1e-4 of the spikes.
"""
import numpy as np
import pytest
import torch

from ironclust_gb300 import _lib, irc, synth
from oracle import accuracy as A
from oracle import oracle as O

pytestmark = pytest.mark.gpu

KNN = 30


def bits(a):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return a.view(np.int32) if a.dtype == np.float32 else a


def host(out):
    return {k: (v.cpu().numpy() if isinstance(v, torch.Tensor) else v) for k, v in out.items()}


def ref_loop(refk, Fd, plan, rho=None):
    """The reference kernels once per query chunk + MATLAB sort (kNN) or
    MATLAB min (delta), exactly as search_knn_drift_ / search_delta_drift_
    run them (matlab/irc2.m:3764-3788, :3829-3864)."""
    n = int(plan["n_out"])
    nC, nF = Fd.shape[1], Fd.shape[0]
    a = np.zeros(n, np.float32)
    b = np.zeros((n, KNN), np.int32) if rho is None else np.zeros(n, np.int32)
    for i in range(len(plan["q0"])):
        r0, r1 = int(plan["roff"][i]), int(plan["roff"][i + 1])
        IBB = torch.from_numpy(np.ascontiguousarray(plan["rs"][r0:r1])).to(Fd.device)
        NBB = torch.from_numpy(np.ascontiguousarray(plan["rn"][r0:r1])).to(Fd.device)
        q0, nq = int(plan["q0"][i]), int(plan["nq"][i])
        vn = [nC, nF, r1 - r0, q0, nq]
        o = q0 - int(plan["q_base"])
        if rho is None:
            D, I = refk.search_min_drift(Fd, IBB, NBB, vn)
            a[o:o + nq], b[o:o + nq] = O.post_sort_knn(D.cpu().numpy(), I.cpu().numpy(), KNN)
        else:
            D, I = refk.search_delta_drift(Fd, rho, IBB, NBB, vn)
            a[o:o + nq], b[o:o + nq] = O.post_min(D.cpu().numpy(), I.cpu().numpy())
    return a, b


def check_fp64(acc, n, what):
    assert acc["recall_vs_fp64"] >= 0.999, (what, acc)
    assert acc["rho_max_rel_err"] <= 1e-4, (what, acc)
    assert acc["nneigh_errors"] == 0, (what, acc)
    assert acc["delta_max_rel_err"] <= 1e-4, (what, acc)
    assert acc["nneigh_rho_order_flips"] <= max(1, n // 10000), (what, acc)


def run_workload(name, gpu):
    site = synth.make_workload(name)
    plan = synth.site_plan(site)
    Fd = torch.from_numpy(site["F"]).to(gpu)
    return site, plan, Fd


@pytest.fixture(scope="module")
def static20k(gpu):
    return run_workload("static20k", gpu)


@pytest.fixture(scope="module")
def drift400k(gpu):
    site, plan, Fd = run_workload("drift400k", gpu)
    P = irc.Plan(plan)
    ex = host(irc.knn_rho_delta_site(P, Fd, knn=KNN, mode="exact"))
    _lib.check(_lib.lib().irc_plan_check(P.h, irc._stream()), "irc_plan_check")
    yield site, plan, Fd, P, ex
    P.close()


@pytest.fixture(scope="module")
def drift400k_fp64(drift400k):
    site, plan = drift400k[0], drift400k[1]
    return A.fp64_reference(site["F"], plan, KNN)


def test_static20k_ref_equals_reference_kernels(static20k, refk):
    site, plan, Fd = static20k
    P = irc.Plan(plan)
    out = irc.site_knn(P, Fd, knn=KNN, mode="ref")
    vr, mi = ref_loop(refk, Fd, plan)
    assert np.array_equal(bits(out["vrKnn"]), bits(vr))
    assert np.array_equal(out["miKnn"].cpu().numpy(), mi)
    de, nn = irc.site_delta(P, Fd, out["rho"], mode="ref")
    d_ref, n_ref = ref_loop(refk, Fd, plan, rho=out["rho"])
    assert np.array_equal(bits(de), bits(d_ref * out["rho"].cpu().numpy()))
    assert np.array_equal(nn.cpu().numpy(), n_ref)
    P.close()


def test_static20k_exact_and_bf16(static20k):
    site, plan, Fd = static20k
    P = irc.Plan(plan)
    ex = host(irc.knn_rho_delta_site(P, Fd, knn=KNN, mode="exact"))
    idx, d2 = O.exact_knn_f32(site["F"], plan, KNN)
    assert np.array_equal(ex["miKnn"], idx) and np.array_equal(bits(ex["d2Knn"]), bits(d2))
    nn, _ = O.exact_delta_f32(site["F"], ex["rho"], plan)
    assert np.array_equal(ex["nneigh"], nn)
    ref = A.fp64_reference(site["F"], plan, KNN)
    bf = host(irc.knn_rho_delta_site(P, Fd, knn=KNN, mode="bf16"))
    _lib.check(_lib.lib().irc_plan_check(P.h, irc._stream()), "irc_plan_check")
    check_fp64(A.compare(bf, ref), site["F"].shape[0], "static20k bf16")
    P.close()


def test_drift400k_ref_equals_reference_kernels_every_chunk(drift400k, refk):
    site, plan, Fd, P, _ = drift400k
    out = irc.site_knn(P, Fd, knn=KNN, mode="ref")
    vr, mi = ref_loop(refk, Fd, plan)
    assert np.array_equal(bits(out["vrKnn"]), bits(vr))
    assert np.array_equal(out["miKnn"].cpu().numpy(), mi)
    de, nn = irc.site_delta(P, Fd, out["rho"], mode="ref")
    d_ref, n_ref = ref_loop(refk, Fd, plan, rho=out["rho"])
    assert np.array_equal(bits(de), bits(d_ref * out["rho"].cpu().numpy()))
    assert np.array_equal(nn.cpu().numpy(), n_ref)


def test_drift400k_exact_equals_fp32_oracle(drift400k):
    site, plan, _, _, ex = drift400k
    idx, d2 = O.exact_knn_f32(site["F"], plan, KNN)
    assert np.array_equal(ex["miKnn"], idx)
    assert np.array_equal(bits(ex["d2Knn"]), bits(d2))
    nn, dd = O.exact_delta_f32(site["F"], ex["rho"], plan)
    assert np.array_equal(ex["nneigh"], nn)
    want = (np.sqrt(dd.astype(np.float32)) * ex["rho"]).astype(np.float32)
    assert np.array_equal(bits(ex["delta"]), bits(want))


def test_drift400k_exact_vs_fp64(drift400k, drift400k_fp64):
    site, _, _, _, ex = drift400k
    acc = A.compare(ex, drift400k_fp64)
    print("drift400k exact vs fp64:", acc)
    check_fp64(acc, site["F"].shape[0], "drift400k exact")


@pytest.mark.parametrize("mode", ["bf16"])
def test_drift400k_tensor_core_vs_fp64(drift400k, drift400k_fp64, mode):
    site, _, Fd, P, ex = drift400k
    out = host(irc.knn_rho_delta_site(P, Fd, knn=KNN, mode=mode))
    _lib.check(_lib.lib().irc_plan_check(P.h, irc._stream()), "irc_plan_check")
    acc = A.compare(out, drift400k_fp64)
    print("drift400k %s vs fp64:" % mode, acc)
    check_fp64(acc, site["F"].shape[0], "drift400k " + mode)


def test_probe10m_bf16_vs_fp64_on_a_1m_subsample(gpu):
    b, _ = synth.make_probe()
    Fd = torch.from_numpy(b.F).to(gpu)
    P = irc.Plan(b.plan)
    out = host(irc.knn_rho_delta_site(P, Fd, knn=KNN, mode="bf16"))
    _lib.check(_lib.lib().irc_plan_check(P.h, irc._stream()), "irc_plan_check")
    P.close()
    del Fd
    rng = np.random.default_rng(2024)
    order = rng.permutation(b.n_sites)
    picked, total = [], 0
    for s in order:
        picked.append(int(s))
        total += int(b.sizes[s])
        if total >= 1_000_000:
            break
    stats = []
    for s in picked:
        sl = b.site_slice(s)
        base = int(b.bases[s])
        Fs = np.ascontiguousarray(b.F[sl, :int(b.dims[s])])
        ref = A.fp64_reference(Fs, b.site_plans[s], KNN)
        o = dict(miKnn=out["miKnn"][sl] - base, rho=out["rho"][sl], delta=out["delta"][sl],
                 nneigh=out["nneigh"][sl] - base)
        stats.append(A.compare(o, ref))
    n = sum(x["checked"] for x in stats)
    agg = dict(checked=n,
               recall_vs_fp64=sum(x["recall_vs_fp64"] * x["checked"] for x in stats) / n,
               rho_max_rel_err=max(x["rho_max_rel_err"] for x in stats),
               delta_max_rel_err=max(x["delta_max_rel_err"] for x in stats),
               nneigh_errors=sum(x["nneigh_errors"] for x in stats),
               nneigh_rho_order_flips=sum(x["nneigh_rho_order_flips"] for x in stats))
    print("probe10m bf16 vs fp64 (%d sites):" % len(picked), agg)
    assert n >= 1_000_000
    check_fp64(agg, n, "probe10m bf16")
