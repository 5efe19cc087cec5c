"""A batch of sites (different feature dimensions, chunk sizes down to a
single query) through one plan equals each site run on its own: bit for bit
in the REF and EXACT forms (zero-padded features add exactly 0), and for the
BF16 form wherever its filter kept the true neighbours (>= 99.9% of rows;
the position of the norm terms in K moves with the padding, so the
approximate distances may round differently)."""
import numpy as np
import pytest
import torch

from ironclust_gb300 import batch, irc, synth

pytestmark = pytest.mark.gpu

SPECS = [dict(n_spk=3000, n_dim=18, n_clusters=5, n_chunks=40, seed=1),
         dict(n_spk=700, n_dim=33, n_clusters=4, n_chunks=40, seed=2),
         dict(n_spk=9000, n_dim=24, n_clusters=8, n_chunks=40, seed=3),
         dict(n_spk=90, n_dim=24, n_clusters=3, n_chunks=40, seed=4),      # ~2 queries per chunk
         dict(n_spk=5200, n_dim=33, n_clusters=6, n_chunks=12, seed=5)]    # 433 per chunk: 128-row items


@pytest.fixture(scope="module")
def sites():
    return [synth.make_site(**s) for s in SPECS]


def _site_result(site, mode, gpu):
    plan = synth.site_plan(site)
    P = irc.Plan(plan)
    F = torch.from_numpy(site["F"]).to(gpu)
    out = irc.knn_rho_delta_site(P, F, knn=30, mode=mode)
    return {k: (v.cpu().numpy() if v is not None else None) for k, v in out.items()}


@pytest.mark.parametrize("mode", ["ref", "exact", "bf16"])
def test_batch_equals_sites(gpu, sites, mode):
    b = batch.SiteBatch(sites)
    P = irc.Plan(b.plan)
    F = torch.from_numpy(b.F).to(gpu)
    out = irc.knn_rho_delta_site(P, F, knn=30, mode=mode)
    got = {k: (v.cpu().numpy() if v is not None else None) for k, v in out.items()}
    for i, site in enumerate(sites):
        want = _site_result(site, mode, gpu)
        sl = b.site_slice(i)
        mi = b.split_knn(got["miKnn"], i)
        if mode == "bf16":
            same = np.all(mi == want["miKnn"], axis=1).mean()
            assert same >= 0.999, (i, same)
        else:
            assert np.array_equal(mi, want["miKnn"]), i
            assert np.array_equal(got["vrKnn"][sl].view(np.int32), want["vrKnn"].view(np.int32)), i
            assert np.array_equal(got["delta"][sl].view(np.int32), want["delta"].view(np.int32)), i
            assert np.array_equal(got["nneigh"][sl] - int(b.bases[i]), want["nneigh"]), i


def test_batch_plan_packs_small_chunks(sites):
    b = batch.SiteBatch(sites)
    nq = b.plan["nq"]
    assert (nq <= 32).sum() > 40 and (nq > 128).sum() >= 12
    assert b.F.shape == (sum(s["F"].shape[0] for s in sites), 33)
    # padding columns are zero
    assert not b.F[b.site_slice(0), 18:].any()


@pytest.mark.parametrize("mode", ["ref", "bf16"])
def test_c_batch_plan_and_stack_equal_the_host_batch(gpu, sites, mode):
    """irc_batch_plan_create + irc_batch_stack (the route of a C or MATLAB
    host) build the same batch as the host code: same stacked matrix, same
    results through irc_knn_rho_delta_site, bit for bit."""
    b = batch.SiteBatch(sites)
    Fs = b.stack_device([torch.from_numpy(s["F"]).to(gpu) for s in sites])
    assert np.array_equal(Fs.cpu().numpy(), b.F)
    Pc, Ph = b.c_plan(), irc.Plan(b.plan)
    r1 = irc.knn_rho_delta_site(Pc, Fs, knn=30, mode=mode)
    r2 = irc.knn_rho_delta_site(Ph, torch.from_numpy(b.F).to(gpu), knn=30, mode=mode)
    for k in ("miKnn", "nneigh"):
        assert np.array_equal(r1[k].cpu().numpy(), r2[k].cpu().numpy()), k
    for k in ("rho", "delta"):
        assert np.array_equal(r1[k].cpu().numpy().view(np.int32), r2[k].cpu().numpy().view(np.int32)), k


def test_fused_entry_with_external_rho_and_errors(gpu, sites):
    """irc_knn_rho_delta_site with R given equals the two-call sequence with
    the same R; without R a plan whose queries are not all of F is refused."""
    import ctypes as C
    from ironclust_gb300 import _lib
    site = sites[2]
    plan = synth.site_plan(site)
    P = irc.Plan(plan)
    F = torch.from_numpy(site["F"]).to(gpu)
    k = irc.site_knn(P, F, 30, "exact")
    R = (k["rho"] * 0.5).contiguous()                 # any rho of every column
    d1, n1 = irc.site_delta(P, F, R, "exact", 512, 30, k["miKnn"], k["d2Knn"])
    n = P.n_out
    out = [torch.empty(n, dtype=torch.float32, device=gpu), torch.empty(n, dtype=torch.float32, device=gpu),
           torch.empty((n, 30), dtype=torch.int32, device=gpu), torch.empty((n, 30), dtype=torch.float32, device=gpu),
           torch.empty(n, dtype=torch.float32, device=gpu), torch.empty(n, dtype=torch.int32, device=gpu)]
    p = lambda t: C.c_void_p(t.data_ptr())
    L = _lib.lib()
    _lib.check(L.irc_knn_rho_delta_site(P.h, p(F), F.shape[1], p(R), 30, _lib.MODES["exact"], *[p(t) for t in out],
                                        irc._stream()), "irc_knn_rho_delta_site")
    assert np.array_equal(out[4].cpu().numpy().view(np.int32), d1.cpu().numpy().view(np.int32))
    assert np.array_equal(out[5].cpu().numpy(), n1.cpu().numpy())
    sub = dict(plan, n_f=F.shape[0] + 10)               # queries no longer all of F
    F2 = torch.cat([F, torch.zeros((10, F.shape[1]), device=gpu)])
    P2 = irc.Plan(sub)
    with pytest.raises(_lib.IrcError):
        _lib.check(L.irc_knn_rho_delta_site(P2.h, p(F2), F.shape[1], None, 30, _lib.MODES["exact"],
                                            *[p(t) for t in out], irc._stream()), "irc_knn_rho_delta_site")


def test_c_batch_plan_rejects_a_run_leaving_its_site(gpu, sites):
    import ctypes as C
    from ironclust_gb300 import _lib
    b = batch.SiteBatch(sites[:2])
    ps = b.site_plans
    rs = [p["rs"].copy() for p in ps]
    rs[0][-1] = int(b.sizes[0])                         # starts past the end of site 0
    cat = lambda parts: np.ascontiguousarray(np.concatenate(parts), np.int32)
    arrs = [np.array([len(p["q0"]) for p in ps], np.int32), np.ascontiguousarray(b.bases, np.int64),
            cat([p["q0"] for p in ps]), cat([p["nq"] for p in ps]), cat([p["roff"] for p in ps]), cat(rs),
            cat([p["rn"] for p in ps])]
    h = C.c_void_p()
    rc = _lib.lib().irc_batch_plan_create(C.byref(h), 2, *[a.ctypes.data_as(C.c_void_p) for a in arrs])
    assert rc != 0 and not h.value


@pytest.mark.parametrize("mode", ["bf16", "fp8"])
def test_site_dims_skip_padding_with_identical_results(gpu, sites, mode):
    """irc_plan_set_site_dims: the re-rank stops at each site's own width;
    the padded features are zero in both rows, so every output is the same
    bit for bit as without the widths."""
    b = batch.SiteBatch(sites)
    F = torch.from_numpy(b.F).to(gpu)
    P0, P1 = irc.Plan(b.plan), b.make_plan()
    r0 = irc.knn_rho_delta_site(P0, F, knn=30, mode=mode)
    r1 = irc.knn_rho_delta_site(P1, F, knn=30, mode=mode)
    for k in ("miKnn", "nneigh"):
        assert np.array_equal(r0[k].cpu().numpy(), r1[k].cpu().numpy()), k
    for k in ("rho", "delta", "d2Knn"):
        assert np.array_equal(r0[k].cpu().numpy().view(np.int32), r1[k].cpu().numpy().view(np.int32)), k
    P1.set_site_dims(np.zeros(1, np.int64), np.zeros(0, np.int32))       # nSites = 0 clears
    r2 = irc.knn_rho_delta_site(P1, F, knn=30, mode=mode)
    assert np.array_equal(r2["miKnn"].cpu().numpy(), r0["miKnn"].cpu().numpy())


def test_site_dims_reject_a_chunk_outside_its_site(gpu, sites):
    from ironclust_gb300 import _lib
    b = batch.SiteBatch(sites[:2])
    P = irc.Plan(b.plan)
    with pytest.raises(_lib.IrcError):                                   # sites split inside a chunk
        P.set_site_dims(np.array([0, 7, b.F.shape[0]], np.int64), np.array([18, 33], np.int32))
    with pytest.raises(_lib.IrcError):                                   # rows not covering nF
        P.set_site_dims(np.array([0, 10], np.int64), np.array([18], np.int32))
    with pytest.raises(_lib.IrcError):                                   # width out of range
        P.set_site_dims(np.ascontiguousarray(b.bases, np.int64), np.array([18, 99], np.int32))
    P.set_site_dims(b.bases, b.dims)
