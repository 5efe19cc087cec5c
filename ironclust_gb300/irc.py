"""Host-side mirror of IronClust's MATLAB hot-path wrappers over the C ABI.

The reference host is MATLAB; this module restates its wrappers in Python
so they can drive the sm_103a library (libircgb300.so) the way the MATLAB
code drives the reference kernels, and so the parity tests read like the
reference's call sites.  PyTorch only provides device memory and streams.

Feature matrices are torch float32 CUDA tensors of shape [n, nC] (C order),
which is byte-identical to MATLAB's column-major [nC x n].  Kernel outputs
MATLAB sees as [nT x nA] are returned as [nA, nT] tensors (same bytes).

Reference call sites mirrored here:
  search_knn_drift_    matlab/irc2.m:3731-3789   -> search_knn_drift
  search_delta_drift_  matlab/irc2.m:3794-3865   -> search_delta_drift_host
  rho_paged_site_      matlab/irc2.m:3635-3680   -> rho_site
  delta_paged_site_    matlab/irc2.m:3684-3726   -> delta_site
  sort_ normalisation  matlab/irc2.m:3263-3264   -> sort_rho
  postCluster_         matlab/irc2.m:6520-6535   -> post_cluster, assign_cluster_knn
  cuda_knn_            matlab/irc.m:24365-24401  -> cuda_knn
  cuda_delta_knn_      matlab/irc.m:24519-24553  -> cuda_delta_knn_host
  cuda_rho_drift_      matlab/irc.m:24612-24637  -> cuda_rho_drift
  cuda_delta_drift_    matlab/irc.m:24641-24666  -> cuda_delta_drift
  calc_dc2_drift_      matlab/irc.m:24582-24608  -> calc_dc2_drift
  cluster_drift_       matlab/irc.m:24041-24180  -> cluster_drift (GPU branch)
  rho_drift_knn_       matlab/irc.m:24336-24361  -> rho_drift_knn
  delta_drift_knn_     matlab/irc.m:24477-24515  -> delta_drift_knn
  cuda_knn__           matlab/irc.m:24437-24465  -> knn_vr
  calc_drift_          matlab/irc2.m:6373-6465   -> calc_drift
  cuda_rho_, cuda_delta_ (time-window mode) matlab/irc.m:2528-2560, :2651-2688
                                                 -> rho_spacetime, delta_spacetime
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, lib
from .drift import build_plan

SINGLE_INF = 3.402e38                       # MATLAB double literal
SQRT_SINGLE_INF_F = np.float32(np.sqrt(SINGLE_INF))   # single(sqrt(SINGLE_INF)), matlab/irc2.m:3725


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _i32host(v):
    return np.ascontiguousarray(v, dtype=np.int32)


def _dev_f32(x, device="cuda"):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float32).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(device)


def _dev_i32(x, device="cuda"):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.int32).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.int32)).to(device)


def _mode(mode):
    return _lib.MODES[mode] if isinstance(mode, str) else int(mode)


# ---------------------------------------------------------------------------
# drop-in kernels (one call == one MATLAB feval)
# ---------------------------------------------------------------------------

def search_min_drift(F, IBB, NBB, vnConst, nThreads=1024, mode="ref", knn=30):
    """feval(search_min_drift, D, I, F, IBB, NBB, vnConst); returns (D, I) as [nA, nThreads]."""
    vn = _i32host(vnConst)
    nA = int(vn[4])
    D = torch.empty((nA, nThreads), dtype=torch.float32, device=F.device)
    I = torch.empty((nA, nThreads), dtype=torch.int32, device=F.device)
    check(lib().irc_search_min_drift(_p(D), _p(I), _p(F), _p(IBB), _p(NBB),
                                     vn.ctypes.data_as(C.c_void_p), nThreads, _mode(mode), knn,
                                     _stream()), "irc_search_min_drift")
    return D, I


def search_delta_drift(F, R, IBB, NBB, vnConst, nThreads=512):
    vn = _i32host(vnConst)
    nA = int(vn[4])
    D = torch.empty((nA, nThreads), dtype=torch.float32, device=F.device)
    I = torch.empty((nA, nThreads), dtype=torch.int32, device=F.device)
    check(lib().irc_search_delta_drift(_p(D), _p(I), _p(F), _p(R), _p(IBB), _p(NBB),
                                       vn.ctypes.data_as(C.c_void_p), nThreads, _stream()),
          "irc_search_delta_drift")
    return D, I


def cuda_knn_index(B, A, knn, nThreads=512):
    """feval(cuda_knn_index, K, I, B, A, vnConst); returns K [nA], I [nA, knn]."""
    nB, nA, nC = B.shape[0], A.shape[0], A.shape[1]
    vn = _i32host([nB, nA, nC, knn])
    K = torch.empty(nA, dtype=torch.float32, device=A.device)
    I = torch.empty((nA, knn), dtype=torch.int32, device=A.device)
    check(lib().irc_cuda_knn_index(_p(K), _p(I), _p(B), _p(A), vn.ctypes.data_as(C.c_void_p),
                                   nThreads, _stream()), "irc_cuda_knn_index")
    return K, I


def cuda_delta_knn(B, A, R_B, R_A, nThreads=128):
    """feval(cuda_delta_knn, D, N, B, A, R_B, R_A, vnConst); returns D [nA], N [nA] (uint32 bits in int32)."""
    nB, nA, nC = B.shape[0], A.shape[0], A.shape[1]
    vn = _i32host([nB, nA, nC])
    D = torch.empty(nA, dtype=torch.float32, device=A.device)
    N = torch.empty(nA, dtype=torch.int32, device=A.device)
    check(lib().irc_cuda_delta_knn(_p(D), _p(N), _p(B), _p(A), _p(R_B), _p(R_A),
                                   vn.ctypes.data_as(C.c_void_p), nThreads, _stream()),
          "irc_cuda_delta_knn")
    return D, N


def rho_drift(miSite12_colmajor, mrFet1, mrFet2, n1, dc2):
    """feval(jrc3_cuda_rho_drift, vrRho1, miSite12, mrFet1, mrFet2, vnConst, dc2).
    miSite12_colmajor: int32 device tensor of 2*n12 entries (MATLAB [n12 x 2])."""
    n12, nC = mrFet1.shape
    vn = _i32host([n1, n12, nC])
    rho = torch.empty(n1, dtype=torch.float32, device=mrFet1.device)
    check(lib().irc_rho_drift(_p(rho), _p(miSite12_colmajor), _p(mrFet1), _p(mrFet2),
                              vn.ctypes.data_as(C.c_void_p), C.c_float(dc2), _stream()),
          "irc_rho_drift")
    return rho


def delta_drift(miSite12_colmajor, mrFet1, mrFet2, vrRho12, n1, dc2):
    """feval(jrc3_cuda_delta_drift, vrDelta1, viNneigh1, miSite12, mrFet1, mrFet2, vrRho1, vnConst, dc2).
    Returns delta [n1] and nneigh [n1] (1-based, uint32 bits in int32)."""
    n12, nC = mrFet1.shape
    vn = _i32host([n1, n12, nC])
    de = torch.empty(n1, dtype=torch.float32, device=mrFet1.device)
    nn = torch.empty(n1, dtype=torch.int32, device=mrFet1.device)
    check(lib().irc_delta_drift(_p(de), _p(nn), _p(miSite12_colmajor), _p(mrFet1), _p(mrFet2), _p(vrRho12),
                                vn.ctypes.data_as(C.c_void_p), C.c_float(dc2), _stream()), "irc_delta_drift")
    return de, nn


# ---------------------------------------------------------------------------
# MATLAB post-processing on the device
def cuda_knn_kth(B, A, knn, nThreads=256):
    """irc_cuda_knn (cuda_knn.cu): the knn-th binned-minimum distance [nA]."""
    K = torch.empty(A.shape[0], dtype=torch.float32, device=A.device)
    vn = _i32host([B.shape[0], A.shape[0], A.shape[1], knn])
    check(lib().irc_cuda_knn(_p(K), _p(B), _p(A), vn.ctypes.data_as(C.c_void_p), nThreads, _stream()),
          "irc_cuda_knn")
    return K


def cuda_knn_full(B, A, knn, nThreads=512):
    """irc_cuda_knn_full (cuda_knn_full.cu): K, I as [nA, knn] (== MATLAB [knn x nA])."""
    nA = A.shape[0]
    K = torch.empty((nA, knn), dtype=torch.float32, device=A.device)
    I = torch.empty((nA, knn), dtype=torch.int32, device=A.device)
    vn = _i32host([B.shape[0], nA, A.shape[1], knn])
    check(lib().irc_cuda_knn_full(_p(K), _p(I), _p(B), _p(A), vn.ctypes.data_as(C.c_void_p), nThreads,
                                  _stream()), "irc_cuda_knn_full")
    return K, I


def cuda_knn_ib(B, A, IB, knn, nThreads=512):
    """irc_cuda_knn_ib (cuda_knn_ib.cu): candidates = B columns IB (1-based)."""
    nA = A.shape[0]
    IB = _dev_i32(IB, A.device)
    K = torch.empty(nA, dtype=torch.float32, device=A.device)
    I = torch.empty((nA, knn), dtype=torch.int32, device=A.device)
    vn = _i32host([IB.numel(), nA, A.shape[1], knn])
    check(lib().irc_cuda_knn_ib(_p(K), _p(I), _p(B), _p(A), _p(IB), B.shape[0], vn.ctypes.data_as(C.c_void_p),
                                nThreads, _stream()), "irc_cuda_knn_ib")
    return K, I


def cuda_rho_st(mrFet12, ord12, n1, dn_max, dc2, fDc_spk=0):
    """irc_cuda_rho (jrc3_cuda_rho): time-window density of the first n1 spikes."""
    rho = torch.empty(n1, dtype=torch.float32, device=mrFet12.device)
    vn = _i32host([n1, mrFet12.shape[0], mrFet12.shape[1], dn_max, fDc_spk])
    check(lib().irc_cuda_rho(_p(rho), _p(mrFet12), _p(_dev_i32(ord12, mrFet12.device)),
                             vn.ctypes.data_as(C.c_void_p), C.c_float(dc2), _stream()), "irc_cuda_rho")
    return rho


def cuda_delta_st(mrFet12, ord12, rr12, n1, dn_max, dc2, fDc_spk=0, nThreads=128):
    """irc_cuda_delta (jrc3_cuda_delta): delta and nneigh (1-based) of the first n1 spikes."""
    de = torch.empty(n1, dtype=torch.float32, device=mrFet12.device)
    nn = torch.empty(n1, dtype=torch.int32, device=mrFet12.device)
    vn = _i32host([n1, mrFet12.shape[0], mrFet12.shape[1], dn_max, fDc_spk])
    check(lib().irc_cuda_delta(_p(de), _p(nn), _p(mrFet12), _p(_dev_i32(ord12, mrFet12.device)),
                               _p(_dev_i32(rr12, mrFet12.device)), vn.ctypes.data_as(C.c_void_p),
                               C.c_float(dc2), nThreads, _stream()), "irc_cuda_delta")
    return de, nn


# ---------------------------------------------------------------------------

def matlab_sort_knn(D, I, knn):
    """[vs, ord] = sort(D) (stable, NaN last); vrKnn = vs(knn,:); miKnn = I(ord(1:knn,:))."""
    key = torch.where(torch.isnan(D), torch.full_like(D, float("inf")), D)
    nanrank = torch.isnan(D).to(torch.int8)
    # stable sort by value, then a stable sort by the NaN flag keeps NaN last
    v, order = torch.sort(key, dim=1, stable=True)
    order = torch.gather(order, 1, torch.argsort(torch.gather(nanrank, 1, order), dim=1, stable=True))
    vs = torch.gather(D, 1, order)
    return vs[:, knn - 1].contiguous(), torch.gather(I, 1, order[:, :knn]).contiguous()


def matlab_min(D, I):
    """[vrMin, viMin] = min(D) over columns (first index, NaN skipped)."""
    key = torch.where(torch.isnan(D), torch.full_like(D, float("inf")), D)
    m = key.min(dim=1, keepdim=True).values
    first = (key == m).to(torch.int8).argmax(dim=1, keepdim=True)
    return torch.gather(D, 1, first).squeeze(1), torch.gather(I, 1, first).squeeze(1)


# ---------------------------------------------------------------------------
# per-chunk MATLAB loops (the unchanged host driving the drop-in kernels)
# ---------------------------------------------------------------------------

def search_knn_drift(plan, F, knn=30, nThreads=1024, mode="ref"):
    """search_knn_drift_ (matlab/irc2.m:3731-3789): one drop-in launch per
    drift chunk plus the MATLAB column sort.  Returns vrKnn [n_out], miKnn
    [n_out, knn] (1-based into F)."""
    n_out = plan["n_out"]
    vrKnn = torch.zeros(n_out, dtype=torch.float32, device=F.device)
    miKnn = torch.zeros((n_out, knn), dtype=torch.int32, device=F.device)
    nC, nF = F.shape[1], F.shape[0]
    for i in range(len(plan["q0"])):
        r0, r1 = int(plan["roff"][i]), int(plan["roff"][i + 1])
        IBB = _dev_i32(plan["rs"][r0:r1], F.device)
        NBB = _dev_i32(plan["rn"][r0:r1], F.device)
        q0, nq = int(plan["q0"][i]), int(plan["nq"][i])
        D, I = search_min_drift(F, IBB, NBB, [nC, nF, r1 - r0, q0, nq], nThreads, mode, knn)
        v, m = matlab_sort_knn(D, I, knn)
        o = q0 - plan["q_base"]
        vrKnn[o:o + nq] = v
        miKnn[o:o + nq] = m
    return vrKnn, miKnn


def search_delta_drift_host(plan, F, R, nThreads=512):
    """search_delta_drift_ (matlab/irc2.m:3794-3865): per-chunk launch + column min."""
    n_out = plan["n_out"]
    vrDelta = torch.zeros(n_out, dtype=torch.float32, device=F.device)
    viNneigh = torch.zeros(n_out, dtype=torch.int32, device=F.device)
    nC, nF = F.shape[1], F.shape[0]
    for i in range(len(plan["q0"])):
        r0, r1 = int(plan["roff"][i]), int(plan["roff"][i + 1])
        IBB = _dev_i32(plan["rs"][r0:r1], F.device)
        NBB = _dev_i32(plan["rn"][r0:r1], F.device)
        q0, nq = int(plan["q0"][i]), int(plan["nq"][i])
        D, I = search_delta_drift(F, R, IBB, NBB, [nC, nF, r1 - r0, q0, nq], nThreads)
        v, m = matlab_min(D, I)
        o = q0 - plan["q_base"]
        vrDelta[o:o + nq] = v
        viNneigh[o:o + nq] = m
    return vrDelta, viNneigh


# ---------------------------------------------------------------------------
# fused per-site path
# ---------------------------------------------------------------------------

class Plan:
    """Device-resident launch plan of one site (irc_plan_create)."""

    def __init__(self, plan):
        self.d = plan
        self.h = C.c_void_p()
        arrs = [_i32host(plan[k]) for k in ("q0", "nq", "roff", "rs", "rn")]
        self._keep = arrs
        check(lib().irc_plan_create(C.byref(self.h), *[a.ctypes.data_as(C.c_void_p) for a in arrs],
                                    len(arrs[0]), int(plan["q_base"]), int(plan["n_out"]),
                                    int(plan["n_f"])), "irc_plan_create")

    @classmethod
    def from_drift(cls, viDrift_out, vl_in, mlDrift):
        return cls(build_plan(viDrift_out, vl_in, mlDrift))

    @classmethod
    def from_handle(cls, handle, plan):
        """Wrap a plan the library created (irc_batch_plan_create); plan = its
        arrays as a dict, for host-side use."""
        self = cls.__new__(cls)
        self.d, self.h, self._keep = plan, handle, []
        return self

    @property
    def n_out(self):
        return int(self.d["n_out"])

    def set_site_dims(self, row_base, dims):
        """irc_plan_set_site_dims: rows row_base[k] .. row_base[k+1]-1 form
        site k, whose features past dims[k] are zero (a stacked batch)."""
        rb = np.ascontiguousarray(row_base, np.int64)
        dd = np.ascontiguousarray(dims, np.int32)
        check(lib().irc_plan_set_site_dims(self.h, len(dd), rb.ctypes.data_as(C.c_void_p),
                                           dd.ctypes.data_as(C.c_void_p)), "irc_plan_set_site_dims")
        return self

    def close(self):
        if self.h:
            lib().irc_plan_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def site_knn(plan, F, knn=30, mode="ref", nThreads=1024, want_d2=None):
    """irc_site_knn: kNN + rho of every query of the plan.
    Returns dict(vrKnn, rho, miKnn [n_out, knn] 1-based, d2Knn or None)."""
    n = plan.n_out
    dev = F.device
    vrKnn = torch.empty(n, dtype=torch.float32, device=dev)
    rho = torch.empty(n, dtype=torch.float32, device=dev)
    miKnn = torch.empty((n, knn), dtype=torch.int32, device=dev)
    m = _mode(mode)
    if want_d2 is None:
        want_d2 = m != _lib.MODE_REF
    d2 = torch.empty((n, knn), dtype=torch.float32, device=dev) if want_d2 else None
    check(lib().irc_site_knn(plan.h, _p(F), F.shape[1], knn, nThreads, m, _p(vrKnn), _p(rho),
                             _p(miKnn), _p(d2), _stream()), "irc_site_knn")
    return dict(vrKnn=vrKnn, rho=rho, miKnn=miKnn, d2Knn=d2)


def site_delta(plan, F, R, mode="ref", nThreads=512, knn=30, miKnn=None, d2Knn=None):
    """irc_site_delta: delta (= nearest higher-rho distance .* rho) and nneigh (1-based)."""
    n = plan.n_out
    delta = torch.empty(n, dtype=torch.float32, device=F.device)
    nneigh = torch.empty(n, dtype=torch.int32, device=F.device)
    check(lib().irc_site_delta(plan.h, _p(F), F.shape[1], _p(R), nThreads, _mode(mode), knn,
                               _p(miKnn), _p(d2Knn), _p(delta), _p(nneigh), _stream()),
          "irc_site_delta")
    return delta, nneigh


def knn_rho_delta_site(plan, F, knn=30, mode="ref", nThreads_rho=1024, nThreads_delta=512):
    """One single-page site (or a batch plan) end to end: kNN, rho = 1/d_knn,
    delta, nneigh -- one irc_knn_rho_delta_site call with MATLAB's bin counts.
    Requires every column of F to be a query (the plan covers all of F)."""
    if plan.n_out != F.shape[0] or int(plan.d["q_base"]) != 0:
        raise ValueError("knn_rho_delta_site: the plan must cover every column of F")
    if (nThreads_rho, nThreads_delta) != (1024, 512):
        k = site_knn(plan, F, knn, mode, nThreads_rho)
        delta, nneigh = site_delta(plan, F, k["rho"], mode, nThreads_delta, knn, k["miKnn"], k["d2Knn"])
        k.update(delta=delta, nneigh=nneigh)
        return k
    n, dev = plan.n_out, F.device
    m = _mode(mode)
    out = dict(vrKnn=torch.empty(n, dtype=torch.float32, device=dev),
               rho=torch.empty(n, dtype=torch.float32, device=dev),
               miKnn=torch.empty((n, knn), dtype=torch.int32, device=dev),
               d2Knn=torch.empty((n, knn), dtype=torch.float32, device=dev) if m != _lib.MODE_REF else None,
               delta=torch.empty(n, dtype=torch.float32, device=dev),
               nneigh=torch.empty(n, dtype=torch.int32, device=dev))
    check(lib().irc_knn_rho_delta_site(plan.h, _p(F), F.shape[1], None, knn, m, _p(out["vrKnn"]), _p(out["rho"]),
                                       _p(out["miKnn"]), _p(out["d2Knn"]), _p(out["delta"]), _p(out["nneigh"]),
                                       _stream()), "irc_knn_rho_delta_site")
    return out


# ---------------------------------------------------------------------------
# rho_paged_site_ / delta_paged_site_ / sort_ post-processing (host logic)
# ---------------------------------------------------------------------------

def rho_post(vrKnn, miKnn, viSpk_out, knn):
    """rho = 1 ./ vrKnn; miKnn -> global int64 ids; pad rows to knn by
    repeating the last (matlab/irc2.m:3669-3676).  numpy in, numpy out."""
    vrKnn = np.asarray(vrKnn, np.float32)
    with np.errstate(divide="ignore"):
        rho = (np.float32(1.0) / vrKnn).astype(np.float32)
    mi = np.asarray(viSpk_out, np.int64)[np.asarray(miKnn, np.int64) - 1]
    if mi.shape[1] < knn:
        mi = np.concatenate([mi, np.repeat(mi[:, -1:], knn - mi.shape[1], axis=1)], axis=1)
    return rho, mi


def delta_post(vrDelta_times_rho, viNneigh, viSpk_out):
    """nneigh -> global id; NaN/Inf delta -> sqrt(SINGLE_INF) with nneigh set
    to the spike's own local position (matlab/irc2.m:3720-3725, kept as is)."""
    d = np.asarray(vrDelta_times_rho, np.float32).copy()
    nn = np.asarray(viSpk_out, np.int64)[np.asarray(viNneigh, np.int64) - 1]
    bad = np.flatnonzero(~np.isfinite(d))
    nn[bad] = bad + 1
    d[bad] = SQRT_SINGLE_INF_F
    return d, nn


def _dev_i64(x, device="cuda"):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.int64).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.int64)).to(device)


def sort_rho(vrRho):
    """sort_'s output normalisation on the device (matlab/irc2.m:3263-3264):
    vrRho / max(vrRho) (NaN skipped by max) and ordrho = the 1-based order of
    sort(vrRho, 'descend') (NaN first, ties in index order).  Returns CUDA
    tensors (float32 [n], int64 [n]); the input is not modified."""
    r = _dev_f32(vrRho).clone()
    order = torch.empty(r.numel(), dtype=torch.int64, device=r.device)
    check(lib().irc_sort_rho(_p(r), _p(order), C.c_int64(r.numel()), _stream()), "irc_sort_rho")
    return r, order


def assign_cluster_knn(rho, delta, ordrho, nneigh, miKnn, delta_cut=1.0, min_count=0):
    """The cluster assignment of postCluster_ (matlab/irc2.m:6520-6535):
    assignCluster_knn_ (:6640-6694) + dpclus_remove_count_ (:6735-6750).

    rho, delta: [n] normalised (as sort_ leaves them); ordrho, nneigh: [n]
    1-based; miKnn: [n, knn] kNN ids of every spike (row s = MATLAB column
    s).  Returns dict(viClu [n] int32, icl [nClu] int64 1-based centres,
    vnSpk_clu [nClu] int32, nClu, nClu_pre, nClu_post); tensors on the
    device."""
    rho, delta = _dev_f32(rho), _dev_f32(delta)
    dev = rho.device
    ordrho, nneigh, mk = _dev_i64(ordrho, dev), _dev_i64(nneigh, dev), _dev_i64(miKnn, dev)
    n = rho.numel()
    if mk.dim() != 2 or mk.shape[0] != n:
        raise ValueError("assign_cluster_knn: miKnn must be [nSpk, knn]")
    viClu = torch.empty(n, dtype=torch.int32, device=dev)
    icl = torch.empty(n, dtype=torch.int64, device=dev)
    vn = torch.empty(n, dtype=torch.int32, device=dev)
    counts = np.zeros(3, np.int64)
    check(lib().irc_assign_cluster_knn(_p(viClu), _p(icl), _p(vn), C.c_int64(n),
                                       counts.ctypes.data_as(C.c_void_p), _p(rho), _p(delta), _p(ordrho),
                                       _p(nneigh), _p(mk), C.c_int(mk.shape[1]), C.c_int64(n),
                                       C.c_float(delta_cut), C.c_int(min_count), _stream()),
          "irc_assign_cluster_knn")
    k = int(counts[0])
    return dict(viClu=viClu, icl=icl[:k], vnSpk_clu=vn[:k], nClu=k, nClu_pre=int(counts[1]),
                nClu_post=int(counts[2]))


def post_cluster(S_clu, P=None):
    """postCluster_ (matlab/irc2.m:6520-6535) on the device.  S_clu holds
    rho, delta, ordrho, nneigh (as sort_ leaves them) and miKnn [n, knn];
    P may set delta_cut (default 1) and min_count (default 0).  Returns the
    S_auto fields viClu, icl, nClu, vnSpk_clu, nSpk_unique, plus nClu_pre
    and nClu_post (the counts postCluster_ prints)."""
    P = P or {}
    a = assign_cluster_knn(S_clu["rho"], S_clu["delta"], S_clu["ordrho"], S_clu["nneigh"], S_clu["miKnn"],
                           float(P.get("delta_cut", 1.0)), int(P.get("min_count", 0)))
    a["nSpk_unique"] = int(a["vnSpk_clu"].sum().item()) if a["nClu"] else 0
    return a


# ---------------------------------------------------------------------------
# irc.m (v4) wrappers
# ---------------------------------------------------------------------------

def cuda_knn(mrFet, vi2, vi1, knn=30, nC_max=45):
    """cuda_knn_ (matlab/irc.m:24365-24401): gathers B = mrFet(:,vi2),
    A = mrFet(:,vi1) (0-based index vectors here), knn = min(knn, n2).
    Returns vrKnn [n1], miKnn [n1, knn] mapped through vi2 (0-based)."""
    if mrFet.shape[1] > nC_max:
        raise ValueError("cuda_knn: nC > nC_max (the reference falls back to the CPU)")
    vi2 = torch.as_tensor(vi2, device=mrFet.device, dtype=torch.long)
    vi1 = torch.as_tensor(vi1, device=mrFet.device, dtype=torch.long)
    knn = min(knn, vi2.numel())
    K, I = cuda_knn_index(mrFet[vi2].contiguous(), mrFet[vi1].contiguous(), knn)
    return K, vi2[I.long() - 1]


def cuda_delta_knn_host(mrFet, vrRho, vi2, vi1):
    """cuda_delta_knn_ (matlab/irc.m:24519-24553); returns D [n1] and N (0-based
    through vi2; the reference's self-index fallback is an A-space index that
    MATLAB also maps through vi2)."""
    vi2 = torch.as_tensor(vi2, device=mrFet.device, dtype=torch.long)
    vi1 = torch.as_tensor(vi1, device=mrFet.device, dtype=torch.long)
    D, N = cuda_delta_knn(mrFet[vi2].contiguous(), mrFet[vi1].contiguous(),
                          vrRho[vi2].contiguous(), vrRho[vi1].contiguous())
    return D, vi2[N.long() - 1]


def cuda_delta_drift(viSite1, viSite2, mrFet1, mrFet2, vrRho12, n1, dc2):
    """cuda_delta_drift_ (matlab/irc.m:24641-24666) for one drift window of
    n12 spikes (own chunk first): delta = sqrt(min d2 / dc2) and nneigh
    (1-based into the window)."""
    site = torch.cat([torch.as_tensor(viSite1, dtype=torch.int32),
                      torch.as_tensor(viSite2, dtype=torch.int32)]).to(mrFet1.device)
    return delta_drift(site, mrFet1.contiguous(), mrFet2.contiguous(),
                       torch.as_tensor(vrRho12, dtype=torch.float32, device=mrFet1.device).contiguous(),
                       n1, float(np.float32(dc2)))


def cuda_rho_drift(viSite1, viSite2, mrFet1, mrFet2, n1, dc2):
    """cuda_rho_drift_ (matlab/irc.m:24612-24637) for one drift window of
    n12 spikes (own chunk first, n1 of them)."""
    site = torch.cat([torch.as_tensor(viSite1, dtype=torch.int32),
                      torch.as_tensor(viSite2, dtype=torch.int32)]).to(mrFet1.device)
    return rho_drift(site, mrFet1.contiguous(), mrFet2.contiguous(), n1, float(np.float32(dc2)))


def knn_vr(mrFet, vi2, vi1, knn=30, nThreads=256):
    """cuda_knn__ (matlab/irc.m:24437-24465): the knn-th binned-minimum
    distance of each spike vi1 (0-based indices) among vi2, knn = min(knn, n2)."""
    vi2 = torch.as_tensor(vi2, device=mrFet.device, dtype=torch.long)
    vi1 = torch.as_tensor(vi1, device=mrFet.device, dtype=torch.long)
    return cuda_knn_kth(mrFet[vi2].contiguous(), mrFet[vi1].contiguous(), min(knn, vi2.numel()), nThreads)


def calc_dc2_drift(n1, viSite1, viSite2, mrFet1, mrFet2, n_sites, dc_subsample=1000, dc_percent=2.0):
    """calc_dc2_drift_ (matlab/irc.m:24582-24608) on the device
    (irc_calc_dc2_drift): the distance cut-off of the time-drift mode for one
    window (own chunk's n1 spikes first).  viSite1/viSite2: host int arrays of
    1-based sites; mrFet1/mrFet2: device [n12, nC] primary / secondary
    features.  Returns (dc2, dc2_site [n_sites], NaN where a site has no
    queries)."""
    s1, s2 = _i32host(viSite1), _i32host(viSite2)
    f1, f2 = _dev_f32(mrFet1, mrFet1.device), _dev_f32(mrFet2, mrFet1.device)
    dc2 = C.c_float()
    site = np.zeros(n_sites, np.float32)
    check(lib().irc_calc_dc2_drift(C.byref(dc2), site.ctypes.data_as(C.c_void_p), int(n1), int(f1.shape[0]),
                                   int(f1.shape[1]), s1.ctypes.data_as(C.c_void_p), s2.ctypes.data_as(C.c_void_p),
                                   _p(f1), _p(f2), int(n_sites), int(dc_subsample), float(dc_percent), _stream()),
          "irc_calc_dc2_drift")
    return np.float32(dc2.value), site


def drift_windows(cviSpk_drift, miSort_drift):
    """The drift windows of cluster_drift_ (matlab/irc.m:24084-24087): window
    i = the spikes of chunks miSort_drift[:, i] (0-based chunk ids, its own
    chunk first), concatenated; returns [(own spikes, window spikes)]."""
    return [(np.asarray(own, np.int64),
             np.concatenate([np.asarray(cviSpk_drift[j], np.int64) for j in miSort_drift[:, i]]))
            for i, own in enumerate(cviSpk_drift)]


def cluster_drift(viSite_spk, viSite2_spk, F1, F2, cviSpk_drift, miSort_drift, n_sites, dc_subsample=1000,
                  dc_percent=2.0):
    """rho, delta and nneigh of the time-drift mode (vcCluster = 'drift'):
    the GPU branch of cluster_drift_ (matlab/irc.m:24041-24180).  dc2 comes
    from the first window (calc_dc2_drift_); rho then delta window by window
    (jrc3_cuda_rho_drift / jrc3_cuda_delta_drift, the window's own spikes
    first); NaN deltas become the largest delta.  viSite_spk, viSite2_spk:
    host 1-based sites of every spike; F1, F2: device [nSpk, nC] primary /
    secondary features.  Returns dict(rho, delta, nneigh (0-based global),
    dc2, dc2_site)."""
    dev = F1.device
    n = F1.shape[0]
    rho = torch.zeros(n, dtype=torch.float32, device=dev)
    delta = torch.zeros(n, dtype=torch.float32, device=dev)
    nneigh = torch.zeros(n, dtype=torch.int64, device=dev)
    s1_all, s2_all = np.asarray(viSite_spk, np.int32), np.asarray(viSite2_spk, np.int32)
    wins = drift_windows(cviSpk_drift, miSort_drift)
    dc2 = site = None
    for own, w in wins:
        wt = torch.as_tensor(w, device=dev)
        f1, f2 = F1[wt].contiguous(), F2[wt].contiguous()
        if dc2 is None:
            dc2, site = calc_dc2_drift(len(own), s1_all[w], s2_all[w], f1, f2, n_sites, dc_subsample, dc_percent)
        rho[torch.as_tensor(own, device=dev)] = cuda_rho_drift(s1_all[w], s2_all[w], f1, f2, len(own), dc2)
    for own, w in wins:
        wt = torch.as_tensor(w, device=dev)
        d, nn = cuda_delta_drift(s1_all[w], s2_all[w], F1[wt].contiguous(), F2[wt].contiguous(), rho[wt],
                                 len(own), dc2)
        ot = torch.as_tensor(own, device=dev)
        delta[ot] = d
        nneigh[ot] = wt[nn.long() - 1]
    bad = torch.isnan(delta)
    if bad.any():
        delta[bad] = delta[~bad].max()
    return dict(rho=rho, delta=delta, nneigh=nneigh, dc2=dc2, dc2_site=site)


def rho_drift_knn(mrFet12, viDrift_spk12, mlDrift, n1, knn=30, nC_max=45):
    """rho_drift_knn_ (matlab/irc.m:24336-24361) for one site: for every drift
    chunk, its own spikes (among the first n1) against the spikes of the
    chunks linked to it (mlDrift[candidate chunk, chunk]) through cuda_knn_
    (cuda_knn_index, knn = min(knn, n2)); rho = 1 ./ vrKnn; kNN lists shorter
    than knn padded by repeating their last row.  viDrift_spk12: host 1-based
    chunk ids of the n12 spikes; mlDrift: host bool [nT x nT].  Returns
    (rho [n1], miKnn [n1, knn] 0-based into mrFet12)."""
    vd = np.asarray(viDrift_spk12, np.int64)
    ml = np.asarray(mlDrift, bool)
    dev = mrFet12.device
    rho = torch.zeros(n1, dtype=torch.float32, device=dev)
    miKnn = torch.zeros((n1, knn), dtype=torch.long, device=dev)
    for d in range(1, ml.shape[0] + 1):
        vi1 = np.flatnonzero(vd[:n1] == d)
        if not vi1.size:
            continue
        vi2 = np.flatnonzero(ml[vd - 1, d - 1])
        K, I = cuda_knn(mrFet12, vi2, vi1, knn, nC_max)
        t1 = torch.as_tensor(vi1, device=dev)
        rho[t1] = 1.0 / K
        if I.shape[1] < knn:
            I = torch.cat([I, I[:, -1:].expand(-1, knn - I.shape[1])], 1)
        miKnn[t1] = I
    return rho, miKnn


def delta_drift_knn(mrFet12, viDrift_spk12, mlDrift, vrRho12, n1):
    """delta_drift_knn_ (matlab/irc.m:24477-24515) for one site: for every
    drift chunk, cuda_delta_knn_ (cuda_delta_knn) of its own spikes against
    the spikes of its linked chunks; delta .*= rho; a NaN or Inf delta becomes
    sqrt(SINGLE_INF) with the spike's own position as nneigh.  Returns (delta
    [n1], nneigh [n1] 0-based into mrFet12)."""
    vd = np.asarray(viDrift_spk12, np.int64)
    ml = np.asarray(mlDrift, bool)
    dev = mrFet12.device
    delta = torch.zeros(n1, dtype=torch.float32, device=dev)
    nneigh = torch.zeros(n1, dtype=torch.long, device=dev)
    for d in range(1, ml.shape[0] + 1):
        vi1 = np.flatnonzero(vd[:n1] == d)
        if not vi1.size:
            continue
        vi2 = np.flatnonzero(ml[vd - 1, d - 1])
        D, N = cuda_delta_knn_host(mrFet12, vrRho12, vi2, vi1)
        t1 = torch.as_tensor(vi1, device=dev)
        delta[t1] = D
        nneigh[t1] = N
    delta = delta * vrRho12[:n1]
    bad = ~torch.isfinite(delta)
    pos = torch.arange(n1, device=dev)
    nneigh = torch.where(bad, pos, nneigh)
    delta = torch.where(bad, torch.full_like(delta, float(SQRT_SINGLE_INF_F)), delta)
    return delta, nneigh


def _dn_max(n1, n2, nTime_clu):
    from .drift import matlab_round
    return int(matlab_round((n1 + n2) / nTime_clu))


def rho_spacetime(mrFet12, viiSpk12_ord, n1, n2, dc2, nTime_clu, fDc_spk=0):
    """cuda_rho_ (matlab/irc.m:2528-2560), GPU branch: dn_max =
    round((n1 + n2) / nTime_clu); mrFet12 [n12, nC] with the n1 queries first."""
    return cuda_rho_st(mrFet12.contiguous(), viiSpk12_ord, n1, _dn_max(n1, n2, nTime_clu),
                       float(np.float32(dc2)), fDc_spk)


def delta_spacetime(mrFet12, viiSpk12_ord, viiRho12_ord, n1, n2, dc2, nTime_clu, fDc_spk=0, nThreads=128):
    """cuda_delta_ (matlab/irc.m:2651-2688), GPU branch (an empty or NaN dc2
    becomes 1, as there)."""
    if dc2 is None or np.isnan(dc2):
        dc2 = 1.0
    return cuda_delta_st(mrFet12.contiguous(), viiSpk12_ord, viiRho12_ord, n1, _dn_max(n1, n2, nTime_clu),
                         float(np.float32(dc2)), fDc_spk, nThreads)


def calc_drift(vrAmp_spk, vrPos_spk, n_sites, nTime_drift, nTime_batch, nTime_max_drift=256,
               nQuantile_drift=10, members=False):
    """calc_drift_ (matlab/irc2.m:6373-6465) on the device (irc_calc_drift).

    vrAmp_spk, vrPos_spk: [nSpk] spike amplitudes and positions (numpy or
    CUDA tensors).  Returns (viLim_drift, mlDrift): 0-based chunk limits
    [n+1] (chunk i = spikes viLim[i]..viLim[i+1]-1) and the linkage matrix
    (mlDrift[i, j]: chunk i is among the nTime_batch nearest of chunk j);
    with members=True also the [nTime_batch, n] member lists in distance
    order."""
    from .drift import mi2ml_drift
    amp, pos = _dev_f32(vrAmp_spk), _dev_f32(vrPos_spk, vrAmp_spk.device if isinstance(vrAmp_spk, torch.Tensor)
                                            else "cuda")
    n_spk = amp.numel()
    n_cap = max(int(nTime_drift), 1)
    nb = max(int(nTime_batch), 1)
    mi = torch.empty((n_cap, nb), dtype=torch.int32, device=amp.device)
    lim = torch.empty(n_cap + 1, dtype=torch.int64, device=amp.device)
    n_out = C.c_int(0)
    check(lib().irc_calc_drift(_p(mi), _p(lim), C.byref(n_out), _p(amp), _p(pos), C.c_int64(n_spk), int(n_sites),
                               int(nTime_drift), int(nTime_batch), int(nTime_max_drift), int(nQuantile_drift),
                               _stream()), "irc_calc_drift")
    n = n_out.value
    lim_h = lim[: n + 1].cpu().numpy()
    if n == 1:
        ml = np.ones((1, 1), bool)
        mem = np.zeros((1, 1), np.int64)
    else:
        mem = mi[:n].cpu().numpy().astype(np.int64).T          # [nTime_batch, n]
        ml = mi2ml_drift(mem)
    return (lim_h, ml, mem) if members else (lim_h, ml)
