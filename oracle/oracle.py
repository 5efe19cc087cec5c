"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker.  The shipped library never
calls it.

* ``search_min_drift`` ... ``rho_drift``: CPU restatements of the reference
  kernels (irc_oracle.c), bit-for-bit.
* ``post_sort_knn`` / ``post_min``: the MATLAB post-processing of their
  outputs (matlab/irc2.m:3784-3787, :3855-3857).
* ``exact_knn_f64`` / ``exact_delta_f64``: double-precision ground truth.
* ``site_knn_cpu`` / ``site_delta_cpu``: the reference CPU path (knn_cpu_,
  delta_cpu_), also the timed CPU baseline.
* ``calc_dc2_drift``: the distance cut-off of the time-drift clustering mode
  (calc_dc2_drift_, matlab/irc.m:24582-24608).
* ``sort_rho`` / ``assign_cluster_knn``: the clustering step after the
  path -- sort_'s rho normalisation and ordrho (matlab/irc2.m:3263-3264),
  postCluster_ / assignCluster_knn_ / cell2map_ / dpclus_remove_count_
  (matlab/irc2.m:6520-6805), restated in irc_oracle_cluster.c.
* ``RefKernels``: the reference's own CUDA kernels (PTX built from the
  reference sources) launched with the MATLAB launch configuration on a GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None
_P = C.c_void_p


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build_oracle_lib()
        _lib = C.CDLL(path)
        for name in ("orc_search_min_drift", "orc_search_delta_drift", "orc_cuda_knn_index",
                     "orc_cuda_delta_knn", "orc_rho_drift", "orc_post_sort_knn", "orc_post_min",
                     "orc_exact_knn_f64", "orc_exact_delta_f64", "orc_knn_cpu", "orc_delta_cpu",
                     "orc_site_knn_cpu", "orc_site_delta_cpu", "orc_exact_knn_f32",
                     "orc_exact_delta_f32", "orc_delta_drift", "orc_sort_rho", "orc_cuda_knn",
                     "orc_cuda_knn_full", "orc_cuda_knn_ib", "orc_cuda_rho", "orc_cuda_delta"):
            getattr(_lib, name).restype = None
        _lib.orc_assign_cluster_knn.restype = C.c_int
        _lib.orc_calc_dc2_drift.restype = C.c_float
        _lib.orc_calc_dc2_drift.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, C.c_int, C.c_int,
                                            C.c_double]
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _fet(F):
    """Features as a C-contiguous [n, nC] float32 array (== MATLAB [nC x n])."""
    F = _f32(F)
    assert F.ndim == 2
    return F


# --- kernel restatements ------------------------------------------------------

def search_min_drift(F, IBB, NBB, vnConst, nT=1024):
    F = _fet(F)
    vn = _i32(vnConst)
    nA = int(vn[4])
    D = np.empty((nA, nT), np.float32)
    I = np.empty((nA, nT), np.int32)
    lib().orc_search_min_drift(_ptr(D), _ptr(I), _ptr(F), _ptr(_i32(IBB)), _ptr(_i32(NBB)),
                               _ptr(vn), C.c_int(nT))
    return D, I       # row a = MATLAB column a of the [nT x nA] output


def search_delta_drift(F, R, IBB, NBB, vnConst, nT=512):
    F = _fet(F)
    vn = _i32(vnConst)
    nA = int(vn[4])
    D = np.empty((nA, nT), np.float32)
    I = np.empty((nA, nT), np.int32)
    lib().orc_search_delta_drift(_ptr(D), _ptr(I), _ptr(F), _ptr(_f32(R)), _ptr(_i32(IBB)),
                                 _ptr(_i32(NBB)), _ptr(vn), C.c_int(nT))
    return D, I


def cuda_knn_index(B, A, knn, nT=512):
    B, A = _fet(B), _fet(A)
    nB, nA, nC = B.shape[0], A.shape[0], A.shape[1]
    vn = _i32([nB, nA, nC, knn])
    K = np.empty(nA, np.float32)
    I = np.empty((nA, knn), np.int32)
    lib().orc_cuda_knn_index(_ptr(K), _ptr(I), _ptr(B), _ptr(A), _ptr(vn), C.c_int(nT))
    return K, I


def cuda_knn(B, A, knn, nT=256):
    B, A = _fet(B), _fet(A)
    vn = _i32([B.shape[0], A.shape[0], A.shape[1], knn])
    K = np.empty(A.shape[0], np.float32)
    lib().orc_cuda_knn(_ptr(K), _ptr(B), _ptr(A), _ptr(vn), C.c_int(nT))
    return K


def cuda_knn_full(B, A, knn, nT=512):
    B, A = _fet(B), _fet(A)
    nA = A.shape[0]
    vn = _i32([B.shape[0], nA, A.shape[1], knn])
    K = np.empty((nA, knn), np.float32)
    I = np.empty((nA, knn), np.int32)
    lib().orc_cuda_knn_full(_ptr(K), _ptr(I), _ptr(B), _ptr(A), _ptr(vn), C.c_int(nT))
    return K, I


def cuda_knn_ib(B, A, IB, knn, nT=512):
    """IB: 1-based B columns (the candidates)."""
    B, A, IB = _fet(B), _fet(A), _i32(IB)
    nA = A.shape[0]
    vn = _i32([IB.size, nA, A.shape[1], knn])
    K = np.empty(nA, np.float32)
    I = np.empty((nA, knn), np.int32)
    lib().orc_cuda_knn_ib(_ptr(K), _ptr(I), _ptr(B), _ptr(A), _ptr(IB), _ptr(vn), C.c_int(nT))
    return K, I


def cuda_rho(mrFet12, ord12, n1, dn_max, dc2, fDc_spk=0):
    F = _fet(mrFet12)
    vn = _i32([n1, F.shape[0], F.shape[1], dn_max, fDc_spk])
    rho = np.empty(n1, np.float32)
    lib().orc_cuda_rho(_ptr(rho), _ptr(F), _ptr(_i32(ord12)), _ptr(vn), C.c_float(dc2))
    return rho


def cuda_delta(mrFet12, ord12, rr12, n1, dn_max, dc2, fDc_spk=0, nT=128):
    F = _fet(mrFet12)
    vn = _i32([n1, F.shape[0], F.shape[1], dn_max, fDc_spk])
    de = np.empty(n1, np.float32)
    nn = np.empty(n1, np.uint32)
    lib().orc_cuda_delta(_ptr(de), _ptr(nn), _ptr(F), _ptr(_i32(ord12)), _ptr(_i32(rr12)), _ptr(vn),
                         C.c_float(dc2), C.c_int(nT))
    return de, nn


def cuda_delta_knn(B, A, R_B, R_A, nT=128):
    B, A = _fet(B), _fet(A)
    nB, nA, nC = B.shape[0], A.shape[0], A.shape[1]
    vn = _i32([nB, nA, nC])
    D = np.empty(nA, np.float32)
    N = np.empty(nA, np.uint32)
    lib().orc_cuda_delta_knn(_ptr(D), _ptr(N), _ptr(B), _ptr(A), _ptr(_f32(R_B)), _ptr(_f32(R_A)),
                             _ptr(vn), C.c_int(nT))
    return D, N


def rho_drift(miSite12, mrFet1, mrFet2, n1, dc2):
    """miSite12: [n12, 2] (primary, secondary site); features [n12, nC]."""
    f1, f2 = _fet(mrFet1), _fet(mrFet2)
    n12, nC = f1.shape
    site = _i32(np.asarray(miSite12).T)           # MATLAB column-major [n12 x 2]
    vn = _i32([n1, n12, nC])
    rho = np.empty(n1, np.float32)
    lib().orc_rho_drift(_ptr(rho), _ptr(site), _ptr(f1), _ptr(f2), _ptr(vn), C.c_float(dc2))
    return rho


def delta_drift(miSite12, mrFet1, mrFet2, rho, n1, dc2):
    """jrc3_cuda_delta_drift restated; rho: [n12]."""
    f1, f2 = _fet(mrFet1), _fet(mrFet2)
    n12, nC = f1.shape
    site = _i32(np.asarray(miSite12).T)
    vn = _i32([n1, n12, nC])
    de = np.empty(n1, np.float32)
    nn = np.empty(n1, np.uint32)
    lib().orc_delta_drift(_ptr(de), _ptr(nn), _ptr(site), _ptr(f1), _ptr(f2), _ptr(_f32(rho)), _ptr(vn),
                          C.c_float(dc2))
    return de, nn


# --- MATLAB post-processing ----------------------------------------------------

def post_sort_knn(D, I, knn):
    D, I = _f32(D), _i32(I)
    nA, nT = D.shape
    vr = np.empty(nA, np.float32)
    mi = np.empty((nA, knn), np.int32)
    lib().orc_post_sort_knn(_ptr(D), _ptr(I), C.c_int(nT), C.c_int(nA), C.c_int(knn),
                            _ptr(vr), _ptr(mi))
    return vr, mi


def post_min(D, I):
    D, I = _f32(D), _i32(I)
    nA, nT = D.shape
    vr = np.empty(nA, np.float32)
    vi = np.empty(nA, np.int32)
    lib().orc_post_min(_ptr(D), _ptr(I), C.c_int(nT), C.c_int(nA), _ptr(vr), _ptr(vi))
    return vr, vi


# --- plan-level references -------------------------------------------------------

def _plan_args(plan):
    return [_i32(plan[k]) for k in ("q0", "nq", "roff", "rs", "rn")]


def exact_knn_f64(F, plan, knn, exclude_zero=True):
    F = _fet(F)
    q0, nq, roff, rs, rn = _plan_args(plan)
    qb, nout = int(plan["q_base"]), int(plan["n_out"])
    idx = np.zeros((nout, knn), np.int32)
    d2 = np.full((nout, knn), np.nan)
    lib().orc_exact_knn_f64(_ptr(idx), _ptr(d2), _ptr(F), C.c_int(F.shape[1]), _ptr(q0), _ptr(nq),
                            _ptr(roff), _ptr(rs), _ptr(rn), C.c_int(len(q0)), C.c_int(qb),
                            C.c_int(knn), C.c_int(int(exclude_zero)))
    return idx, d2


def exact_delta_f64(F, R, plan, exclude_zero=True):
    F = _fet(F)
    q0, nq, roff, rs, rn = _plan_args(plan)
    qb, nout = int(plan["q_base"]), int(plan["n_out"])
    nn = np.zeros(nout, np.int32)
    d2 = np.full(nout, np.inf)
    R64 = np.ascontiguousarray(R, dtype=np.float64)     # an FP64 rho keeps its own order
    lib().orc_exact_delta_f64(_ptr(nn), _ptr(d2), _ptr(F), _ptr(R64), C.c_int(F.shape[1]),
                              _ptr(q0), _ptr(nq), _ptr(roff), _ptr(rs), _ptr(rn),
                              C.c_int(len(q0)), C.c_int(qb), C.c_int(int(exclude_zero)))
    return nn, d2


def exact_knn_f32(F, plan, knn):
    """True top-knn in the reference FP32 arithmetic, (d2, index) order."""
    F = _fet(F)
    q0, nq, roff, rs, rn = _plan_args(plan)
    qb, nout = int(plan["q_base"]), int(plan["n_out"])
    idx = np.zeros((nout, knn), np.int32)
    d2 = np.zeros((nout, knn), np.float32)
    lib().orc_exact_knn_f32(_ptr(idx), _ptr(d2), _ptr(F), C.c_int(F.shape[1]), _ptr(q0), _ptr(nq),
                            _ptr(roff), _ptr(rs), _ptr(rn), C.c_int(len(q0)), C.c_int(qb),
                            C.c_int(knn))
    return idx, d2


def exact_delta_f32(F, R, plan):
    """Nearest unmasked (R[c] > R[q]) candidate in FP32 arithmetic."""
    F = _fet(F)
    q0, nq, roff, rs, rn = _plan_args(plan)
    qb, nout = int(plan["q_base"]), int(plan["n_out"])
    nn = np.zeros(nout, np.int32)
    d2 = np.zeros(nout, np.float32)
    lib().orc_exact_delta_f32(_ptr(nn), _ptr(d2), _ptr(F), _ptr(_f32(R)), C.c_int(F.shape[1]),
                              _ptr(q0), _ptr(nq), _ptr(roff), _ptr(rs), _ptr(rn),
                              C.c_int(len(q0)), C.c_int(qb))
    return nn, d2


def site_knn_cpu(F, plan, knn):
    F = _fet(F)
    q0, nq, roff, rs, rn = _plan_args(plan)
    qb, nout = int(plan["q_base"]), int(plan["n_out"])
    vr = np.zeros(nout, np.float32)
    mi = np.zeros((nout, knn), np.int32)
    lib().orc_site_knn_cpu(_ptr(vr), _ptr(mi), _ptr(F), C.c_int(F.shape[1]), _ptr(q0), _ptr(nq),
                           _ptr(roff), _ptr(rs), _ptr(rn), C.c_int(len(q0)), C.c_int(qb),
                           C.c_int(knn))
    return vr, mi


def site_delta_cpu(F, R, plan):
    F = _fet(F)
    q0, nq, roff, rs, rn = _plan_args(plan)
    qb, nout = int(plan["q_base"]), int(plan["n_out"])
    de = np.zeros(nout, np.float32)
    nn = np.zeros(nout, np.int32)
    lib().orc_site_delta_cpu(_ptr(de), _ptr(nn), _ptr(F), _ptr(_f32(R)), C.c_int(F.shape[1]),
                             _ptr(q0), _ptr(nq), _ptr(roff), _ptr(rs), _ptr(rn),
                             C.c_int(len(q0)), C.c_int(qb))
    return de, nn


def calc_dc2_drift(n1, viSite1, viSite2, F1, F2, n_sites, dc_subsample=1000, dc_percent=2.0):
    """calc_dc2_drift_ (matlab/irc.m:24582-24608) restated: (dc2, dc2_site).
    viSite1/viSite2: 1-based sites of the window's n12 spikes (own chunk's n1
    first); F1/F2: primary / secondary features [n12, nC]."""
    F1, F2 = _fet(F1), _fet(F2)
    s1, s2 = _i32(viSite1), _i32(viSite2)
    site = np.zeros(n_sites, np.float32)
    d = lib().orc_calc_dc2_drift(_ptr(site), int(n1), int(F1.shape[0]), int(F1.shape[1]), _ptr(s1), _ptr(s2),
                                 _ptr(F1), _ptr(F2), int(n_sites), int(dc_subsample), float(dc_percent))
    return np.float32(d), site


# --- clustering after the path ---------------------------------------------------------

def sort_rho(rho):
    """vrRho / max(vrRho) and sort(vrRho, 'descend') order (1-based int64)."""
    r = np.array(rho, dtype=np.float32, copy=True)
    order = np.empty(r.size, np.int64)
    lib().orc_sort_rho(_ptr(r), _ptr(order), C.c_int64(r.size))
    return r, order


def assign_cluster_knn(rho, delta, ordrho, nneigh, miKnn, delta_cut=1.0, min_count=0):
    """postCluster_'s cluster assignment.  miKnn: [nSpk, knn] (row s = MATLAB
    column s), any int64 ids.  Returns a dict with viClu (int32 labels, 0 =
    none), icl (1-based centre spike ids), vnSpk_clu, nClu, nClu_pre, nClu_post;
    raises ValueError where MATLAB would raise an index error."""
    rho, delta = _f32(rho), _f32(delta)
    ordrho = np.ascontiguousarray(ordrho, dtype=np.int64)
    nneigh = np.ascontiguousarray(nneigh, dtype=np.int64)
    mk = np.ascontiguousarray(miKnn, dtype=np.int64)
    n = rho.size
    knn = mk.shape[1]
    viClu = np.empty(n, np.int32)
    icl = np.empty(max(n, 1), np.int64)
    vn = np.empty(max(n, 1), np.int32)
    cnt = np.zeros(3, np.int64)
    rc = lib().orc_assign_cluster_knn(_ptr(viClu), _ptr(icl), _ptr(vn), _ptr(cnt), _ptr(rho), _ptr(delta),
                                      _ptr(ordrho), _ptr(nneigh), _ptr(mk), C.c_int(knn), C.c_int64(n),
                                      C.c_float(delta_cut), C.c_int(min_count))
    if rc != 0:
        raise ValueError("assign_cluster_knn: index out of range")
    k = int(cnt[0])
    return dict(viClu=viClu, icl=icl[:k].copy(), vnSpk_clu=vn[:k].copy(), nClu=k,
                nClu_pre=int(cnt[1]), nClu_post=int(cnt[2]))


# --- the reference kernels on a GPU --------------------------------------------------

class RefKernels:
    """The reference's CUDA kernels (compiled from its sources to PTX) launched
    with the MATLAB launch configuration.  Arguments are torch CUDA tensors.
    Feature tensors are [n, nC] (== MATLAB [nC x n]); 2-D outputs are
    returned as [nA, nT] (== MATLAB [nT x nA])."""

    def __init__(self):
        import torch
        self.torch = torch
        path = build_oracle.build_harness()
        self.h = C.CDLL(path)
        ptx_dir = build_oracle.REF_OUT
        for k in build_oracle.REF_KERNELS:
            if not os.path.exists(os.path.join(ptx_dir, k + ".ptx")):
                raise FileNotFoundError("reference PTX missing: %s" % k)
        torch.cuda.init()
        torch.empty(1, device="cuda")          # make the primary context current
        rc = self.h.refh_init(ptx_dir.encode())
        if rc != 0:
            raise RuntimeError("refh_init failed: cudaError %d" % rc)

    def _s(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr())

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference kernel launch failed: cudaError %d" % rc)

    def search_min_drift(self, F, IBB, NBB, vnConst, nT=1024):
        t = self.torch
        vn = t.tensor([int(v) for v in vnConst], dtype=t.int32, device=F.device)
        nA = int(vnConst[4])
        D = t.zeros((nA, nT), dtype=t.float32, device=F.device)
        I = t.zeros((nA, nT), dtype=t.int32, device=F.device)
        self._check(self.h.refh_search_min_drift(self._p(D), self._p(I), self._p(F), self._p(IBB),
                                                 self._p(NBB), self._p(vn), C.c_int(nT),
                                                 C.c_int(nA), self._s()))
        return D, I

    def search_delta_drift(self, F, R, IBB, NBB, vnConst, nT=512):
        t = self.torch
        vn = t.tensor([int(v) for v in vnConst], dtype=t.int32, device=F.device)
        nA = int(vnConst[4])
        D = t.zeros((nA, nT), dtype=t.float32, device=F.device)
        I = t.zeros((nA, nT), dtype=t.int32, device=F.device)
        self._check(self.h.refh_search_delta_drift(self._p(D), self._p(I), self._p(F), self._p(R),
                                                   self._p(IBB), self._p(NBB), self._p(vn),
                                                   C.c_int(nT), C.c_int(nA), self._s()))
        return D, I

    def cuda_knn_index(self, B, A, knn):
        t = self.torch
        nB, nA, nC = B.shape[0], A.shape[0], A.shape[1]
        vn = t.tensor([nB, nA, nC, knn], dtype=t.int32, device=A.device)
        K = t.zeros(nA, dtype=t.float32, device=A.device)
        I = t.zeros((nA, knn), dtype=t.int32, device=A.device)
        self._check(self.h.refh_cuda_knn_index(self._p(K), self._p(I), self._p(B), self._p(A),
                                               self._p(vn), C.c_int(nA), self._s()))
        return K, I

    def cuda_delta_knn(self, B, A, R_B, R_A):
        t = self.torch
        nB, nA, nC = B.shape[0], A.shape[0], A.shape[1]
        vn = t.tensor([nB, nA, nC], dtype=t.int32, device=A.device)
        D = t.zeros(nA, dtype=t.float32, device=A.device)
        N = t.zeros(nA, dtype=t.int32, device=A.device)
        self._check(self.h.refh_cuda_delta_knn(self._p(D), self._p(N), self._p(B), self._p(A),
                                               self._p(R_B), self._p(R_A), self._p(vn),
                                               C.c_int(nA), self._s()))
        return D, N

    def delta_drift(self, miSite12_colmajor, mrFet1, mrFet2, rho, n1, dc2):
        t = self.torch
        n12, nC = mrFet1.shape
        vn = t.tensor([n1, n12, nC], dtype=t.int32, device=mrFet1.device)
        de = t.zeros(n1, dtype=t.float32, device=mrFet1.device)
        nn = t.zeros(n1, dtype=t.int32, device=mrFet1.device)
        self._check(self.h.refh_delta_drift(self._p(de), self._p(nn), self._p(miSite12_colmajor), self._p(mrFet1),
                                            self._p(mrFet2), self._p(rho), self._p(vn), C.c_float(dc2),
                                            C.c_int(n1), self._s()))
        return de, nn

    def cuda_knn(self, B, A, knn):
        t = self.torch
        nA = A.shape[0]
        vn = t.tensor([B.shape[0], nA, A.shape[1], knn], dtype=t.int32, device=A.device)
        K = t.zeros(nA, dtype=t.float32, device=A.device)
        self._check(self.h.refh_cuda_knn(self._p(K), self._p(B), self._p(A), self._p(vn), C.c_int(nA), self._s()))
        return K

    def cuda_knn_full(self, B, A, knn):
        t = self.torch
        nA = A.shape[0]
        vn = t.tensor([B.shape[0], nA, A.shape[1], knn], dtype=t.int32, device=A.device)
        K = t.zeros((nA, knn), dtype=t.float32, device=A.device)
        I = t.zeros((nA, knn), dtype=t.int32, device=A.device)
        self._check(self.h.refh_cuda_knn_full(self._p(K), self._p(I), self._p(B), self._p(A), self._p(vn),
                                              C.c_int(nA), self._s()))
        return K, I

    def cuda_knn_ib(self, B, A, IB, knn):
        t = self.torch
        nA = A.shape[0]
        vn = t.tensor([IB.numel(), nA, A.shape[1], knn], dtype=t.int32, device=A.device)
        K = t.zeros(nA, dtype=t.float32, device=A.device)
        I = t.zeros((nA, knn), dtype=t.int32, device=A.device)
        self._check(self.h.refh_cuda_knn_ib(self._p(K), self._p(I), self._p(B), self._p(A), self._p(IB),
                                            self._p(vn), C.c_int(nA), self._s()))
        return K, I

    def cuda_rho(self, mrFet12, ord12, n1, dn_max, dc2, fDc_spk=0, nT=128):
        t = self.torch
        n12, nC = mrFet12.shape
        vn = t.tensor([n1, n12, nC, dn_max, fDc_spk], dtype=t.int32, device=mrFet12.device)
        rho = t.zeros(n1, dtype=t.float32, device=mrFet12.device)
        self._check(self.h.refh_cuda_rho(self._p(rho), self._p(mrFet12), self._p(ord12), self._p(vn),
                                         C.c_float(dc2), C.c_int(n1), C.c_int(nT), self._s()))
        return rho

    def cuda_delta(self, mrFet12, ord12, rr12, n1, dn_max, dc2, fDc_spk=0, nT=128):
        t = self.torch
        n12, nC = mrFet12.shape
        vn = t.tensor([n1, n12, nC, dn_max, fDc_spk], dtype=t.int32, device=mrFet12.device)
        de = t.zeros(n1, dtype=t.float32, device=mrFet12.device)
        nn = t.zeros(n1, dtype=t.int32, device=mrFet12.device)
        self._check(self.h.refh_cuda_delta(self._p(de), self._p(nn), self._p(mrFet12), self._p(ord12),
                                           self._p(rr12), self._p(vn), C.c_float(dc2), C.c_int(n1),
                                           C.c_int(nT), self._s()))
        return de, nn

    def rho_drift(self, miSite12_colmajor, mrFet1, mrFet2, n1, dc2):
        t = self.torch
        n12, nC = mrFet1.shape
        vn = t.tensor([n1, n12, nC], dtype=t.int32, device=mrFet1.device)
        rho = t.zeros(n1, dtype=t.float32, device=mrFet1.device)
        self._check(self.h.refh_rho_drift(self._p(rho), self._p(miSite12_colmajor), self._p(mrFet1),
                                          self._p(mrFet2), self._p(vn), C.c_float(dc2),
                                          C.c_int(n1), self._s()))
        return rho
