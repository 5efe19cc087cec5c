"""irc_site_knn_exact_noalloc: the EXACT site kNN for callers that cannot call
cudaMalloc (hosts whose device memory is reserved by their own pool, loops
that must not trigger cudaMalloc's device-wide synchronisation).

The entry point keeps its plan copy and queues in a fixed array inside the
library instead of allocating; its outputs must equal those of the regular
entry point (irc_plan_create + irc_site_knn in IRC_MODE_EXACT) bit for bit,
call after call, since every call reuses that array.  The file is named so
that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from ironclust_gb300 import _lib, irc
from tests.cases import small_site

pytestmark = pytest.mark.gpu


def _host(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def call_noalloc(F, plan, knn):
    n = int(plan["n_out"])
    dev = F.device
    out = dict(vrKnn=torch.full((n,), -1.0, device=dev), rho=torch.full((n,), -1.0, device=dev),
               miKnn=torch.full((n, knn), -1, dtype=torch.int32, device=dev),
               d2Knn=torch.full((n, knn), -1.0, device=dev))
    arrs = [_host(plan[k]) for k in ("q0", "nq", "roff", "rs", "rn")]
    ptr = lambda t: C.c_void_p(t.data_ptr())
    rc = _lib.lib().irc_site_knn_exact_noalloc(
        ptr(F), F.shape[1], *[a.ctypes.data_as(C.c_void_p) for a in arrs], len(arrs[0]),
        int(plan["q_base"]), n, int(plan["n_f"]), knn, ptr(out["vrKnn"]), ptr(out["rho"]),
        ptr(out["miKnn"]), ptr(out["d2Knn"]), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "irc_site_knn_exact_noalloc")
    return out


def same_bits(a, b):
    a, b = a.cpu().numpy(), b.cpu().numpy()
    if a.dtype == np.float32:
        a, b = a.view(np.int32), b.view(np.int32)
    return np.array_equal(a, b)


def test_noalloc_equals_regular_entry_point_twice_in_a_row(gpu):
    knn = 30
    for case in (dict(n=3000, d=24, n_chunks=5, seed=7),
                 dict(n=2500, d=33, n_chunks=4, seed=8, secondary=True)):
        F, plan, _ = small_site(**case)
        Fd = torch.from_numpy(F).to(gpu)
        P = irc.Plan(plan)
        want = irc.site_knn(P, Fd, knn=knn, mode="exact")
        got = call_noalloc(Fd, plan, knn)
        torch.cuda.synchronize()
        for k in ("vrKnn", "rho", "miKnn", "d2Knn"):
            assert same_bits(got[k], want[k]), (case, k)
        P.close()


def test_noalloc_rejects_plans_beyond_the_fixed_array(gpu):
    n_out = 3 << 20                      # more queries than the fixed array can queue
    q0 = _host([0]); nq = _host([16]); roff = _host([0, 1]); rs = _host([0]); rn = _host([16])
    dummy = torch.zeros(16, device=gpu)
    p = C.c_void_p(dummy.data_ptr())
    rc = _lib.lib().irc_site_knn_exact_noalloc(
        p, 1, q0.ctypes.data_as(C.c_void_p), nq.ctypes.data_as(C.c_void_p), roff.ctypes.data_as(C.c_void_p),
        rs.ctypes.data_as(C.c_void_p), rn.ctypes.data_as(C.c_void_p), 1, 0, n_out, n_out, 30, p, p, p, p, None)
    assert rc == _lib.IRC_E_INVAL
    assert b"scratch words" in _lib.lib().irc_last_error()
