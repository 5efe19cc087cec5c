"""irc_site_knn_exact_noalloc: the EXACT site kNN for callers that cannot call
cudaMalloc (hosts whose device memory is reserved by their own pool, loops
that must not trigger cudaMalloc's device-wide synchronisation).

The entry point keeps its plan copy and queues in a fixed array inside the
library instead of allocating; its outputs must equal those of the regular
entry point (irc_plan_create + irc_site_knn in IRC_MODE_EXACT) bit for bit,
call after call, since every call reuses that array: each plan is run twice
in a row, and again after another plan has overwritten the array, and one
plan fills the array to its last word.  The file is named so that pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from ironclust_gb300 import _lib, irc
from tests.cases import small_site
from tests.noalloc_plans import LIMIT_WORDS, boundary_plan, plan_words

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


def regular(F, plan, knn):
    """The regular EXACT entry point, outputs pre-filled like call_noalloc's
    (rows no chunk covers keep the fill in both)."""
    n = int(plan["n_out"])
    P = irc.Plan(plan)
    got = irc.site_knn(P, F, knn=knn, mode="exact")
    torch.cuda.synchronize()
    edge = np.zeros(n + 1, np.int64)
    start = np.asarray(plan["q0"], np.int64) - int(plan["q_base"])
    np.add.at(edge, start, 1)
    np.add.at(edge, start + np.asarray(plan["nq"], np.int64), -1)
    covered = torch.from_numpy(np.cumsum(edge[:n]) > 0).to(F.device)
    P.close()
    fill = dict(vrKnn=-1.0, rho=-1.0, miKnn=-1, d2Knn=-1.0)
    return {k: torch.where(covered.view(-1, *([1] * (v.dim() - 1))), v, torch.full_like(v, fill[k]))
            for k, v in got.items() if v is not None}


def same_bits(a, b):
    a, b = a.cpu().numpy(), b.cpu().numpy()
    if a.dtype == np.float32:
        a, b = a.view(np.int32), b.view(np.int32)
    return np.array_equal(a, b)


def check_equal(got, want, what):
    torch.cuda.synchronize()
    for k in ("vrKnn", "rho", "miKnn", "d2Knn"):
        assert same_bits(got[k], want[k]), (what, k)


def test_noalloc_equals_regular_entry_point_twice_in_a_row(gpu):
    knn = 30
    cases = []
    for case in (dict(n=3000, d=24, n_chunks=5, seed=7),
                 dict(n=2500, d=33, n_chunks=4, seed=8, secondary=True)):
        F, plan, _ = small_site(**case)
        Fd = torch.from_numpy(F).to(gpu)
        cases.append((case, Fd, plan, regular(Fd, plan, knn)))
    for case, Fd, plan, want in cases:
        check_equal(call_noalloc(Fd, plan, knn), want, (case, "first call"))
        check_equal(call_noalloc(Fd, plan, knn), want, (case, "second call in a row"))
    # the first plan again, after the second one overwrote the array
    case, Fd, plan, want = cases[0]
    check_equal(call_noalloc(Fd, plan, knn), want, (case, "after another plan"))


def test_noalloc_plan_filling_the_array_exactly(gpu):
    plan = boundary_plan(extra=1)
    assert plan_words(plan) == LIMIT_WORDS
    rng = np.random.default_rng(11)
    Fd = torch.from_numpy(rng.normal(0, 1, (int(plan["n_f"]), 8)).astype(np.float32)).to(gpu)
    want = regular(Fd, plan, 30)
    check_equal(call_noalloc(Fd, plan, 30), want, "limit, first call")
    check_equal(call_noalloc(Fd, plan, 30), want, "limit, second call")


def test_noalloc_rejects_plans_beyond_the_fixed_array(gpu):
    plan = boundary_plan(extra=2)                 # two words over the array
    dummy = torch.zeros(16, device=gpu)
    p = C.c_void_p(dummy.data_ptr())
    arrs = [_host(plan[k]) for k in ("q0", "nq", "roff", "rs", "rn")]
    rc = _lib.lib().irc_site_knn_exact_noalloc(
        p, 8, *[a.ctypes.data_as(C.c_void_p) for a in arrs], len(arrs[0]), 0, int(plan["n_out"]),
        int(plan["n_f"]), 30, p, p, p, p, None)
    assert rc == _lib.IRC_E_INVAL
    assert b"scratch words" in _lib.lib().irc_last_error()
