"""Host-side checks of irc_site_knn_exact_noalloc (no GPU needed: every
rejection below happens before the entry point touches the device)."""
import ctypes as C

import numpy as np

from ironclust_gb300 import _lib
from tests.noalloc_plans import LIMIT_WORDS, boundary_plan, plan_words


def _call(plan, knn=30, nC=8):
    arrs = [np.ascontiguousarray(plan[k], dtype=np.int32) for k in ("q0", "nq", "roff", "rs", "rn")]
    fake = C.c_void_p(16)                  # never dereferenced: validation fails or the device is absent
    return _lib.lib().irc_site_knn_exact_noalloc(
        fake, nC, *[a.ctypes.data_as(C.c_void_p) for a in arrs], len(arrs[0]), int(plan["q_base"]),
        int(plan["n_out"]), int(plan["n_f"]), knn, fake, fake, fake, fake, None)


def test_plan_two_words_over_the_array_is_rejected():
    plan = boundary_plan(extra=2)
    assert plan_words(plan) == LIMIT_WORDS + 2
    assert _call(plan) == _lib.IRC_E_INVAL
    assert b"scratch words" in _lib.lib().irc_last_error()


def test_plan_filling_the_array_exactly_passes_the_size_check():
    plan = boundary_plan(extra=1)
    assert plan_words(plan) == LIMIT_WORDS
    rc = _call(plan)
    # without a GPU the call then fails at the device lookup, never at the size check
    assert rc != _lib.IRC_E_INVAL or b"scratch words" not in _lib.lib().irc_last_error()


def test_plans_irc_plan_create_rejects_are_rejected():
    base = dict(q0=np.array([0], np.int32), nq=np.array([16], np.int32), roff=np.array([0, 1], np.int32),
                rs=np.array([0], np.int32), rn=np.array([16], np.int32), q_base=0, n_out=16, n_f=16)
    bad = [dict(base, q0=np.array([-16], np.int32), q_base=-16),          # negative query rows
           dict(base, q0=np.array([2**31 - 8], np.int32), n_f=2**31 - 1),  # q0 + nq overflows int32
           dict(base, rs=np.array([8], np.int32))]                         # run past nF
    for plan in bad:
        assert _call(plan) == _lib.IRC_E_INVAL, plan
    # a roff that is not strictly increasing up to its last entry
    plan = dict(base, q0=np.array([0, 0], np.int32), nq=np.array([8, 8], np.int32),
                roff=np.array([0, 3, 1], np.int32))
    assert _call(plan) == _lib.IRC_E_INVAL
