"""The bounded waits of the tensor-core filter: with a poll limit of two
(irc_set_wait_limit) every CTA's pipeline waits give up, the CTAs stop, let
their own copies and MMAs land, free TMEM and set the plan's error word, which
irc_plan_check reports as IRC_E_TIMEOUT.  The context stays usable: with the
default limit restored the same plan gives the same results as before.  Both
unit widths run (chunks of 600 queries: 256-wide units; chunks of 20: four-slot
items on 128-wide units)."""
import ctypes

import numpy as np
import pytest
import torch

from ironclust_gb300 import _lib, irc
from tests.cases import small_site

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [dict(n=3000, d=24, n_chunks=5, seed=7),
                                  dict(n=400, d=33, n_chunks=20, seed=9, sizes=[20] * 20)])
def test_bounded_waits_give_up_and_report_timeout(gpu, case):
    L = _lib.lib()
    F, plan, _ = small_site(**case)
    Fd = torch.from_numpy(F).to(gpu)
    P = irc.Plan(plan)
    want = irc.site_knn(P, Fd, 30, "bf16")
    assert L.irc_plan_check(P.h, irc._stream()) == _lib.IRC_OK
    _lib.check(L.irc_set_wait_limit(2), "irc_set_wait_limit")
    try:
        irc.site_knn(P, Fd, 30, "bf16")
        assert L.irc_plan_check(P.h, irc._stream()) == _lib.IRC_E_TIMEOUT
        assert b"timed out" in L.irc_last_error()
    finally:
        _lib.check(L.irc_set_wait_limit(0), "irc_set_wait_limit")
    got = irc.site_knn(P, Fd, 30, "bf16")
    assert L.irc_plan_check(P.h, irc._stream()) == _lib.IRC_OK
    for k in ("miKnn", "d2Knn", "rho"):
        assert np.array_equal(got[k].cpu().numpy(), want[k].cpu().numpy()), k
    P.close()
