"""Loader of libircgb300.so (the C ABI in include/ircgb300.h).

The library is the only compute path: if it is missing or cannot be loaded
this module raises, there is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libircgb300.so")

IRC_OK = 0
IRC_E_INVAL = -1
IRC_E_NC = -2
IRC_E_CUDA = -3
IRC_E_NOMEM = -4
IRC_E_TIMEOUT = -5
IRC_E_UNSUPPORTED = -6

MODE_REF, MODE_EXACT, MODE_BF16, MODE_FP8 = 0, 1, 2, 3
CLUSTER_MAX_PEAKS = 131072          # IRC_CLUSTER_MAX_PEAKS
MODES = {"ref": MODE_REF, "exact": MODE_EXACT, "bf16": MODE_BF16, "fp8": MODE_FP8}

_P, _I, _F, _L = C.c_void_p, C.c_int, C.c_float, C.c_int64

# name -> argtypes (every entry returns int)
SIGNATURES = {
    "irc_version": [],
    "irc_last_error": [],
    "irc_status_string": [_I],
    "irc_search_min_drift": [_P, _P, _P, _P, _P, _P, _I, _I, _I, _P],
    "irc_search_delta_drift": [_P, _P, _P, _P, _P, _P, _P, _I, _P],
    "irc_cuda_knn_index": [_P, _P, _P, _P, _P, _I, _P],
    "irc_cuda_delta_knn": [_P, _P, _P, _P, _P, _P, _P, _I, _P],
    "irc_rho_drift": [_P, _P, _P, _P, _P, _F, _P],
    "irc_delta_drift": [_P, _P, _P, _P, _P, _P, _P, _F, _P],
    "irc_calc_dc2_drift": [_P, _P, _I, _I, _I, _P, _P, _P, _P, _I, _I, C.c_double, _P],
    "irc_plan_create": [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I],
    "irc_plan_destroy": [_P],
    "irc_plan_check": [_P, _P],
    "irc_plan_tc_layout": [_P, _I, _I],
    "irc_plan_tc_units": [_P, _I],
    "irc_plan_set_site_dims": [_P, _I, _P, _P],
    "irc_plan_tc_bytes": [_P, _I],
    "irc_plan_set_tc_buffer": [_P, _P, C.c_size_t],
    "irc_knn_rho_delta_site": [_P, _P, _I, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P],
    "irc_batch_plan_create": [_P, _I, _P, _P, _P, _P, _P, _P, _P],
    "irc_batch_stack": [_P, _I, _P, _P, _P, _I, _P],
    "irc_profile_begin": [_I],
    "irc_set_wait_limit": [_I],
    "irc_profile_end": [_P, _P, _P],
    "irc_site_knn": [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _P],
    "irc_site_delta": [_P, _P, _I, _P, _I, _I, _I, _P, _P, _P, _P, _P],
    "irc_site_knn_exact_noalloc": [_P, _I, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P],
    "irc_cuda_knn": [_P, _P, _P, _P, _I, _P],
    "irc_cuda_knn_full": [_P, _P, _P, _P, _P, _I, _P],
    "irc_cuda_knn_ib": [_P, _P, _P, _P, _P, _I, _P, _I, _P],
    "irc_cuda_rho": [_P, _P, _P, _P, _F, _P],
    "irc_cuda_delta": [_P, _P, _P, _P, _P, _P, _F, _I, _P],
    "irc_calc_drift": [_P, _P, _P, _P, _P, _L, _I, _I, _I, _I, _I, _P],
    "irc_fet_load_site": [_P, _P, _P, _I, _P, _P, _I, _I, _P, _P, _L, _P],
    "irc_knn_save_site": [C.c_char_p, _I, _P, _I, _I, _L, _P, _L, _P],
    "irc_sort_save": [C.c_char_p, _P, _P, _P, _P, _L, _P],
    "irc_f16_to_f32": [_P, _P, _L, _P],
    "irc_sort_load": [C.c_char_p, _P, _P, _P, _P, _L, _P],
    "irc_sort_rho": [_P, _P, _L, _P],
    "irc_assign_cluster_knn": [_P, _P, _P, _L, _P, _P, _P, _P, _P, _P, _I, _L, _F, _I, _P],
}

_lib = None


class IrcError(RuntimeError):
    def __init__(self, status, where, msg):
        super().__init__("%s failed (%d): %s" % (where, status, msg))
        self.status = status


def lib():
    """Load (building first if absent) and return the ctypes library."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build
            build.build()
        if not os.path.exists(LIB_PATH):
            raise ImportError("libircgb300.so is missing: run ironclust_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, argt in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = argt
            f.restype = (C.c_char_p if name in ("irc_last_error", "irc_status_string") else
                         C.c_size_t if name == "irc_plan_tc_bytes" else C.c_int)
        _lib = L
    return _lib


def check(status, where):
    if status != IRC_OK:
        raise IrcError(status, where, lib().irc_last_error().decode(errors="replace"))
    return status
