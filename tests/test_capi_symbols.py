"""The C ABI library loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

from ironclust_gb300 import _lib, build

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ircgb300.h")


def declared_symbols():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(irc_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_entry_points():
    syms = declared_symbols()
    for s in ("irc_search_min_drift", "irc_search_delta_drift", "irc_cuda_knn_index",
              "irc_cuda_delta_knn", "irc_rho_drift", "irc_site_knn", "irc_site_delta"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_signature_table_matches_header():
    assert set(_lib.SIGNATURES) == set(declared_symbols())


def test_status_strings_without_gpu():
    L = _lib.lib()
    assert L.irc_version() >= 10000
    assert L.irc_status_string(_lib.IRC_E_NC) == b"feature count above the kernel maximum"


def test_argument_validation_needs_no_gpu():
    L = _lib.lib()
    vn = (ctypes.c_int32 * 5)(64 + 1, 10, 1, 0, 10)      # nC above the maximum
    rc = L.irc_search_min_drift(ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1),
                                ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.cast(vn, ctypes.c_void_p),
                                1024, 0, 30, None)
    assert rc == _lib.IRC_E_NC
    assert b"nC" in L.irc_last_error()
    rc = L.irc_search_min_drift(None, None, None, None, None, None, 1024, 0, 30, None)
    assert rc == _lib.IRC_E_INVAL
