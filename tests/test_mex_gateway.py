"""The MATLAB gateway (mex/ircgb300_mex.c) type-checks against the C ABI
(include/ircgb300.h) with declaration-only stand-ins for MATLAB's headers
(tests/mexstub): every library call it makes exists with those argument
types.  MATLAB itself is absent, so the gateway cannot run here."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not found")
def test_mex_gateway_type_checks_against_the_header():
    cmd = ["gcc", "-fsyntax-only", "-std=c11", "-DMATLAB_MEX_FILE", "-I", os.path.join(ROOT, "tests", "mexstub"),
           "-I", os.path.join(ROOT, "include"), "-Wall", "-Werror", os.path.join(ROOT, "mex", "ircgb300_mex.c")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
