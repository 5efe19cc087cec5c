"""Build recipe for the oracle (test infrastructure, not product code).

Three artefacts:

* ``oracle/_build/libirc_oracle.so`` -- the CPU restatement in
  ``irc_oracle.c`` and ``irc_oracle_cluster.c`` (gcc, OpenMP, ``-ffp-contract=off`` so that the only fused
  multiply-adds are the explicit ``fmaf`` calls that restate nvcc's
  contraction of the reference kernels).
* ``oracle/_build/libirc_refharness.so`` -- ``ref_harness.cu``, a host-only
  launcher for the reference kernels (built on any machine with nvcc).
* ``oracle/_ref/*.ptx`` -- the reference's own kernel sources compiled to PTX
  exactly as ``irc2 compile`` does (``nvcc -ptx -m 64 -arch <sm>``,
  matlab/irc2.m:7605), here for sm_103a.  Only built where the reference
  checkout is present; elsewhere the previously built files are used.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference's kernel sources (read-only); absent on machines that only run the prebuilt files
REFERENCE_MATLAB = os.environ.get("IRC_REFERENCE_MATLAB", "/root/reference/matlab")
REF_KERNELS = ["search_min_drift", "search_delta_drift", "cuda_knn_index",
               "cuda_delta_knn", "irc_cuda_rho_drift", "irc_cuda_delta_drift", "cuda_knn",
               "cuda_knn_full", "cuda_knn_ib", "irc_cuda_rho", "irc_cuda_delta"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle_lib(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "irc_oracle.c"), os.path.join(HERE, "irc_oracle_cluster.c")]
    out = os.path.join(BUILD, "libirc_oracle.so")
    if force or _stale(out, srcs):
        _run(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]
             + srcs + ["-o", out, "-lm"])
    return out


def build_harness(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_harness.cu")
    out = os.path.join(BUILD, "libirc_refharness.so")
    if force or _stale(out, [src]):
        _run([NVCC, "-O2", "-shared", "-Xcompiler", "-fPIC", src, "-o", out])
    return out


def build_ref_ptx(force=False):
    """Compile the reference kernels to PTX (only where the sources exist)."""
    if not os.path.isdir(REFERENCE_MATLAB):
        return [os.path.join(REF_OUT, k + ".ptx") for k in REF_KERNELS]
    os.makedirs(REF_OUT, exist_ok=True)
    jobs = []
    for k in REF_KERNELS:
        src = os.path.join(REFERENCE_MATLAB, k + ".cu")
        out = os.path.join(REF_OUT, k + ".ptx")
        if force or _stale(out, [src]):
            jobs.append([NVCC, "-ptx", "-m64", "-arch=sm_103a", src, "-o", out])
    with ThreadPoolExecutor(max_workers=6) as ex:
        list(ex.map(_run, jobs))
    return [os.path.join(REF_OUT, k + ".ptx") for k in REF_KERNELS]


def build_all(force=False):
    with ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_oracle_lib, force), ex.submit(build_harness, force),
                ex.submit(build_ref_ptx, force)]
        return [f.result() for f in futs]


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
