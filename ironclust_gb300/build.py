"""In-tree build of libircgb300.so (nvcc, sm_103a only).

Every translation unit under csrc/ is compiled in parallel to an object in
``ironclust_gb300/_build/`` and linked into ``ironclust_gb300/libircgb300.so``
(C ABI declared in include/ircgb300.h).  The CUDA runtime is linked
statically, so the library loads on machines without a GPU driver (the
first CUDA call then reports the missing device).
"""
from __future__ import annotations

import glob
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libircgb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def build(force=False, verbose=False, extra=()):
    """Compile (if stale) and return the path of libircgb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    hdr_time = max(os.path.getmtime(h) for h in headers())
    objs, jobs = [], []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append([NVCC, "-c", src, "-o", obj] + ARCH + FLAGS + list(extra))
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if jobs or force or not os.path.exists(LIB):
        logs.append(_run([NVCC, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC"]))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "-v" in sys.argv else []))
