"""Build ``libmpsgb300.so`` in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel into ``mps_gb300/_build/`` and linked into
``mps_gb300/libmpsgb300.so``.  Used by ``__graft_entry__.build()`` and by the package on first
import when the library is missing.  Run ``python -m mps_gb300.build`` to rebuild by hand.

``build(checked=True)`` (``python -m mps_gb300.build --checked``) makes the device-checked debug
library ``libmpsgb300_checked.so`` instead (objects in ``_build_checked/``, compiled with
``MPSG_DEVICE_CHECKS``); ``MPSG_LIBRARY=checked`` makes the package load it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmpsgb300.so")

SOURCES = ["planner.cpp", "ops.cu", "capi.cu", "kernels_copy.cu", "kernels_f64.cu", "linalg.cu",
           "krylov.cu", "kernels_split.cu", "noalloc.cu", "batch.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr", "-I", CSRC]
LIBS = ["-lcudart", "-lcusolver", "-lcublas"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mps_gb300")


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> str:
    build_dir = BUILD + "_checked" if checked else BUILD
    lib = LIB.replace(".so", "_checked.so") if checked else LIB
    flags = CFLAGS + (["-DMPSG_DEVICE_CHECKS"] if checked else [])
    os.makedirs(build_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "mpsgb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append([cc, *ARCH, *flags, "-c", path, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg, flush=True)
    if force or jobs or not os.path.exists(lib):
        tmp = lib + ".tmp"
        run([cc, *ARCH, "-shared", "-o", tmp, *objs, *LIBS])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, checked="--checked" in sys.argv))
