"""Compile libia.so (all CUDA sources in csrc/) for sm_103a, in-tree.

Each translation unit compiles in parallel to an object file under
``inverseacoustics_gb300/_build/``; the objects link into
``inverseacoustics_gb300/libia.so`` (static CUDA runtime, C ABI only).
``build(debug_bounds=True)`` makes the bounds-checked debug library
``libia_debug.so`` (IA_DEBUG_BOUNDS; objects under ``_build_debug/``).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libia.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                  glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(out, ins):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in ins)


def build(verbose: bool = False, force: bool = False, extra_flags=None, debug_bounds: bool = False) -> str:
    bdir = BUILD + "_debug" if debug_bounds else BUILD
    lib = os.path.join(HERE, "libia_debug.so") if debug_bounds else LIB
    os.makedirs(bdir, exist_ok=True)
    nvcc = _nvcc()
    deps = _deps()
    flags = NVCC_FLAGS + list(extra_flags or []) + (["-DIA_DEBUG_BOUNDS"] if debug_bounds else [])
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(bdir, os.path.basename(src).replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + deps):
            jobs.append([nvcc, *ARCH, *flags, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, fu in zip(jobs, futs):
                r = fu.result()
                if verbose or r.returncode != 0:
                    print(" ".join(j))
                    print(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed for {j[-3]}")
    if force or jobs or _stale(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", lib, *objs, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"link of {os.path.basename(lib)} failed")
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
