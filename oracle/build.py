"""Build recipe for the oracle's compiled parts.

ORACLE / TEST INFRASTRUCTURE ONLY.

  build_oracle()  gcc: oracle/ibem_oracle.c -> oracle/_build/libiaoracle.so
                  (the C restatement; built here and on the GPU host)
  build_ref()     nvcc: the reference's own CPU path, compiled from its
                  headers where they lie (<reference>/CUDA) through
                  oracle/ref_entry.cu + oracle/lapack_shim.c, linked against
                  scipy's bundled OpenBLAS -> oracle/_ref/libiaref.so.
                  Only where the reference tree is present.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# Where the reference's CUDA/ headers lie.  This recipe compiles them in
# place, so it is the one file that names the read-only mount of the
# reference tree; IA_REFERENCE_CUDA or build_ref(reference_cuda_dir=...) point it
# elsewhere, and build_ref returns None (nothing built) where none exists.
_REFERENCE_MOUNT = "/root/reference/CUDA"


def reference_cuda(explicit: str | None = None) -> str | None:
    """The reference's CUDA/ directory: the argument, else IA_REFERENCE_CUDA,
    else the mount; None when that directory does not exist."""
    d = explicit or os.environ.get("IA_REFERENCE_CUDA") or _REFERENCE_MOUNT
    return d if os.path.isdir(d) else None


def build_oracle(verbose=False) -> str:
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libiaoracle.so")
    src = os.path.join(HERE, "ibem_oracle.c")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-o", out, src, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def _openblas():
    import scipy
    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cand = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so")))
    return libs, (os.path.basename(cand[0]) if cand else None)


def build_ref(verbose=False, reference_cuda_dir: str | None = None) -> str | None:
    ref_dir = reference_cuda(reference_cuda_dir)
    if ref_dir is None:
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libiaref.so")
    srcs = [os.path.join(HERE, "ref_entry.cu"), os.path.join(HERE, "lapack_shim.c")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    libdir, blas = _openblas()
    if blas is None:
        return None
    cmd = ["nvcc", "-std=c++17", "-arch=sm_100", "-rdc=true", "-O2", "-Xcompiler", "-fPIC", "-shared",
           "-diag-suppress", "1650", "-DC_AIR=343.0", "-DRHO_AIR=1.21", f"-I{ref_dir}", *srcs,
           "-o", out, f"-L{libdir}", f"-l:{blas}", f"-Xlinker", f"-rpath={libdir}", "-lcublas", "-lcusolver",
           "-lcudadevrt"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref(verbose=True))
    sys.exit(0)
