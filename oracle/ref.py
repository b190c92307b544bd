"""ctypes bindings to the reference's own CPU path, compiled from the
reference's headers into ``oracle/_ref/libiaref.so`` by ``oracle/build.py``.

ORACLE / TEST INFRASTRUCTURE ONLY.  Used to generate the golden fixtures under
tests/golden/ and, where the library exists, as a cross-check in the CPU test
suite.  The product path never imports this module.

Bound entry points (reference signatures):
  esm(int m, int l, double *r_ms, double *r_lh, cuDoubleComplex **m_e,
      cuDoubleComplex **h, double k, double r_i)                 CUDA/esm.cuh:112
  ibem(int m, int l, int n, double *r_ms, int *e_n, double *r_lh,
       cuDoubleComplex **m_e, cuDoubleComplex **h, double k, int n_ch,
       double *cp)                                              CUDA/ibem.cuh:424
  invr(..., cuDoubleComplex **q_e, double k, int n_ch, double *cp, int n_am)
                                                                 CUDA/invr.cuh:457
The reference reads IPF.txt / IPFs.txt from the current directory
(CUDA/ibem.cuh:434,450); ``ibem`` here writes the given rules to a temporary
directory in the reference's text format and runs there.
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libiaref.so")

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        _lib.esm.argtypes = [C.c_int, C.c_int, P, P, C.POINTER(P), C.POINTER(P), C.c_double, C.c_double]
        _lib.ibem.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, C.POINTER(P), C.POINTER(P), C.c_double, C.c_int, P]
        _lib.invr.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, C.POINTER(P), C.POINTER(P), C.POINTER(P),
                              C.c_double, C.c_int, P, C.c_int]
        _lib.ref_sphere.argtypes = [P, P, C.POINTER(P), C.POINTER(P), C.POINTER(P), C.c_double, C.c_double,
                                    C.c_double, C.c_int, C.c_int]
        _lib.ref_cart2sph.argtypes = [C.c_int, P, C.POINTER(P)]
        _lib.ref_geometry.argtypes = [C.c_char_p, C.c_double, C.c_double, C.POINTER(P), C.POINTER(P), C.POINTER(P),
                                      C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _lib.ref_free.argtypes = [P]
        _lib.ref_c_air.restype = C.c_double
        _lib.ref_rho_air.restype = C.c_double
    return _lib


def constants():
    L = lib()
    return L.ref_c_air(), L.ref_rho_air()


def _take(ptr: C.c_void_p, count: int, dtype=np.complex128) -> np.ndarray:
    itemsize = np.dtype(dtype).itemsize
    buf = (C.c_char * (count * itemsize)).from_address(ptr.value)
    out = np.frombuffer(buf, dtype=dtype).copy()
    lib().ref_free(ptr)
    return out


def _soa(P) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(P, dtype=np.float64)).ravel()


def esm(r_ms, r_lh, k, r_i):
    """Reference esm(): returns (Me m x m, He l x m) column-major as 2-D arrays."""
    r_ms, r_lh = _soa(r_ms), _soa(r_lh)
    m, l = r_ms.size // 3, r_lh.size // 3
    me, h = C.c_void_p(), C.c_void_p()
    lib().esm(m, l, r_ms.ctypes.data, r_lh.ctypes.data, C.byref(me), C.byref(h), float(k), float(r_i))
    Me = _take(me, m * m).reshape(m, m, order="F")
    He = _take(h, l * m).reshape(l, m, order="F")
    return Me, He


def write_rules(dirname, regular, singular):
    """Write quadrature rules in the reference's text format: a count line then
    'xi1 xi2 w' rows (IPF.txt); the singular file has one $PAGE per vertex
    (IPFs.txt, read at CUDA/ibem.cuh:450-475)."""
    regular = np.asarray(regular)
    singular = np.asarray(singular)
    with open(os.path.join(dirname, "IPF.txt"), "w") as f:
        f.write(f"{regular.shape[0]}\n")
        for row in regular:
            f.write("%.17g %.17g %.17g\n" % tuple(row))
    with open(os.path.join(dirname, "IPFs.txt"), "w") as f:
        f.write(f"{singular.shape[1]}\n")
        for pg in range(3):
            f.write(f"$PAGE {pg + 1}\n")
            for row in singular[pg]:
                f.write("%.17g %.17g %.17g\n" % tuple(row))


def ibem(nodes, elems, mics, k, regular, singular, chief=None):
    """Reference ibem(): returns (Z m x m, H l x m)."""
    r_ms, r_lh = _soa(nodes), _soa(mics)
    e_n = np.ascontiguousarray(np.asarray(elems, dtype=np.int32)).ravel()
    m, l, n = r_ms.size // 3, r_lh.size // 3, e_n.size // 3
    n_ch = 0 if chief is None else np.asarray(chief).shape[1]
    cp = _soa(chief) if n_ch else np.zeros(3)
    me, h = C.c_void_p(), C.c_void_p()
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        write_rules(d, regular, singular)
        os.chdir(d)
        try:
            lib().ibem(m, l, n, r_ms.ctypes.data, e_n.ctypes.data, r_lh.ctypes.data, C.byref(me), C.byref(h),
                       float(k), n_ch, cp.ctypes.data)
        finally:
            os.chdir(cwd)
    Z = _take(me, m * m).reshape(m, m, order="F")
    H = _take(h, l * m).reshape(l, m, order="F")
    return Z, H


def invr(nodes, elems, mics, k, regular, singular, n_am):
    """Reference invr() with n_ch = 0: returns (q_e m x n_am, the left singular
    vectors of G Z; h l x n_am; m_e m x n_am).  Its output products take n_am
    as the inner dimension (CUDA/invr.cuh:904,907), so only n_am = m gives
    H U and Z U."""
    r_ms, r_lh = _soa(nodes), _soa(mics)
    e_n = np.ascontiguousarray(np.asarray(elems, dtype=np.int32)).ravel()
    m, l, n = r_ms.size // 3, r_lh.size // 3, e_n.size // 3
    me, h, qe = C.c_void_p(), C.c_void_p(), C.c_void_p()
    cp = np.zeros(3)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        write_rules(d, regular, singular)
        os.chdir(d)
        try:
            lib().invr(m, l, n, r_ms.ctypes.data, e_n.ctypes.data, r_lh.ctypes.data, C.byref(me), C.byref(h),
                       C.byref(qe), float(k), 0, cp.ctypes.data, int(n_am))
        finally:
            os.chdir(cwd)
    Q = _take(qe, m * n_am).reshape(m, n_am, order="F")
    Hh = _take(h, l * n_am).reshape(l, n_am, order="F")
    Me = _take(me, m * n_am).reshape(m, n_am, order="F")
    return Q, Hh, Me


def sphere(nodes, mics, k, u, a):
    r_ms, r_lh = _soa(nodes), _soa(mics)
    m, l = r_ms.size // 3, r_lh.size // 3
    ps, ph, vs = C.c_void_p(), C.c_void_p(), C.c_void_p()
    lib().ref_sphere(r_ms.ctypes.data, r_lh.ctypes.data, C.byref(ps), C.byref(ph), C.byref(vs), float(k), float(u),
                     float(a), m, l)
    return _take(ps, m), _take(ph, l), _take(vs, m)


def cart2sph(P):
    r = _soa(P)
    m = r.size // 3
    out = C.c_void_p()
    lib().ref_cart2sph(m, r.ctypes.data, C.byref(out))
    return _take(out, 3 * m, np.float64).reshape(3, m)


def read_reference_rules(ref_cuda_dir):
    """Parse the reference's IPF.txt (regular) and IPFs.txt (singular, 3 pages)
    into arrays (nq, 3) and (3, nqs, 3) of (xi1, xi2, w)."""
    with open(os.path.join(ref_cuda_dir, "IPF.txt")) as f:
        lines = [s for s in f.read().split("\n") if s.strip()]
    nreg = int(lines[0])
    reg = np.array([[float(x) for x in s.split()] for s in lines[1:1 + nreg]])
    with open(os.path.join(ref_cuda_dir, "IPFs.txt")) as f:
        lines = [s for s in f.read().split("\n") if s.strip()]
    nsg = int(lines[0])
    pages, cur = [], []
    for s in lines[1:]:
        if s.startswith("$PAGE"):
            if cur:
                pages.append(cur)
            cur = []
            continue
        cur.append([float(x) for x in s.split()])
    pages.append(cur)
    sing = np.array(pages)
    assert sing.shape == (3, nsg, 3)
    return reg, sing


def geometry(path, k, t):
    """Reference geometry() (CUDA/utils.cuh:291): gmsh v2.2 nodes, triangles
    and field points r (1 + 2 pi t / k).  Returns (r_ms (3, m), r_lh (3, l),
    e_n (3, n))."""
    P = C.c_void_p
    rm, rl, en = P(), P(), P()
    m, l, n = C.c_int(), C.c_int(), C.c_int()
    lib().ref_geometry(str(path).encode(), float(k), float(t), C.byref(rm), C.byref(rl), C.byref(en), C.byref(m),
                       C.byref(l), C.byref(n))
    r_ms = _take(rm, 3 * m.value, np.float64).reshape(3, m.value)
    r_lh = _take(rl, 3 * l.value, np.float64).reshape(3, l.value)
    e_n = _take(en, 3 * n.value, np.int32).reshape(3, n.value)
    return r_ms, r_lh, e_n
