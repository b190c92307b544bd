"""Triangle quadrature rules for the IBEM assembly.

A rule is an (nq, 3) array of barycentric (xi1, xi2, w) rows with the weights
summing to 1/2 (the area of the reference triangle), the convention of the
reference's IPF.txt / IPFs.txt (CUDA/ibem.cuh:276-311).  A singular rule is
(3, nqs, 3): page p is for a collocation point at vertex p of the element
(shape function p equals 1 there).

``radon7`` and ``duffy`` are the rules libia.so builds in when no rule is
given (the same formulas, evaluated in C++); ``read_ipf`` / ``write_ipf``
read and write the reference's text format so its own tables can be used.
"""
from __future__ import annotations

import math

import numpy as np


def radon7() -> np.ndarray:
    """Radon's 7-point rule, exact for degree 5 (Radon 1948; Dunavant 1985)."""
    s15 = math.sqrt(15.0)
    a1, b1, w1 = (6 - s15) / 21, (9 + 2 * s15) / 21, (155 - s15) / 1200
    a2, b2, w2 = (6 + s15) / 21, (9 - 2 * s15) / 21, (155 + s15) / 1200
    pts = [(1 / 3, 1 / 3, 9 / 40), (a1, a1, w1), (b1, a1, w1), (a1, b1, w1), (a2, a2, w2), (b2, a2, w2),
           (a2, b2, w2)]
    r = np.array(pts, dtype=np.float64)
    r[:, 2] *= 0.5
    return r


def gauss_legendre01(n: int):
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def duffy(nu: int = 4, nv: int = 4) -> np.ndarray:
    """Duffy (1982) collapsed-square rule for a 1/r singularity at a vertex:
    N_p = 1 - u, N_{p+1} = u (1 - v), N_{p+2} = u v, weight w_u w_v u, with
    Gauss-Legendre points in u and v.  Returns (3, nu*nv, 3)."""
    xu, wu = gauss_legendre01(nu)
    xv, wv = gauss_legendre01(nv)
    out = np.zeros((3, nu * nv, 3))
    for p in range(3):
        q = 0
        for a in range(nu):
            for b in range(nv):
                u, v = xu[a], xv[b]
                N = [0.0, 0.0, 0.0]
                N[p] = 1.0 - u
                N[(p + 1) % 3] = u * (1.0 - v)
                N[(p + 2) % 3] = u * v
                out[p, q] = (N[0], N[1], wu[a] * wv[b] * u)
                q += 1
    return out


def builtin():
    """The rules libia.so uses when none is passed: (radon7, duffy(4, 4))."""
    return radon7(), duffy(4, 4)


def read_ipf(regular_path: str, singular_path: str):
    """Read rules in the reference's text format: first line the point count,
    then 'xi1 xi2 w' rows; the singular file has '$PAGE 1..3' separators."""
    with open(regular_path) as f:
        lines = [s for s in f.read().split("\n") if s.strip()]
    n = int(lines[0])
    reg = np.array([[float(x) for x in s.split()] for s in lines[1:1 + n]])
    with open(singular_path) as f:
        lines = [s for s in f.read().split("\n") if s.strip()]
    ns = int(lines[0])
    pages, cur = [], None
    for s in lines[1:]:
        if s.startswith("$PAGE"):
            if cur is not None:
                pages.append(cur)
            cur = []
            continue
        cur.append([float(x) for x in s.split()])
    pages.append(cur)
    sing = np.array(pages)
    if reg.shape != (n, 3) or sing.shape != (3, ns, 3):
        raise ValueError("malformed rule files")
    return reg, sing


def write_ipf(regular_path: str, singular_path: str, regular, singular):
    with open(regular_path, "w") as f:
        f.write(f"{len(regular)}\n")
        for row in regular:
            f.write("%.17g %.17g %.17g\n" % tuple(row))
    with open(singular_path, "w") as f:
        f.write(f"{singular.shape[1]}\n")
        for p in range(3):
            f.write(f"$PAGE {p + 1}\n")
            for row in singular[p]:
                f.write("%.17g %.17g %.17g\n" % tuple(row))
