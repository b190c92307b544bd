"""The drop-in headers (include/compat/): a program written against the
reference's call surface compiles against libia.so (CPU suite) and, on the
GPU, gives the oracle's results (GPU suite)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, relerr
from inverseacoustics_gb300 import geometry as g
from inverseacoustics_gb300 import quadrature as Q
from oracle import ia_oracle as O

SRC = os.path.join(ROOT, "tests", "compat", "compat_user.cu")
LIBDIR = os.path.join(ROOT, "inverseacoustics_gb300")


def _build(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "compat_user")
    cmd = [nvcc, "-std=c++17", "-O2", f"-I{ROOT}/include/compat", f"-I{ROOT}/include", SRC, "-o", exe,
           f"-L{LIBDIR}", "-lia", "-Xlinker", f"-rpath={LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_compat_program_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
    assert os.path.exists(exe)


def _write_ipf(d, reg, sing, truncate_reg=False, bad_count=False, pages=3):
    nq = reg.shape[0]
    lines = [str(nq + 1 if bad_count else nq)] + [f"{a!r} {b!r} {w!r}" for a, b, w in reg]
    if truncate_reg:
        lines = lines[:-2]
    (d / "IPF.txt").write_text("\n".join(lines) + "\n")
    nqs = sing.shape[1]
    out = [str(nqs)]
    for p in range(pages):
        out.append(f"$PAGE {p + 1}")
        out += [f"{a!r} {b!r} {w!r}" for a, b, w in sing[p]]
    (d / "IPFs.txt").write_text("\n".join(out) + "\n")


def test_compat_quadrature_files(tmp_path):
    """Like the reference, the drop-in ibem()/invr() read IPF.txt and IPFs.txt
    from the current directory; with neither present the built-in rules are
    used; a file that is present but does not parse (partner file missing,
    truncated table, wrong count, a missing page) makes the call throw rather
    than fall back to rules the caller did not ask for (the reference exits on
    a missing file, CUDA/ibem.cuh:270-273, and reads past a short one)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "compat_ipf")
    src = os.path.join(ROOT, "tests", "compat", "compat_ipf.cu")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", f"-I{ROOT}/include/compat", f"-I{ROOT}/include", src, "-o", exe,
                        f"-L{LIBDIR}", "-lia", "-Xlinker", f"-rpath={LIBDIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    reg, sing = Q.builtin()      # (nq, 3) and (3 pages, nqs, 3) rows of xi1, xi2, w

    def run(setup):
        d = tmp_path / setup
        d.mkdir()
        if setup == "valid":
            _write_ipf(d, reg, sing)
        elif setup == "only_regular":
            _write_ipf(d, reg, sing)
            (d / "IPFs.txt").unlink()
        elif setup == "truncated":
            _write_ipf(d, reg, sing, truncate_reg=True)
        elif setup == "bad_count":
            _write_ipf(d, reg, sing, bad_count=True)
        elif setup == "missing_page":
            _write_ipf(d, reg, sing, pages=2)
        out = subprocess.run([exe], capture_output=True, text=True, cwd=d)
        assert out.returncode == 0, out.stderr
        return out.stdout.strip()

    assert run("none") == "builtin"
    assert run("valid") == f"rules {reg.shape[0]} {sing.shape[1]}"
    for bad in ("only_regular", "truncated", "bad_count", "missing_page"):
        assert run(bad).startswith("error ibem: IPF.txt / IPFs.txt present but malformed"), bad


@pytest.mark.gpu
def test_compat_program_matches_oracle(tmp_path, cuda):
    exe = _build(tmp_path)
    nodes, elems = g.icosphere(1, 0.1)
    mics = g.hemisphere_array(np.random.default_rng(2), 42, 0.3)   # l == m keeps the reference esm valid too
    m, l, n = nodes.shape[1], mics.shape[1], elems.shape[1]
    k, r_i = 2 * np.pi * 900 / 343.5, 0.7
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([m, l, n], np.int32).tofile(f)
        np.array([k, r_i]).tofile(f)
        nodes.ravel().tofile(f)
        mics.ravel().tofile(f)
        elems.astype(np.int32).ravel().tofile(f)
    r = subprocess.run([exe, str(fin), str(fout)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    with open(fout, "rb") as f:
        raw = f.read()
    c, rho = 343.5, 1.19                 # the headers keep the reference's default constants
    off = 0

    def take(count, dtype=np.complex128):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    Me = take(m * m).reshape(m, m, order="F")
    He = take(l * m).reshape(l, m, order="F")
    Mo, Ho = O.esm(nodes, mics, k, r_i, c, rho)
    assert relerr(Me, Mo) < 1e-10 and relerr(He, Ho) < 1e-10
    Z = take(m * m).reshape(m, m, order="F")
    H = take(l * m).reshape(l, m, order="F")
    reg, sing = Q.builtin()           # no IPF.txt in the working directory -> built-in rules
    Zo, Hio = O.ibem(nodes, elems, mics, k, reg, sing, c, rho)
    assert relerr(Z, Zo) < 1e-10 and relerr(H, Hio) < 1e-10
    hm = take(m * 16).reshape(m, 16, order="F")
    hh = take(l * 16).reshape(l, 16, order="F")
    hq = take(m * 16).reshape(m, 16, order="F")
    hmo, hho, hqo = O.hels(g.cartesian_to_spherical(nodes), g.cartesian_to_spherical(mics), k, 3, c, rho)
    assert relerr(hm, hmo) < 1e-10 and relerr(hh, hho) < 1e-10 and relerr(hq, hqo) < 1e-10
    p = min(l, m)
    s = take(p, np.float64)
    assert np.max(np.abs(s - np.linalg.svd(H, compute_uv=False))) < 1e-12 * s[0]
    x = take(m)
    b = (1.0 + 0.1 * np.arange(l)) - 0.05j * np.arange(l)
    U, so, V = O.csvd(H)
    assert relerr(x, O.tsvd(U, so, V, b, 5)) < 1e-9
    pr = take(l)
    assert relerr(pr, H @ x) < 1e-12
    w = take(1, np.float64)[0]
    assert abs(w - O.sound_power(H @ x, b, 0.3)) < 1e-10 * abs(w)
    # invr, n_am = 9: the sphere's singular values of G Z come in multiplets
    # (1, 3, 5, ...), so the 9 leading vectors are compared as a subspace
    rq = take(m * 9).reshape(m, 9, order="F")
    rh = take(l * 9).reshape(l, 9, order="F")
    rm = take(m * 9).reshape(m, 9, order="F")
    _, Uo, _, _, Zr, Gr = O.bem_modes_complex(nodes, elems, mics, k, reg, sing, c, rho, 9)
    assert np.max(np.abs(rq.conj().T @ rq - np.eye(9))) < 1e-12
    assert np.linalg.norm(rq @ rq.conj().T - Uo @ Uo.conj().T) < 1e-9
    assert relerr(rh, Hio @ rq) < 1e-10 and relerr(rm, Zo @ rq) < 1e-10
