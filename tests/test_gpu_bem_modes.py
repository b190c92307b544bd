"""GPU suite: BEM radiation modes (ia_bem_modes_batch, ia_bem_modes_complex_batch,
ia_invr) against the oracle's restatement of MATLAB/invrS.m and the C++
invr() (CUDA/invr.cuh:457-909), and against the reference invr()'s own
outputs (golden fixture).

Geometry: an icosphere (162 nodes) scaled to an ellipsoid (0.1, 0.08, 0.06 m)
so that few singular values are degenerate, 24 field points at 0.3 m.

Bounds.  Real variant (singular vectors of R = Re(G Z) as eigenvectors of
R R^T): s^2 within 1e-12 s_1^2 (FP64) / 1e-10 s_1^2 (mixed); vectors of modes
with s_j > 1e-3 s_1 and a relative gap in s^2 above 1e-3, 1e-8 (FP64) / 1e-6
(mixed), up to sign, and the device sign convention exactly; residual
||R R^T U - U s^2|| within 1e-11 s_1^2.  Complex variant (FP64 Jacobi SVD of
G Z; mixed: subspace iteration on the real representation of (G Z)(G Z)^H):
s within 1e-11 s_1 (FP64) / 1e-9 s_1 (mixed); vectors with a relative gap
above 1e-4 within 1e-9 (FP64) / 1e-7 (mixed) after the phase convention.
Both: H_r = H U and P_r = Z U with the oracle's
H and Z and the device U, 1e-11 relative (FP64) / 1e-8 (mixed)."""
import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from inverseacoustics_gb300 import quadrature as Q
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu
C, RHO = 343.0, 1.21


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


@pytest.fixture(scope="module")
def ellipsoid():
    nodes, elems = g.icosphere(2, 1.0)
    nodes = np.ascontiguousarray(nodes * np.array([[0.1], [0.08], [0.06]]))
    mics = g.hemisphere_array(np.random.default_rng(7), 24, 0.3)
    ks = 2 * np.pi * np.array([120.0, 700.0, 1600.0]) / C
    return nodes, elems, mics, ks


def _run(ctx, cuda, ellipsoid, nm, precision, complex_modes, cp=None):
    from inverseacoustics_gb300 import api
    import torch
    nodes, elems, mics, ks = ellipsoid
    mesh = api.Mesh(ctx, nodes, elems)
    cfg = api.default_config(precision=precision)
    out = api.bem_modes_batch(ctx, mesh, T(mics, cuda), T(ks, cuda), nm, cfg, cp=None if cp is None else T(cp, cuda),
                              complex_modes=complex_modes)
    torch.cuda.synchronize()
    s, U, Hr, Pr, info = (None if a is None else a.cpu().numpy() for a in out)
    mesh.close()
    return s, U, Hr, Pr, info


@pytest.mark.parametrize("precision", [0, 1])
def test_bem_modes_real_match_oracle(cuda, ctx, ellipsoid, precision):
    nodes, elems, mics, ks = ellipsoid
    nm = 12
    s, U, Hr, Pr, info = _run(ctx, cuda, ellipsoid, nm, precision, False)
    assert int(np.abs(info).sum()) == 0
    reg, sing = Q.builtin()
    s2_tol, vec_tol, prod_tol = (1e-12, 1e-8, 1e-11) if precision == 0 else (1e-10, 1e-6, 1e-8)
    checked = 0
    for f, k in enumerate(ks):
        so, Uo, _, _, Zo, Go = O.bem_modes(nodes, elems, mics, k, reg, sing, C, RHO, nm + 1)
        _, Ho = O.ibem(nodes, elems, mics, k, reg, sing, C, RHO)
        X = U[f].T                                          # m x nm
        s1 = so[0]
        assert np.max(np.abs(s[f] ** 2 - so[:nm] ** 2)) <= s2_tol * s1 ** 2
        assert np.all(np.diff(s[f]) <= 0)
        assert np.max(np.abs(X.T @ X - np.eye(nm))) < 1e-12
        R = (Go @ Zo).real
        assert np.linalg.norm(R @ (R.T @ X) - X * s[f] ** 2) <= 1e-11 * s1 ** 2
        for j in range(nm):
            if so[j] < 1e-3 * s1:
                continue
            gap = min(so[j - 1] ** 2 - so[j] ** 2 if j > 0 else np.inf, so[j] ** 2 - so[j + 1] ** 2) / s1 ** 2
            if gap < 1e-3:
                continue
            assert np.linalg.norm(X[:, j] - Uo[:, j]) <= vec_tol, (f, j)
            checked += 1
        for j in range(nm):
            a = np.abs(X[:, j])
            assert X[int(np.argmax(a >= a.max() * (1 - 1e-6))), j] > 0
        assert relerr(Hr[f].T, Ho @ X) < prod_tol
        assert relerr(Pr[f].T, Zo @ X) < prod_tol
    assert checked >= 12


@pytest.mark.parametrize("precision", [0, 1])
def test_bem_modes_complex_match_oracle(cuda, ctx, ellipsoid, precision):
    nodes, elems, mics, ks = ellipsoid
    nm = 10
    s, U, Hr, Pr, info = _run(ctx, cuda, ellipsoid, nm, precision, True)
    assert int(np.abs(info).sum()) == 0
    reg, sing = Q.builtin()
    s_tol, vec_tol, prod_tol = (1e-11, 1e-9, 1e-11) if precision == 0 else (1e-9, 1e-7, 1e-8)
    checked = 0
    for f, k in enumerate(ks):
        so, Uo, _, _, Zo, _ = O.bem_modes_complex(nodes, elems, mics, k, reg, sing, C, RHO, nm + 1)
        _, Ho = O.ibem(nodes, elems, mics, k, reg, sing, C, RHO)
        X = U[f].T
        assert np.max(np.abs(s[f] - so[:nm])) <= s_tol * so[0]
        assert np.max(np.abs(X.conj().T @ X - np.eye(nm))) < 1e-12
        for j in range(nm):
            gap = min(so[j - 1] - so[j] if j > 0 else np.inf, so[j] - so[j + 1]) / so[0]
            if gap < 1e-4:
                continue
            assert np.linalg.norm(X[:, j] - Uo[:, j]) <= vec_tol, (f, j)
            checked += 1
        assert relerr(Hr[f].T, Ho @ X) < prod_tol
        assert relerr(Pr[f].T, Zo @ X) < prod_tol
    assert checked >= 20


@pytest.mark.parametrize("precision", [0, 1])
def test_bem_modes_chief_least_squares(cuda, ctx, ellipsoid, precision):
    """Two CHIEF points inside the surface: Z by least squares (invr.cuh:860
    zgels, invrS.m:159 backslash).  Mixed precision: double-float rows, FP64
    least squares, modes by subspace iteration on the real representation."""
    nodes, elems, mics, ks = ellipsoid
    cp = np.array([[0.01, 0.02, -0.01], [-0.03, 0.0, 0.015]]).T.copy()
    nm = 8
    s, U, Hr, Pr, info = _run(ctx, cuda, ellipsoid, nm, precision, True, cp=cp)
    assert int(np.abs(info).sum()) == 0
    reg, sing = Q.builtin()
    s_tol, proj_tol, prod_tol = (1e-11, 1e-8, 1e-11) if precision == 0 else (1e-9, 1e-7, 1e-9)
    for f, k in enumerate(ks):
        so, Uo, _, _, Zo, _ = O.bem_modes_complex(nodes, elems, mics, k, reg, sing, C, RHO, nm, chief=cp)
        _, Ho = O.ibem(nodes, elems, mics, k, reg, sing, C, RHO, cp)
        X = U[f].T
        assert np.max(np.abs(s[f] - so)) <= s_tol * so[0]
        assert np.linalg.norm(X @ X.conj().T - Uo @ Uo.conj().T) < proj_tol
        assert relerr(Hr[f].T, Ho @ X) < prod_tol and relerr(Pr[f].T, Zo @ X) < prod_tol


def test_bem_modes_batch_is_per_frequency(cuda, ctx, ellipsoid):
    """A frequency's modes do not depend on the rest of the batch: bitwise equal
    alone and inside a batch."""
    nodes, elems, mics, ks = ellipsoid
    full = _run(ctx, cuda, ellipsoid, 6, 0, False)
    one = _run(ctx, cuda, (nodes, elems, mics, ks[1:2]), 6, 0, False)
    for a, b in zip(full[:4], one[:4]):
        assert np.array_equal(a[1], b[0])


def _clusters(s, rel=1e-6):
    out, start = [], 0
    for j in range(1, len(s) + 1):
        if j == len(s) or s[j - 1] - s[j] > rel * s[0]:
            out.append((start, j))
            start = j
    return out


def test_invr_matches_reference_golden(cuda, golden):
    """ia_invr with n_am = m against the reference invr() itself: the sphere's
    singular values of G Z come in multiplets, so q is compared through the
    projector onto each cluster; h q^H and m_e q^H (= H and Z) directly."""
    from inverseacoustics_gb300 import api
    nodes, elems, mics, k = golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["ks"][1]
    rules = (golden["rule_regular"], golden["rule_singular"])
    c, rho = float(golden["c"]), float(golden["rho"])
    m = nodes.shape[1]
    me, h, q = api.invr(nodes, elems, mics, k, m, rules=rules, c=c, rho=rho)
    Qr = golden["invr_q"]
    assert np.max(np.abs(q.conj().T @ q - np.eye(m))) < 1e-12
    assert relerr(me @ q.conj().T, golden["invr_m"] @ Qr.conj().T) < 1e-10
    assert relerr(h @ q.conj().T, golden["invr_h"] @ Qr.conj().T) < 1e-10
    so = O.bem_modes_complex(nodes, elems, mics, k, *rules, c, rho, m)[0]
    for a, b in _clusters(so):
        if so[a] < 1e-8 * so[0]:
            break
        P = q[:, a:b] @ q[:, a:b].conj().T
        Pr = Qr[:, a:b] @ Qr[:, a:b].conj().T
        assert np.linalg.norm(P - Pr) < 1e-8, (a, b)
    # n_am < m: the leading columns of the same modes
    me8, h8, q8 = api.invr(nodes, elems, mics, k, 9, rules=rules, c=c, rho=rho)
    assert np.array_equal(q8, q[:, :9])
    assert relerr(h8, h[:, :9]) < 1e-14 and relerr(me8, me[:, :9]) < 1e-14


def test_bem_modes_complex_mixed_dense_spectrum(cuda, ctx):
    """Mixed complex variant on a 642-node sphere (radius 0.1 m, 48 field
    points), whose G Z has a dense spectrum of multiplets: s within 1e-10 s_1,
    columns orthonormal, residuals ||(G Z)(G Z)^H u - s^2 u|| within
    1e-9 s_1^2, and every multiplet that lies wholly inside the nm leading
    modes spanned to 1e-7 (projectors).  nm = 32 and frequencies at which a
    multiplet straddles the 64th real Ritz value of the doubled spectrum."""
    from inverseacoustics_gb300 import api
    nodes, elems = g.icosphere(3, 0.1)
    mics = g.hemisphere_array(np.random.default_rng(11), 48, 0.5)
    ks = 2 * np.pi * np.array([200.0, 1500.0, 2600.0]) / C
    nm = 32
    mesh = api.Mesh(ctx, nodes, elems)
    s, U, Hr, Pr, info = (a.cpu().numpy() for a in api.bem_modes_batch(
        ctx, mesh, T(mics, cuda), T(ks, cuda), nm, api.default_config(precision=1), complex_modes=True))
    mesh.close()
    assert int(np.abs(info).sum()) == 0
    reg, sing = Q.builtin()
    for f, k in enumerate(ks):
        so, Uo, _, _, Zo, Go = O.bem_modes_complex(nodes, elems, mics, k, reg, sing, C, RHO, nodes.shape[1])
        Y = Go @ Zo
        X = U[f].T
        assert np.max(np.abs(s[f] - so[:nm])) <= 1e-10 * so[0]
        assert np.max(np.abs(X.conj().T @ X - np.eye(nm))) < 1e-12
        res = np.linalg.norm(Y @ (Y.conj().T @ X) - X * s[f] ** 2, axis=0)
        assert res.max() <= 1e-9 * so[0] ** 2
        for a, b in _clusters(so, 1e-8):
            if b > nm:
                break
            P = X[:, a:b] @ X[:, a:b].conj().T
            Po = Uo[:, a:b] @ Uo[:, a:b].conj().T
            assert np.linalg.norm(P - Po) < 1e-7, (f, a, b)


def test_bem_modes_complex_mixed_many_modes(cuda, ctx, ellipsoid):
    """Mixed complex variant with nm + max(nm, oversample) above m / 2: the
    FP64 Jacobi SVD of the double-float G Z, so s agrees with the FP64 run to
    the assembly's accuracy and the columns are orthonormal."""
    nm = 90
    s1, U1, _, _, info1 = _run(ctx, cuda, ellipsoid, nm, 1, True)
    s0, U0, _, _, info0 = _run(ctx, cuda, ellipsoid, nm, 0, True)
    assert int(np.abs(info1).sum()) == 0 and int(np.abs(info0).sum()) == 0
    for f in range(len(ellipsoid[3])):
        assert np.max(np.abs(s1[f] - s0[f])) <= 1e-10 * s0[f][0]
        X = U1[f].T
        assert np.max(np.abs(X.conj().T @ X - np.eye(nm))) < 1e-12


def test_bem_modes_complex_all_modes_full_sphere(cuda, ctx):
    """FP64 complex variant with every mode (n_am = m, the drop-in invr()'s
    natural call) on the 642-node sphere: the SVD of the whole 642 x 642 G Z.
    It runs round by round over the whole GPU (one CTA per column pair and
    bin); the test prints its time.  s within 1e-11 s_1 of LAPACK's, columns
    orthonormal to 1e-12, residuals ||(G Z)(G Z)^H u - s^2 u|| within
    1e-11 s_1^2."""
    import time
    import torch
    from inverseacoustics_gb300 import api
    nodes, elems = g.icosphere(3, 0.1)
    m = nodes.shape[1]
    mics = g.hemisphere_array(np.random.default_rng(11), 48, 0.5)
    ks = 2 * np.pi * np.array([900.0]) / C
    mesh = api.Mesh(ctx, nodes, elems)
    args = (T(mics, cuda), T(ks, cuda), m, api.default_config(precision=0))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = api.bem_modes_batch(ctx, mesh, *args, complex_modes=True)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    s, U, Hr, Pr, info = (a.cpu().numpy() for a in out)
    mesh.close()
    print(f"\ncomplex BEM modes, all {m} of the 642-node sphere, FP64: {dt:.3f} s per frequency")
    assert int(np.abs(info).sum()) == 0
    reg, sing = Q.builtin()
    so, Uo, _, _, Zo, Go = O.bem_modes_complex(nodes, elems, mics, ks[0], reg, sing, C, RHO, m)
    Y = Go @ Zo
    X = U[0].T
    assert np.max(np.abs(s[0] - so)) <= 1e-11 * so[0]
    assert np.max(np.abs(X.conj().T @ X - np.eye(m))) < 1e-12
    res = np.linalg.norm(Y @ (Y.conj().T @ X) - X * s[0] ** 2, axis=0)
    assert res.max() <= 1e-11 * so[0] ** 2
