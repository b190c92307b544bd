"""CPU suite: the oracle pinned against the reference's own outputs (golden
vectors from its compiled CPU code), analytic known answers and
independent scipy implementations."""
import math

import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from oracle import ia_oracle as O


def test_rules_weights(golden):
    assert golden["rule_regular"].shape == (13, 3)
    assert abs(golden["rule_regular"][:, 2].sum() - 0.5) < 1e-14
    for p in range(3):
        assert abs(golden["rule_singular"][p, :, 2].sum() - 0.5) < 1e-13


def test_oracle_ibem_matches_reference(golden):
    c, rho = float(golden["c"]), float(golden["rho"])
    for i in range(2):
        Z, H = O.ibem(golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["ks"][i],
                      golden["rule_regular"], golden["rule_singular"], c, rho)
        assert relerr(Z, golden[f"ibem_Z_{i}"]) < 1e-12
        assert relerr(H, golden[f"ibem_H_{i}"]) < 1e-12


def test_oracle_ibem_chief_matches_reference(golden):
    c, rho = float(golden["c"]), float(golden["rho"])
    Z, H = O.ibem(golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["ks"][0],
                  golden["rule_regular"], golden["rule_singular"], c, rho, golden["chief"])
    assert relerr(Z, golden["ibem_chief_Z"]) < 1e-12
    assert relerr(H, golden["ibem_chief_H"]) < 1e-12


def test_oracle_transfer_equals_ibem_H(golden):
    c, rho = float(golden["c"]), float(golden["rho"])
    H = O.ibem_transfer(golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["ks"][1],
                        golden["rule_regular"], golden["rule_singular"], c, rho)
    assert relerr(H, golden["ibem_H_1"]) < 1e-12


def _invr_golden_problem(golden):
    return (golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["ks"][1], golden["rule_regular"],
            golden["rule_singular"], float(golden["c"]), float(golden["rho"]))


def test_oracle_mass_matrix_properties(golden):
    """G symmetric, sparse on the node-node pattern, and its entries sum to
    sum_e |n_e| sum_q w_q (the polyhedral area when the weights sum to 1/2)."""
    nodes, elems, reg = golden["mesh_nodes"], golden["mesh_elems"], golden["rule_regular"]
    G = O.mass_matrix(nodes, elems, reg)
    assert np.max(np.abs(G - G.T)) <= 1e-15 * np.max(G)
    v = nodes[:, elems]
    an = np.linalg.norm(np.cross((v[:, 0] - v[:, 2]).T, (v[:, 1] - v[:, 2]).T), axis=1)
    assert abs(G.sum() - an.sum() * reg[:, 2].sum()) < 1e-14 * G.sum()
    pattern = np.zeros_like(G, dtype=bool)
    for a in range(3):
        for b in range(3):
            pattern[elems[a], elems[b]] = True
    assert np.all(G[~pattern] == 0) and np.all(G[pattern] > 0)


def test_oracle_bem_modes_pinned_to_reference_invr(golden):
    """The reference invr() (n_am = m) returns q = U, h = H U and m_e = Z U
    with U the left singular vectors of G Z: Z and H recovered from them match
    the oracle's, and U diagonalises the oracle's (G Z)(G Z)^H with its
    singular values -- which pins the oracle's mass matrix G."""
    prob = _invr_golden_problem(golden)
    Q = golden["invr_q"]
    m = Q.shape[0]
    assert np.max(np.abs(Q.conj().T @ Q - np.eye(m))) < 1e-13
    s, U, h, me, Z, G = O.bem_modes_complex(*prob, m)
    assert relerr(Z, golden["invr_m"] @ Q.conj().T) < 1e-13
    assert relerr(h @ U.conj().T, golden["invr_h"] @ Q.conj().T) < 1e-13
    M = G @ Z
    D = Q.conj().T @ M @ M.conj().T @ Q
    assert np.max(np.abs(D - np.diag(np.diag(D)))) < 1e-13 * np.abs(D).max()
    assert np.max(np.abs(np.sqrt(np.diag(D).real) - s)) < 1e-13 * s[0]


def test_oracle_bem_modes_real_variant(golden):
    """invrS.m: U_r are the left singular vectors of Re(G Z); H_r = H U_r and
    P_r = Z U_r; sign convention of the device path."""
    prob = _invr_golden_problem(golden)
    s, Ur, Hr, Pr, Z, G = O.bem_modes(*prob, 12)
    R = (G @ Z).real
    assert np.max(np.abs(Ur.T @ Ur - np.eye(12))) < 1e-13
    assert np.linalg.norm(R @ R.T @ Ur - Ur * s**2) < 1e-12 * s[0] ** 2
    Zo, Ho = O.ibem(*prob)
    assert relerr(Hr, Ho @ Ur) < 1e-14 and relerr(Pr, Zo @ Ur) < 1e-14
    for j in range(12):
        a = np.abs(Ur[:, j])
        assert Ur[int(np.argmax(a >= a.max() * (1 - 1e-6))), j] > 0


def test_oracle_esm_matches_reference(golden):
    Me, He = O.esm(golden["esm_src"], golden["esm_fld"], float(golden["esm_k"]), float(golden["esm_ri"]),
                   float(golden["c"]), float(golden["rho"]))
    assert relerr(Me, golden["esm_Me"]) < 1e-12
    assert relerr(He, golden["esm_He"]) < 1e-12


def test_analytic_sphere_matches_reference(golden):
    k = golden["ks"][1]
    ps = g.pulsating_sphere_pressure(golden["mesh_nodes"], k, float(golden["kat_a"]), float(golden["kat_u"]))
    ph = g.pulsating_sphere_pressure(golden["mics"], k, float(golden["kat_a"]), float(golden["kat_u"]))
    assert relerr(ps, golden["kat_ps"]) < 1e-14
    assert relerr(ph, golden["kat_ph"]) < 1e-14


def test_cart2sph_matches_reference(golden):
    assert np.allclose(g.cartesian_to_spherical(golden["sph_in"]), golden["sph_out"], rtol=0, atol=1e-14)


def test_ibem_sphere_kat_reference_rules(golden):
    """IBEM of a pulsating sphere against the analytic field (the reference's
    own KAT, CUDA/utils.cuh:384): discretisation error only."""
    nodes, elems = g.icosphere(2, 0.1)
    mics = golden["mics"]
    k = 2 * np.pi * 700 / 343.0
    Z, H = O.ibem(nodes, elems, mics, k, golden["rule_regular"], golden["rule_singular"], 343.0, 1.21)
    ph = g.pulsating_sphere_pressure(mics, k, 0.1, 1.0)
    assert relerr(H @ np.ones(nodes.shape[1]), ph) < 3e-2


def test_hels_legendre_against_scipy():
    sp = pytest.importorskip("scipy.special")
    x = np.linspace(-0.99, 0.99, 7)
    P = O._assoc_legendre(12, x)
    for n in range(13):
        for m in range(n + 1):
            assert np.allclose(P[n, m], sp.lpmv(m, n, x), rtol=1e-10, atol=1e-12)


def test_hels_ynm_orthonormal():
    """Y_n^m columns are orthonormal under a product Gauss quadrature on the sphere."""
    order = 6
    xg, wg = np.polynomial.legendre.leggauss(16)
    nphi = 32
    phi = 2 * np.pi * np.arange(nphi) / nphi
    el = np.arccos(xg)
    AZ, EL = np.meshgrid(phi, el, indexing="ij")
    W = np.outer(np.full(nphi, 2 * np.pi / nphi), wg).ravel()
    Y = O._ynm_columns(order, AZ.ravel(), EL.ravel())
    G = (Y.conj().T * W) @ Y
    assert np.abs(G - np.eye(G.shape[0])).max() < 1e-12


def test_hels_monopole_expansion():
    """A monopole at the origin is exactly h_0 Y_0^0: He column 0 times
    ik sqrt(4 pi)/(4 pi) equals exp(ikr)/(4 pi r)."""
    P = g.cartesian_to_spherical(g.planar_array(4, 4, 0.05, 0.2))
    k = 2 * np.pi * 1000 / 343.0
    _, He, _ = O.hels(P, P, k, 3, 343.0, 1.21)
    r = P[2]
    coef = 1j * k * math.sqrt(4 * math.pi) / (4 * math.pi)
    assert relerr(He[:, 0] * coef, np.exp(1j * k * r) / (4 * np.pi * r)) < 1e-13


def test_gcv_standard_is_grid_minimum():
    rng = np.random.default_rng(5)
    A = g.complex_normal(rng, (40, 25)) @ np.diag(np.logspace(0, -6, 25))
    b = A @ g.complex_normal(rng, 25) + 1e-3 * g.complex_normal(rng, 40)
    U, s, V = O.csvd(A)
    lam = O.gcv(U, s, b)
    beta = U.conj().T @ b
    d0 = O.gcv_delta0(b, beta, 40, 25)
    fine = np.exp(np.linspace(math.log(lam) - 0.05, math.log(lam) + 0.05, 2001))
    G = [O.gcv_function(s, beta, la, 40, d0) for la in fine]
    assert abs(math.log(fine[int(np.argmin(G))]) - math.log(lam)) < 1e-4


def test_fminbnd_matches_scipy_bounded():
    opt = pytest.importorskip("scipy.optimize")
    f = lambda x: (x - 0.3) ** 2 + 0.1 * math.sin(5 * x)  # noqa: E731
    ours = O.fminbnd(f, 0.0, 1.0, tolx=1e-10)
    theirs = opt.minimize_scalar(f, bounds=(0.0, 1.0), method="bounded", options={"xatol": 1e-10}).x
    assert abs(ours - theirs) < 1e-8


def test_tikhonov_normal_equations():
    rng = np.random.default_rng(7)
    A = g.complex_normal(rng, (30, 50))
    b = g.complex_normal(rng, 30)
    U, s, V = O.csvd(A)
    lam = 0.37
    x = O.tikhonov(U, s, V, b, lam)
    lhs = A.conj().T @ A @ x + lam ** 2 * x
    assert relerr(lhs, A.conj().T @ b) < 1e-12


def test_tsvd_and_range():
    rng = np.random.default_rng(8)
    A = g.complex_normal(rng, (20, 12))
    b = g.complex_normal(rng, 20)
    U, s, V = O.csvd(A)
    x = O.tsvd(U, s, V, b, 12)
    assert relerr(x, np.linalg.lstsq(A, b, rcond=None)[0]) < 1e-12
    with pytest.raises(ValueError):
        O.tsvd(U, s, V, b, 0)
    with pytest.raises(ValueError):
        O.tsvd(U, s, V, b, 13)


def test_sinc_resistance_properties():
    P, area = g.plate_grid(0.5, 0.4, 8, 6)
    k = 2 * np.pi * 500 / 343.0
    R = O.sinc_resistance(P, k, 343.0, 1.21, area)
    assert np.allclose(R, R.T)
    w, _ = O.radiation_modes(P, k, 343.0, 1.21, area)
    assert w.min() > -1e-10 * w.max()          # positive semidefinite
    om = k * 343.0
    assert abs(R[0, 0] - om * om * 1.21 * area * area / (4 * np.pi * 343.0)) < 1e-12 * R[0, 0]


def _design_case(seed=0, l=12, subdiv=1, F=3, R=4):
    rng = np.random.default_rng(seed)
    surf, _ = g.icosphere(subdiv, 0.1)
    mics = np.stack([rng.uniform(-.2, .2, l), rng.uniform(-.2, .2, l), np.full(l, .12)])
    k = 2 * np.pi * np.linspace(300.0, 3000.0, F) / 343.0
    q = g.complex_normal(rng, (F, surf.shape[1], R))
    noise = 0.01 * g.complex_normal(rng, (F, l, R))
    loglam = np.array([math.log(0.05 * np.linalg.norm(O.monopole_matrix(mics, O.retreat_sources(surf, 0.04), kk), 2))
                       for kk in k])
    return mics, surf, 0.04, k, loglam, q, noise


def test_design_gradient_matches_central_differences():
    """The FP64 reference gradient of the design loss (adjoint of the
    Tikhonov solve) against central differences, h = 1e-6."""
    mics, surf, d, k, ll, q, noise = _design_case()
    gm, gd, gl = O.esm_design_grad(mics, surf, d, k, ll, q, noise)
    h = 1e-6

    def L(M=mics, D=d, LL=ll):
        return O.esm_design_loss(M, surf, D, k, LL, q, noise)

    fd = np.zeros_like(gm)
    for a in range(3):
        for i in range(mics.shape[1]):
            Mp, Mm = mics.copy(), mics.copy()
            Mp[a, i] += h
            Mm[a, i] -= h
            fd[a, i] = (L(M=Mp) - L(M=Mm)) / (2 * h)
    assert np.max(np.abs(fd - gm)) <= 1e-6 * np.max(np.abs(gm))
    assert abs((L(D=d + h) - L(D=d - h)) / (2 * h) - gd) <= 1e-6 * abs(gd)
    E = np.eye(len(k))
    fl = np.array([(L(LL=ll + h * E[f]) - L(LL=ll - h * E[f])) / (2 * h) for f in range(len(k))])
    assert np.max(np.abs(fl - gl)) <= 1e-6 * np.max(np.abs(gl))


def test_lambda_selectors_restatement():
    """L-curve corner and quasi-optimality restatements: the fminbnd result
    sits at the minimum of the objective on a dense grid of its bracket, the
    corner is inside the grid, and the damped SVD solves its diagonal system."""
    rng = np.random.default_rng(4)
    mics = g.planar_array(8, 8, 0.03, 0.10)
    src, _ = g.icosphere(1, 0.05)
    k = 2 * np.pi * 1200 / 343.0
    G = O.monopole_matrix(mics, src, k)
    b = g.add_noise(rng, G @ g.complex_normal(rng, src.shape[1]), 25.0)
    U, s, V = O.csvd(G)
    beta = U.conj().T @ b
    xi = beta / s
    rho_ls2 = O.gcv_delta0(b, beta, G.shape[0], s.size)      # m > p: least-squares residual term
    assert rho_ls2 > 0
    for method in ("t", "d"):
        lc = O.l_curve(U, s, b, method)
        dense = np.geomspace(lc / 1.2, lc * 1.2, 2001)
        vals = [O.lcfun(la, s, beta, xi, method, rho_ls2) for la in dense]
        assert abs(dense[int(np.argmin(vals))] - lc) <= 2e-3 * lc + 1e-4
        assert s[-1] <= lc <= s[0]
        qo = O.quasiopt(U, s, b, method)
        f = O._filter(s, qo, method)
        # within the bracket the grid minimum gives (here the grid's top end, s_1)
        dense = np.geomspace(max(qo / 1.2, s[-1]), min(qo * 1.2, s[0]), 2001)
        qv = [np.linalg.norm((1 - O._filter(s, la, method)) * O._filter(s, la, method) * xi) for la in dense]
        assert abs(dense[int(np.argmin(qv))] - qo) <= 2e-3 * qo + 1e-4
        assert np.isfinite(f).all()
    x = O.dsvd(U, s, V, b, 0.3)
    assert relerr(V.conj().T @ x * (s + 0.3), U.conj().T @ b) < 1e-12


def _admm_problem(seed, l, m, k=3, noise=1e-3):
    rng = np.random.default_rng(seed)
    A = (rng.normal(size=(l, m)) + 1j * rng.normal(size=(l, m))) / np.sqrt(l)
    xt = np.zeros(m, complex)
    idx = rng.choice(m, k, replace=False)
    xt[idx] = rng.normal(size=k) + 1j * rng.normal(size=k)
    b = A @ xt + noise * (rng.normal(size=l) + 1j * rng.normal(size=l))
    return A, b, xt


def test_admm_l2_fixed_point_is_tikhonov():
    """ADMMG.m case 2 converges to argmin ||Ac - b||^2 + lambda_0 ||c||^2."""
    for l, m in ((20, 60), (40, 12)):
        A, b, _ = _admm_problem(1, l, m)
        c, its, conv = O.admm(A, b, 0.3, 5.0, 1.0, 1e-12, 5000, 2)
        assert conv
        ct = np.linalg.solve(A.conj().T @ A + 0.3 * np.eye(m), A.conj().T @ b)
        assert relerr(c, ct) < 1e-10


def test_admm_l1_fixed_point_is_lasso():
    """ADMMG.m case 1 stops at a lasso point of its current stage lambda:
    2 [A^H (b - A c)]_j = lambda c_j / |c_j| on the support, |.| <= lambda off it."""
    A, b, xt = _admm_problem(2, 30, 80)
    lam0, Nm = 0.5, 2000
    c, its, conv = O.admm(A, b, lam0, 5.0, 1.0, 1e-10, Nm, 1)
    assert conv
    lam = 5 * lam0 * 0.75 ** ((its - 1) // Nm)
    g_ = 2 * A.conj().T @ (b - A @ c)
    on = np.abs(c) > 1e-8
    assert on.sum() >= 3
    assert np.max(np.abs(g_[on] - lam * c[on] / np.abs(c[on]))) < 1e-6
    assert np.max(np.abs(g_[~on])) <= lam * (1 + 1e-6)


def test_admm_gst_threshold_and_x0():
    # p = 1: the generalised soft threshold is the soft threshold lambda_p
    assert O.admm_gst_threshold(0.7, 1.0) == 0.7
    # p = 1/2: tau = (lambda_p)^(2/3) + (lambda_p / 2) (lambda_p)^(-1/3), the
    # point where the thresholded value would reach its fixed point
    lp = 0.4
    assert abs(O.admm_gst_threshold(lp, 0.5) - (lp ** (2 / 3) + 0.5 * lp * lp ** (-1 / 3))) < 1e-15
    # x0: minimum norm for wide A (in the range of A^H), least squares for tall
    A, b, _ = _admm_problem(3, 10, 30)
    x0 = O.admm_x0(A, b)
    assert relerr(A @ x0, b) < 1e-12
    assert relerr(x0, np.linalg.pinv(A) @ b) < 1e-12
    A, b, _ = _admm_problem(4, 30, 10)
    assert relerr(O.admm_x0(A, b), np.linalg.lstsq(A, b, rcond=None)[0]) < 1e-12
