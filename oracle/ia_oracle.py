"""FP64 CPU restatement of the reference's inverse pipeline (the oracle).

ORACLE / TEST INFRASTRUCTURE ONLY.  Imported by tests/, by
__graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline and
reference legs.  The product path (inverseacoustics_gb300) never imports it.

Each function cites the reference code it restates.  Parity pins:
  * esm / ibem against the reference's own compiled CPU code
    (oracle/_ref/libiaref.so), frozen as golden fixtures in tests/golden/
    by tests/golden/make_golden.py;
  * hels against scipy's spherical Bessel and Legendre functions (the
    reference's CPU hels() needs GSL, which is absent);
  * gcv / tikhonov / tsvd / csvd restate MATLAB/regtools/*G.m (MATLAB is
    absent); sinc-R has no reference code and is unpinned;
  * bem_modes / mass_matrix against the reference's own invr() output;
  * admm restates MATLAB/ADMMG.m; with MATLAB absent it is pinned by its
    fixed points only (L2: the Tikhonov solution; L1: the lasso optimality
    conditions), not by reference outputs.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
C_LIB_PATH = os.path.join(HERE, "_build", "libiaoracle.so")
INV4PI = 1.0 / (4.0 * math.pi)
EPS = np.finfo(np.float64).eps

_clib = None


def clib():
    """The C restatement (oracle/ibem_oracle.c), built by oracle/build.py."""
    global _clib
    if _clib is None:
        if not os.path.exists(C_LIB_PATH):
            from oracle import build as _b
            _b.build_oracle()
        _clib = C.CDLL(C_LIB_PATH)
        P = C.c_void_p
        _clib.ora_ibem_assemble.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, C.c_double, C.c_int, P, C.c_int, P,
                                            C.c_int, P, C.c_double, C.c_double, P, P, P, P]
        _clib.ora_sinc_resistance.argtypes = [C.c_int, P, C.c_double, C.c_double, C.c_double, C.c_double, P]
    return _clib


def _soa(P):
    return np.ascontiguousarray(np.asarray(P, dtype=np.float64))


# ---------------------------------------------------------------------------
# ESM  (MATLAB/esmV.m:20-30; CUDA/esm.cuh:112-174)
# ---------------------------------------------------------------------------
def esm_matrices(r_ms, r_lh, k, r_i, c, rho):
    """D, M_sq (m x m; rows = surface points, cols = sources) and M_hq
    (l x m) of the equivalent source method, sources at r_ms * r_i."""
    S = _soa(r_ms).T            # (m, 3)
    Hp = _soa(r_lh).T           # (l, 3)
    Q = S * r_i
    dsq = S[:, None, :] - Q[None, :, :]
    R_sq = np.sqrt((dsq ** 2).sum(-1))
    vr_s = np.sqrt((S ** 2).sum(-1))
    cos_t = (S[:, None, :] * dsq).sum(-1) / (vr_s[:, None] * R_sq)
    ek = np.exp(1j * k * R_sq)
    D = ((1j * k * R_sq - 1.0) / (4 * np.pi * R_sq ** 2)) * ek * cos_t
    M_sq = (1j * rho * k * c) * (ek / (4 * np.pi * R_sq))
    R_hq = np.sqrt(((Hp[:, None, :] - Q[None, :, :]) ** 2).sum(-1))
    M_hq = (1j * rho * k * c) * (np.exp(1j * k * R_hq) / (4 * np.pi * R_hq))
    return D, M_sq, M_hq


def esm(r_ms, r_lh, k, r_i, c, rho):
    """Me = M_sq D^-1 and He = M_hq D^-1 (esmV.m:30; esm.cuh:153-170)."""
    D, M_sq, M_hq = esm_matrices(r_ms, r_lh, k, r_i, c, rho)
    DT = D.T
    Me = np.linalg.solve(DT, M_sq.T).T
    He = np.linalg.solve(DT, M_hq.T).T
    return Me, He


def monopole_matrix(mics, sources, k):
    """Plain ESM transfer matrix G_ij = exp(ik r_ij) / (4 pi r_ij) between
    microphones (rows) and equivalent sources (cols); equals M_hq/(i rho c k)
    of esmV.m:29-30 with the sources given directly."""
    Mi = _soa(mics).T
    Sj = _soa(sources).T
    R = np.sqrt(((Mi[:, None, :] - Sj[None, :, :]) ** 2).sum(-1))
    return np.exp(1j * k * R) / (4 * np.pi * R)


def retreat_sources(surface, retreat):
    """Surface points moved radially toward the origin by ``retreat``."""
    S = _soa(surface)
    rn = np.linalg.norm(S, axis=0)
    return S * (1.0 - retreat / rn)


# ---------------------------------------------------------------------------
# IBEM  (CUDA/ibem.cuh:424-770; OpenBEM collocation)
# ---------------------------------------------------------------------------
def _rule_soa(rule):
    rule = np.asarray(rule, dtype=np.float64)
    return np.ascontiguousarray(rule.T).ravel(), rule.shape[0]


def ibem_assemble(nodes, elems, mics, k, regular, singular, c, rho, chief=None):
    """A, B (scaled by i rho c k) of size (m+n_ch) x m and A_hs, B_hs (l x m),
    exactly the matrices the reference builds before its zgels
    (CUDA/ibem.cuh:479-746)."""
    r_ms = _soa(nodes).ravel()
    r_lh = _soa(mics).ravel()
    e_n = np.ascontiguousarray(np.asarray(elems, dtype=np.int32)).ravel()
    m, l, n = r_ms.size // 3, r_lh.size // 3, e_n.size // 3
    n_ch = 0 if chief is None else np.asarray(chief).shape[1]
    cp = _soa(chief).ravel() if n_ch else np.zeros(3)
    reg, nq = _rule_soa(regular)
    sing = np.asarray(singular, dtype=np.float64)
    nqs = sing.shape[1]
    sg = np.ascontiguousarray(np.concatenate([_rule_soa(sing[p])[0] for p in range(3)]))
    mt = m + n_ch
    A = np.zeros((mt, m), np.complex128, order="F")
    B = np.zeros((mt, m), np.complex128, order="F")
    Ahs = np.zeros((l, m), np.complex128, order="F")
    Bhs = np.zeros((l, m), np.complex128, order="F")
    clib().ora_ibem_assemble(m, l, n, r_ms.ctypes.data, e_n.ctypes.data, r_lh.ctypes.data, float(k), nq,
                             reg.ctypes.data, nqs, sg.ctypes.data, n_ch, cp.ctypes.data, float(c), float(rho),
                             A.ctypes.data, B.ctypes.data, Ahs.ctypes.data, Bhs.ctypes.data)
    return A, B, Ahs, Bhs


def ibem(nodes, elems, mics, k, regular, singular, c, rho, chief=None):
    """Z = A \\ B (least squares when CHIEF rows are present) and
    H = A_hs Z - B_hs (CUDA/ibem.cuh:748-769)."""
    A, B, Ahs, Bhs = ibem_assemble(nodes, elems, mics, k, regular, singular, c, rho, chief)
    if A.shape[0] == A.shape[1]:
        Z = np.linalg.solve(A, B)
    else:
        Z = np.linalg.lstsq(A, B, rcond=None)[0]
    return Z, Ahs @ Z - Bhs


def ibem_transfer(nodes, elems, mics, k, regular, singular, c, rho, chief=None):
    """Only H, computed as W B - B_hs with W = A_hs A^-1 (the same matrix as
    ibem()'s H, through an l-right-hand-side solve)."""
    A, B, Ahs, Bhs = ibem_assemble(nodes, elems, mics, k, regular, singular, c, rho, chief)
    if A.shape[0] != A.shape[1]:
        return ibem(nodes, elems, mics, k, regular, singular, c, rho, chief)[1]
    W = np.linalg.solve(A.T, Ahs.T).T
    return W @ B - Bhs


# ---------------------------------------------------------------------------
# HELS  (CUDA/hels.cuh:222-323; MATLAB/helsV.m)
# ---------------------------------------------------------------------------
def _assoc_legendre(nmax, x):
    """P_n^m(x) for 0 <= m <= n <= nmax with the Condon-Shortley phase, built
    as the reference does: (-1)^m (1-x^2)^{m/2} (2m)!/(2^m m!) C^{m+1/2}_{n-m}(x)
    (CUDA/hels.cuh:239-245), the Gegenbauer polynomial by its three-term
    recurrence (MATLAB/gegenbauer.m:5-27)."""
    x = np.asarray(x, dtype=np.float64)
    P = np.zeros((nmax + 1, nmax + 1) + x.shape)
    for mm in range(nmax + 1):
        lam = mm + 0.5
        pref = (-1.0) ** mm * (1 - x * x) ** (mm / 2.0) * math.factorial(2 * mm) / (2.0 ** mm * math.factorial(mm))
        g_prev2 = np.ones_like(x)
        g_prev1 = 2 * lam * x
        for d in range(nmax - mm + 1):
            if d == 0:
                gd = g_prev2
            elif d == 1:
                gd = g_prev1
            else:
                gd = (2 * (d - 1 + lam) * x * g_prev1 - (d - 1 + 2 * lam - 1) * g_prev2) / d
                g_prev2, g_prev1 = g_prev1, gd
            P[mm + d, mm] = pref * gd
    return P


def _ynm_columns(order, az, el):
    """Y_n^m at points (az, el) for every column i = n^2 + n + m, m = -n..n
    (CUDA/hels.cuh:235, 246-247, 271)."""
    nt = (order + 1) ** 2
    P = _assoc_legendre(order, np.cos(el))
    Y = np.zeros((az.size, nt), np.complex128)
    for i in range(nt):
        nn = int(math.floor(math.sqrt(i)))
        mm = i - nn - nn * nn
        a = abs(mm)
        norm = math.sqrt((2 * nn + 1) * math.factorial(nn - a) / (4 * math.pi * math.factorial(nn + a)))
        y = norm * P[nn, a] * np.exp(1j * a * az)
        if mm < 0:
            y = (-1.0) ** a * np.conj(y)
        Y[:, i] = y
    return Y


def _sph_h(order, x):
    from scipy.special import spherical_jn, spherical_yn
    ns = np.arange(order + 1)[:, None]
    h = spherical_jn(ns, x[None, :]) + 1j * spherical_yn(ns, x[None, :])
    dh = spherical_jn(ns, x[None, :], derivative=True) + 1j * spherical_yn(ns, x[None, :], derivative=True)
    return h, dh


def hels(r_ms_s, r_lh_s, k, order, c, rho):
    """Me (m x nt), He (l x nt), Qe (m x nt): h_n(kr) Y_n^m, h_n(kr) Y_n^m,
    h_n'(kr) k Y_n^m / (i rho c k), h_n = j_n + i y_n (CUDA/hels.cuh:248-257,
    298-302).  Points are (az, el, r) rows (CUDA/utils.cuh:414)."""
    S = _soa(r_ms_s)
    Hp = _soa(r_lh_s)
    ns = np.array([int(math.floor(math.sqrt(i))) for i in range((order + 1) ** 2)])
    Ys = _ynm_columns(order, S[0], S[1])
    Yh = _ynm_columns(order, Hp[0], Hp[1])
    hs, dhs = _sph_h(order, k * S[2])
    hh, _ = _sph_h(order, k * Hp[2])
    Me = hs[ns].T * Ys
    Qe = (1.0 / (1j * rho * c * k)) * (k * dhs[ns].T) * Ys
    He = hh[ns].T * Yh
    return Me, He, Qe


# ---------------------------------------------------------------------------
# radiation resistance (sinc form; no reference code -- unpinned)
# ---------------------------------------------------------------------------
def sinc_resistance(centres, k, c, rho, area):
    x = _soa(centres).ravel()
    n = x.size // 3
    R = np.zeros((n, n), order="F")
    clib().ora_sinc_resistance(n, x.ctypes.data, float(k), float(c), float(rho), float(area), R.ctypes.data)
    return R


def radiation_modes(centres, k, c, rho, area):
    """Eigenpairs of R (descending eigenvalues)."""
    R = sinc_resistance(centres, k, c, rho, area)
    w, V = np.linalg.eigh(R)
    return w[::-1].copy(), V[:, ::-1].copy()


def sound_power_R(R, v):
    """W = 1/2 v^H R v (real R)."""
    return 0.5 * float(np.real(np.vdot(v, R @ v)))


# ---------------------------------------------------------------------------
# BEM radiation modes  (MATLAB/invrS.m:18-170; CUDA/invr.cuh:457-909)
# ---------------------------------------------------------------------------
def mass_matrix(nodes, elems, regular):
    """Surface mass matrix G (m x m) accumulated element by element with the
    regular rule: G[e_a, e_b] += |n_e| sum_q w_q N_a(q) N_b(q), N = (x1, x2,
    1 - x1 - x2) on the element's vertices in order, |n_e| = |(v0 - v2) x
    (v1 - v2)| (MATLAB/invrS.m:54-65; CUDA/invr.cuh:590-624)."""
    P = _soa(nodes)
    E = np.asarray(elems, dtype=np.int64)
    rule = np.asarray(regular, dtype=np.float64)
    N = np.stack([rule[:, 0], rule[:, 1], 1.0 - rule[:, 0] - rule[:, 1]])
    Me = (N * rule[:, 2]) @ N.T
    v = P[:, E]                                    # (3 coords, 3 slots, n)
    an = np.linalg.norm(np.cross((v[:, 0] - v[:, 2]).T, (v[:, 1] - v[:, 2]).T), axis=1)
    m = P.shape[1]
    G = np.zeros((m, m))
    for a in range(3):
        for b in range(3):
            np.add.at(G, (E[a], E[b]), an * Me[a, b])
    return G


def bem_modes(nodes, elems, mics, k, regular, singular, c, rho, nmodes):
    """invrS.m:159-169: Z = A \\ B, R = real(G Z), [U, ~] = svd(R),
    U_r = U(:, 1:n_ma), H_r = (A_hs Z - B_hs) U_r, and the modal surface
    pressures Z U_r.  Returns (s_r, U_r, H_r, P_r, Z, G); each column of U_r
    has its first component within 1e-6 of the largest magnitude positive,
    the sign convention of the device path."""
    Z, H = ibem(nodes, elems, mics, k, regular, singular, c, rho)
    G = mass_matrix(nodes, elems, regular)
    R = (G @ Z).real
    U, s, _ = np.linalg.svd(R)
    Ur = U[:, :nmodes].copy()
    for j in range(nmodes):
        a = np.abs(Ur[:, j])
        i = int(np.argmax(a >= a.max() * (1.0 - 1e-6)))
        if Ur[i, j] < 0:
            Ur[:, j] = -Ur[:, j]
    return s[:nmodes].copy(), Ur, H @ Ur, Z @ Ur, Z, G


def bem_modes_complex(nodes, elems, mics, k, regular, singular, c, rho, nmodes, chief=None):
    """The C++ invr()/invrgpu() form (CUDA/invr.cuh:392-440, 860-907): U from
    the SVD of the complex G Z, h = (A_hs Z - B_hs) U(:, 1:n), m_e = Z U(:, 1:n).
    Each column's phase is fixed so that its first component within 1e-6 of
    the largest magnitude is real and positive.  Returns (s, U, h, m_e, Z, G)."""
    Z, H = ibem(nodes, elems, mics, k, regular, singular, c, rho, chief)
    G = mass_matrix(nodes, elems, regular)
    U, s, _ = np.linalg.svd(G @ Z)
    U = U[:, :nmodes].copy()
    for j in range(nmodes):
        a = np.abs(U[:, j])
        i = int(np.argmax(a >= a.max() * (1.0 - 1e-6)))
        U[:, j] *= np.conj(U[i, j]) / a[i]
    return s[:nmodes].copy(), U, H @ U, Z @ U, Z, G


# ---------------------------------------------------------------------------
# products and sound power (CUDA/utils.cuh:199-289)
# ---------------------------------------------------------------------------
def to_pressure(Me, x):
    return Me @ x


def to_velocity(Qe, x):
    return Qe @ x


def sound_power(p, v, s):
    """W = 1/2 Re(v^H p) S/m (CUDA/utils.cuh:279-280)."""
    return 0.5 * float(np.real(np.vdot(v, p))) * (s / p.size)


# ---------------------------------------------------------------------------
# regularisation  (CUDA/tsvd.cuh; MATLAB/regtools)
# ---------------------------------------------------------------------------
def csvd(A):
    """Compact SVD A = U diag(s) V^H, descending s (csvdG.m:17-24)."""
    A = np.asarray(A)
    m, n = A.shape
    if m >= n:
        U, s, Vh = np.linalg.svd(A, full_matrices=False)
        return U, s, Vh.conj().T
    V, s, Uh = np.linalg.svd(A.conj().T, full_matrices=False)
    return Uh.conj().T, s, V


def tsvd(U, s, V, b, k):
    """x_k = V(:,1:k) diag(1/s(1:k)) U(:,1:p)^H b (tsvdG.m:20-23,
    tsvd.cuh:151-154).  Raises for k outside [1, p] (tsvd.cuh:124)."""
    p = s.size
    if k < 1 or k > p:
        raise ValueError("k out of range")
    beta = U[:, :p].conj().T @ b
    return V[:, :k] @ (beta[:k] / s[:k])


def tikhonov(U, s, V, b, lam):
    """x = V (s beta / (s^2 + lam^2)) (tikhonovG.m:26-30)."""
    if lam < 0:
        raise ValueError("lambda must be >= 0")
    beta = U[:, :s.size].conj().T @ b
    return V[:, :s.size] @ (s * beta / (s * s + lam * lam))


def gcv_grid(s, npoints=200, grid=None):
    """Descending lambda grid: regtools' from s_1 down to max(s_p, 16 eps s_1)
    (gcvG.m:28-30), or a fixed (lo, hi) log-spaced grid."""
    if grid is None:
        rpm = max(s[-1], s[0] * 16 * EPS)
        ratio = (s[0] / rpm) ** (1.0 / (npoints - 1))
        return ratio ** np.arange(npoints - 1, -1, -1) * rpm
    lo, hi = grid
    t = np.arange(npoints) / (npoints - 1)
    return np.exp(math.log(hi) + t * (math.log(lo) - math.log(hi)))


def _gcv_terms(s, b2, delta0, dof, lam, mode):
    if mode == "reference":
        f = lam * lam / (s + lam * lam)            # gcvG.m:47
    else:
        f = lam * lam / (s * s + lam * lam)        # Hansen's Tikhonov filter
    num = float(np.sum(f * f * b2) + delta0)
    den = dof + float(np.sum(f))
    return num, den, f


def gcv_function(s, beta, lam, m, delta0=0.0, mode="standard"):
    b2 = np.abs(beta) ** 2
    num, den, _ = _gcv_terms(s, b2, delta0, m - s.size, lam, mode)
    return num / (den * den)


def gcv_delta0(b, beta, m, p):
    """Intrinsic residual ||b||^2 - ||beta||^2 when m > p (gcvG.m:26,32-35)."""
    d = float(np.vdot(b, b).real - np.vdot(beta, beta).real)
    return d if (m > p and d > 0) else 0.0


GCV_BISECT_ITERS = 64


def gcv(U, s, b, npoints=200, grid=None, mode="standard"):
    """lambda minimising GCV.  Grid search as gcvG.m:28-42, then on the
    bracket [lam_{i+1}, lam_{i-1}] around the grid minimum:
      standard  -- the zero of dG/dlog(lam) by 64 bisection steps in log(lam)
                   (G = (sum f^2|beta|^2 + delta0) / ((m-p) + sum f)^2,
                   f = lam^2/(s^2+lam^2)); the endpoint if G is monotone there;
      reference -- gcvG.m exactly: grid filter lam/(s+lam) (:38), objective
                   filter lam^2/(s+lam^2) (:47), Brent's fminbnd (:51)."""
    m = U.shape[0]
    p = s.size
    beta = U[:, :p].conj().T @ b
    delta0 = gcv_delta0(b, beta, m, p)
    return gcv_from_beta(s, beta, m, delta0, npoints, grid, mode)


def gcv_from_beta(s, beta, m, delta0, npoints=200, grid=None, mode="standard"):
    p = s.size
    b2 = np.abs(beta) ** 2
    lam = gcv_grid(s, npoints, grid)
    dof = m - p
    G = np.empty(npoints)
    for j in range(npoints):
        if mode == "reference":
            f = lam[j] / (s + lam[j])                  # gcvG.m:38
            num = float(np.sum(f * f * b2) + delta0)
            den = dof + float(np.sum(f))
        else:
            num, den, _ = _gcv_terms(s, b2, delta0, dof, lam[j], mode)
        G[j] = num / (den * den)
    jmin = int(np.argmin(G))
    lo = lam[min(jmin + 1, npoints - 1)]
    hi = lam[max(jmin - 1, 0)]
    if mode == "reference":
        fun = lambda la: gcv_function(s, beta, la, m, delta0, "reference")  # noqa: E731
        return fminbnd(fun, lo, hi)
    return _gcv_bisect(s, b2, delta0, dof, lo, hi)


def _gcv_slope_sign_term(s, b2, delta0, dof, t):
    lam = math.exp(t)
    num, den, f = _gcv_terms(s, b2, delta0, dof, lam, "standard")
    dnum = 4.0 * float(np.sum(f * f * (1.0 - f) * b2))
    dden = 2.0 * float(np.sum(f * (1.0 - f)))
    return dnum * den - 2.0 * num * dden


def _gcv_bisect(s, b2, delta0, dof, lo, hi):
    a, b = math.log(lo), math.log(hi)
    if lo == hi:
        return lo
    if _gcv_slope_sign_term(s, b2, delta0, dof, a) >= 0.0:
        return lo
    if _gcv_slope_sign_term(s, b2, delta0, dof, b) <= 0.0:
        return hi
    for _ in range(GCV_BISECT_ITERS):
        mid = 0.5 * (a + b)
        if _gcv_slope_sign_term(s, b2, delta0, dof, mid) < 0.0:
            a = mid
        else:
            b = mid
    return math.exp(0.5 * (a + b))


def fminbnd(fun, ax, bx, tolx=1e-4, maxiter=500):
    """Brent's bounded minimiser (golden section + parabolic steps), with
    MATLAB fminbnd's tolerances: tol1 = sqrt(eps)|x| + tolx/3."""
    seps = math.sqrt(EPS)
    c = 0.5 * (3.0 - math.sqrt(5.0))
    a, b = ax, bx
    v = a + c * (b - a)
    w = xf = v
    d = e = 0.0
    fx = fun(xf)
    fv = fw = fx
    xm = 0.5 * (a + b)
    tol1 = seps * abs(xf) + tolx / 3.0
    tol2 = 2.0 * tol1
    it = 0
    while abs(xf - xm) > (tol2 - 0.5 * (b - a)) and it < maxiter:
        golden = True
        if abs(e) > tol1:
            golden = False
            r = (xf - w) * (fx - fv)
            q = (xf - v) * (fx - fw)
            p = (xf - v) * q - (xf - w) * r
            q = 2.0 * (q - r)
            if q > 0.0:
                p = -p
            q = abs(q)
            r = e
            e = d
            if abs(p) < abs(0.5 * q * r) and p > q * (a - xf) and p < q * (b - xf):
                d = p / q
                x = xf + d
                if (x - a) < tol2 or (b - x) < tol2:
                    si = 1.0 if (xm - xf) >= 0 else -1.0
                    d = tol1 * si
            else:
                golden = True
        if golden:
            e = (a - xf) if xf >= xm else (b - xf)
            d = c * e
        si = 1.0 if d >= 0 else -1.0
        x = xf + si * max(abs(d), tol1)
        fu = fun(x)
        it += 1
        if fu <= fx:
            if x >= xf:
                a = xf
            else:
                b = xf
            v, fv = w, fw
            w, fw = xf, fx
            xf, fx = x, fu
        else:
            if x < xf:
                a = x
            else:
                b = x
            if fu <= fw or w == xf:
                v, fv = w, fw
                w, fw = x, fu
            elif fu <= fv or v == xf or v == w:
                v, fv = x, fu
        xm = 0.5 * (a + b)
        tol1 = seps * abs(xf) + tolx / 3.0
        tol2 = 2.0 * tol1
    return xf


def solve_tikhonov_gcv(H, b, npoints=200, grid=None, mode="standard"):
    """The per-frequency inverse step: csvd, GCV lambda, Tikhonov x."""
    U, s, V = csvd(H)
    lam = gcv(U, s, b, npoints, grid, mode)
    return tikhonov(U, s, V, b, lam), lam, s


# ---------------------------------------------------------------------------
# Differentiable ESM array design (no reference code; the forward operator is
# the plain monopole G of esmV.m:29-30, the inverse tikhonovG.m:26-30 in its
# data-space form).  FP64 reference loss and analytic gradient.
# ---------------------------------------------------------------------------
def esm_design_solve(mics, surface, retreat, k, lam, q, noise=None):
    """One frequency: G, p = G q (+ noise), y = (G G^H + lam^2 I)^-1 p,
    q^ = G^H y.  q (m, R).  Returns (G, y, qhat)."""
    src = retreat_sources(surface, retreat)
    G = monopole_matrix(mics, src, k)
    p = G @ q
    if noise is not None:
        p = p + noise
    K = G @ G.conj().T + lam * lam * np.eye(G.shape[0])
    y = np.linalg.solve(K, p)
    return G, y, G.conj().T @ y


def esm_design_terms(mics, surface, retreat, k, loglam, q, noise=None):
    """Relative reconstruction errors ||q^ - q|| / ||q|| per (frequency,
    field): k, loglam (F,), q (F, m, R), noise (F, l, R) or None -> (F, R)."""
    F, R = q.shape[0], q.shape[2]
    out = np.zeros((F, R))
    for f in range(F):
        nz = None if noise is None else noise[f]
        _, _, qh = esm_design_solve(mics, surface, retreat, k[f], math.exp(loglam[f]), q[f], nz)
        out[f] = np.linalg.norm(qh - q[f], axis=0) / np.linalg.norm(q[f], axis=0)
    return out


def esm_design_loss(mics, surface, retreat, k, loglam, q, noise=None):
    """Mean relative reconstruction error over frequencies and fields."""
    return float(esm_design_terms(mics, surface, retreat, k, loglam, q, noise).mean())


def esm_design_grad(mics, surface, retreat, k, loglam, q, noise=None):
    """Gradient of esm_design_loss by the adjoint of the Tikhonov solve:
    with e = q^ - q, g = e / (||e|| ||q|| F R), z = K^-1 G g, w = g - G^H z,
    dL = Re sum_ij A_ij dG_ij - 2 lam^2 Re(z^H y) dloglam,
    A_ij = sum_r conj(y_ir) w_jr - conj(z_ir) e_jr,
    dG_ij = G_ij (ik - 1/r_ij) dr_ij.  Returns (dL/dmics (3, l), dL/dretreat,
    dL/dloglam (F,))."""
    M = _soa(mics)
    S = _soa(surface)
    unit = S / np.linalg.norm(S, axis=0)
    src = retreat_sources(surface, retreat)
    F, R = q.shape[0], q.shape[2]
    gm = np.zeros_like(M)
    gd = 0.0
    gl = np.zeros(F)
    for f in range(F):
        lam = math.exp(loglam[f])
        nz = None if noise is None else noise[f]
        G, y, qh = esm_design_solve(mics, surface, retreat, k[f], lam, q[f], nz)
        K = G @ G.conj().T + lam * lam * np.eye(G.shape[0])
        e = qh - q[f]
        g = e / (np.linalg.norm(e, axis=0) * np.linalg.norm(q[f], axis=0) * F * R)
        z = np.linalg.solve(K, G @ g)
        w = g - G.conj().T @ z
        A = y.conj() @ w.T - z.conj() @ e.T
        D = M[:, :, None] - src[:, None, :]                  # (3, l, m)
        r = np.sqrt((D * D).sum(0))
        c = np.real(A * G * (1j * k[f] - 1.0 / r)) / r
        gm += (c[None] * D).sum(2)
        gd += float((c[None] * D * unit[:, None, :]).sum())
        gl[f] = -2.0 * lam * lam * float(np.real(np.sum(z.conj() * y)))
    return gm, gd, gl


# ---------------------------------------------------------------------------
# gmsh v2.2 reader (CUDA/utils.cuh:291-382)
# ---------------------------------------------------------------------------
def read_msh(path, k, t):
    """Nodes (3, m), field points (3, m) = nodes (1 + 2 pi t / k), triangles
    (3, n) 0-based: element type 2 whose three vertices differ, in file order
    (utils.cuh:331-357; the tag count is read from the line, the reference
    assumes two)."""
    lines = open(path).read().splitlines()
    i = lines.index("$Nodes")
    m = int(lines[i + 1])
    nodes = np.array([[float(v) for v in lines[i + 2 + j].split()[1:4]] for j in range(m)]).T
    j = lines.index("$Elements")
    ne = int(lines[j + 1])
    tris = []
    for line in lines[j + 2:j + 2 + ne]:
        f = [int(v) for v in line.split()]
        if f[1] != 2:
            continue
        v = f[3 + f[2]:6 + f[2]]
        v = [x - 1 for x in v]
        if v[0] != v[1] and v[0] != v[2] and v[1] != v[2]:
            tris.append(v)
    elems = np.array(tris, dtype=np.int32).T.reshape(3, -1)
    scale = 1.0 + (2.0 * math.pi / k) * t
    return np.ascontiguousarray(nodes), np.ascontiguousarray(nodes * scale), np.ascontiguousarray(elems)


def write_msh(path, nodes, elems, extra_points=0, degenerate=0):
    """gmsh v2.2 ASCII file of the mesh (test input generator): optional point
    elements (type 15) and degenerate triangles to exercise the filter."""
    m, n = nodes.shape[1], elems.shape[1]
    rows = []
    for p in range(extra_points):
        rows.append(f"15 2 0 {p + 1} {p + 1}")
    for e in range(n):
        a, b, c = (int(x) + 1 for x in elems[:, e])
        rows.append(f"2 2 0 1 {a} {b} {c}")
        if e < degenerate:
            rows.append(f"2 2 0 1 {a} {a} {c}")
    with open(path, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % m)
        for j in range(m):
            fh.write("%d %.17g %.17g %.17g\n" % (j + 1, nodes[0, j], nodes[1, j], nodes[2, j]))
        fh.write("$EndNodes\n$Elements\n%d\n" % len(rows))
        for i, r in enumerate(rows):
            fh.write(f"{i + 1} {r}\n")
        fh.write("$EndElements\n")


# ---------------------------------------------------------------------------
# Other lambda selectors and the damped SVD (MATLAB/regtools/l_curveG.m,
# lcfunG.m, quasioptG.m, dsvdG.m), filter 't' (Tikhonov) or 'd' (damped SVD)
# ---------------------------------------------------------------------------
def _filter(s, lam, method):
    return s / (s + lam) if method == "d" else s * s / (s * s + lam * lam)


def lcfun(lam, s, beta, xi, method, rho_ls2=0.0):
    """Negative curvature of the L-curve at lam (lcfunG.m:12-49)."""
    f = _filter(s, lam, method)
    cf = 1.0 - f
    xx, bb = np.abs(xi) ** 2, np.abs(beta) ** 2
    eta = math.sqrt(float(np.sum(f * f * xx)))
    rho = math.sqrt(float(np.sum(cf * cf * bb)) + rho_ls2)
    f1 = -2.0 * f * cf / lam
    f2 = -f1 * (3.0 - 4.0 * f) / lam
    phi = float(np.sum(f * f1 * xx))
    psi = float(np.sum(cf * f1 * bb))
    dphi = float(np.sum((f1 ** 2 + f * f2) * xx))
    dpsi = float(np.sum((-f1 ** 2 + cf * f2) * bb))
    deta, drho = phi / eta, -psi / rho
    ddeta = dphi / eta - deta * (deta / eta)
    ddrho = -dpsi / rho - drho * (drho / rho)
    dle, dlr = deta / eta, drho / rho
    ddle, ddlr = ddeta / eta - dle ** 2, ddrho / rho - dlr ** 2
    return -(dlr * ddle - ddlr * dle) / (dlr ** 2 + dle ** 2) ** 1.5


def l_curve(U, s, b, method="t", npoints=200):
    """L-curve corner (l_curveG.m:21-53): grid from s_1 down to
    max(s_p, 16 eps s_1), grid minimum of the negative curvature, fminbnd on
    the neighbouring grid points; the least-squares residual enters when m > p."""
    m = U.shape[0]
    p = s.size
    beta = U[:, :p].conj().T @ b
    rho_ls2 = gcv_delta0(b, beta, m, p)
    with np.errstate(divide="ignore", invalid="ignore"):
        xi = np.where(s > 0, beta / np.where(s > 0, s, 1.0), 0.0)
    lam = gcv_grid(s, npoints)
    g = np.array([lcfun(la, s, beta, xi, method, rho_ls2) for la in lam])
    gi = int(np.nanargmin(g))
    return fminbnd(lambda la: lcfun(la, s, beta, xi, method, rho_ls2), lam[min(gi + 1, npoints - 1)],
                   lam[max(gi - 1, 0)])


def quasiopt(U, s, b, method="t", npoints=200):
    """Quasi-optimality lambda (quasioptG.m:17-41): Q = ||(1-f) f xi|| on the
    grid from s_1 down to s_p, then fminbnd around the grid minimum."""
    p = s.size
    xi = (U[:, :p].conj().T @ b) / s
    rpm = s[-1] if s[-1] > 0 else s[0] * 16 * EPS
    ratio = (s[0] / rpm) ** (1.0 / (npoints - 1))
    lam = ratio ** np.arange(npoints - 1, -1, -1) * rpm

    def Q(la):
        f = _filter(s, la, method)
        return float(np.linalg.norm((1.0 - f) * f * xi))

    q = np.array([Q(la) for la in lam])
    qi = int(np.nanargmin(q))
    return fminbnd(Q, lam[min(qi + 1, npoints - 1)], lam[max(qi - 1, 0)])


def dsvd(U, s, V, b, lam):
    """Damped SVD x = V (beta / (s + lambda)) (dsvdG.m:21-26)."""
    if lam < 0:
        raise ValueError("Illegal regularization parameter lambda")
    p = s.size
    beta = U[:, :p].conj().T @ b
    return V[:, :p] @ (beta / (s + lam))


def solve_regularized(H, b, method, npoints=200, lam_fixed=None):
    """csvd, then the filter and lambda of the library's IA_METHOD_* names:
    'tikhonov-lcurve', 'tikhonov-quasiopt', 'dsvd-fixed', 'dsvd-lcurve',
    'dsvd-quasiopt'.  Returns (x, lambda, s)."""
    U, s, V = csvd(H)
    filt, sel = method.split("-")
    m = "d" if filt == "dsvd" else "t"
    if sel == "lcurve":
        lam = l_curve(U, s, b, m, npoints)
    elif sel == "quasiopt":
        lam = quasiopt(U, s, b, m, npoints)
    else:
        lam = lam_fixed
    x = dsvd(U, s, V, b, lam) if m == "d" else tikhonov(U, s, V, b, lam)
    return x, lam, s


# ---------------------------------------------------------------------------
# ADMM  (MATLAB/ADMMG.m:1-90)
# ---------------------------------------------------------------------------
def admm_x0(A, b):
    """The starting point x = A \\ b (ADMMG.m:6,32,50): the least-squares
    solution for square and tall A; for wide A the minimum-norm solution
    (MATLAB's backslash returns a basic solution there, which depends on its
    column pivoting)."""
    l, m = A.shape
    if l >= m:
        return np.linalg.lstsq(A, b, rcond=None)[0]
    Q, R = np.linalg.qr(A.conj().T)
    return Q @ np.linalg.solve(R.conj().T, b)


def admm_gst_threshold(lam_p, p):
    """tpgst of ADMMG.m:59, the generalised soft-threshold of |y|."""
    t = 2.0 * lam_p * (1.0 - p)
    return t ** (1.0 / (2.0 - p)) + lam_p * p * t ** ((p - 1.0) / (2.0 - p))


def admm(A, b, lambda_0, rho, gamma, epsilon, Nm, nor, p=None, N=None, x0=None):
    """ADMMG.m:1-90, one right-hand side.  nor 1: L1 (soft threshold,
    continuation lambda = 5 lambda_0 * 0.75^j while above lambda_0 / 10);
    2: L2; 3: Lp (generalised soft threshold, N fixed-point steps).  Every
    c-update solves (2 A^H A + rho I) c = 2 A^H b + rho x - u; the first time
    all three of ||c - c_old||, ||c - x||, ||u - u_old|| are <= epsilon ends
    the whole run.  Returns (c, iterations, converged)."""
    A = np.asarray(A, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    n = A.shape[1]
    x = admm_x0(A, b) if x0 is None else np.array(x0, dtype=np.complex128)
    aa21 = 2.0 * (A.conj().T @ A) + rho * np.eye(n)
    from scipy.linalg import lu_factor, lu_solve
    lu = lu_factor(aa21)          # aa21 \ (...) every iteration, factored once
    aa22 = 2.0 * (A.conj().T @ b)
    c = np.zeros(n, dtype=np.complex128)
    its = 0

    def conv(c, cold, x, u, uold):
        return (np.linalg.norm(c - cold) <= epsilon and np.linalg.norm(c - x) <= epsilon
                and np.linalg.norm(u - uold) <= epsilon)

    if nor == 2:
        u = np.zeros(n, dtype=np.complex128)
        dlr = 2.0 * lambda_0 + rho
        for _ in range(Nm):
            cold = c
            c = lu_solve(lu, aa22 + rho * x - u)
            its += 1
            x = (rho * c + u) / dlr
            uold = u
            u = u + gamma * rho * (c - x)
            if conv(c, cold, x, u, uold):
                return c, its, True
        return c, its, False
    lambda_e = lambda_0 / 10.0
    lam = lambda_0 * 5.0
    u = np.zeros(n, dtype=np.complex128) if nor == 1 else x.copy()
    while lam > lambda_e:
        if nor == 1:
            lr = lam / rho
        else:
            lam_p = 2.0 * lam / rho
            tau = admm_gst_threshold(lam_p, p)
        for _ in range(Nm):
            cold = c
            c = lu_solve(lu, aa22 + rho * x - u)
            its += 1
            y = c + u / rho
            ay = np.abs(y)
            if nor == 1:
                # max(0, |y| - lr) exp(i wrapTo2Pi(angle(y))), ADMMG.m:18
                x = np.maximum(0.0, ay - lr) * np.exp(1j * np.angle(y))
            else:
                keep = ~(ay <= tau)
                s = ay.astype(np.complex128)
                for _d in range(N):
                    s = ay - lam_p * p * np.power(s, complex(p - 1.0, 0.0))
                with np.errstate(invalid="ignore", divide="ignore"):
                    sgn = np.where(ay > 0, y / np.where(ay > 0, ay, 1.0), 0.0)
                x = sgn * s * keep
            uold = u
            u = u + gamma * rho * (c - x)
            if conv(c, cold, x, u, uold):
                return c, its, True
        lam = max(0.75 * lam, lambda_e)
    return c, its, False
