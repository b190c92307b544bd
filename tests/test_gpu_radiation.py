"""GPU suite: radiation modes of the baffled plate (sinc resistance matrix,
leading eigenpairs by subspace iteration, sound power, and the ESM/TSVD
velocity reconstruction of the plate workload) against the oracle (the C
sinc restatement, numpy eigh, the FP64 TSVD restatement).

Bounds: R entrywise 1e-13 of max |R|; eigenvalues 1e-12 lambda_1 (FP64 and
mixed); eigenvectors of well separated modes (lambda > 1e-8 lambda_1, gap >
1e-3 lambda_1) 1e-9 (FP64) / 1e-6 (mixed); sound power 1e-12 relative."""
import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu
C, RHO = 343.0, 1.21


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


@pytest.fixture(scope="module")
def plate():
    return g.radiation_plate(n_freq=256)


def test_sinc_resistance_matches_oracle(cuda, ctx, plate):
    """Evenly spaced block (phase recurrence) and scattered wavenumbers
    (direct sincos) against the oracle's sin(kr)/kr."""
    from inverseacoustics_gb300 import api
    import torch
    x, area = plate.arrays["centres"], plate.params["area"]
    for ks in (plate.k[:8], plate.k[[3, 100, 255]], plate.k[[0]]):
        R = api.sinc_resistance_batch(ctx, T(x, cuda), T(ks, cuda), area)
        torch.cuda.synchronize()
        R = R.cpu().numpy()
        for f, k in enumerate(ks):
            Ro = O.sinc_resistance(x, k, C, RHO, area)
            assert np.max(np.abs(R[f] - Ro)) <= 1e-13 * np.max(np.abs(Ro))
            assert np.array_equal(R[f], R[f].T)


def _check_modes(lam, modes, R, nm, vec_tol, res_tol):
    w, V = np.linalg.eigh(R)
    w, V = w[::-1], V[:, ::-1]
    lam1 = w[0]
    assert np.max(np.abs(lam - w[:nm])) <= 1e-12 * lam1
    X = modes.T                                         # n x nm
    assert np.max(np.abs(X.T @ X - np.eye(nm))) < 1e-12
    res = np.linalg.norm(R @ X - X * lam, axis=0)
    assert np.max(res) <= res_tol * lam1
    checked = 0
    for j in range(nm):
        if w[j] < 1e-8 * lam1:
            continue
        gap = min(w[j - 1] - w[j] if j > 0 else np.inf, w[j] - w[j + 1]) / lam1
        if gap < 1e-3:
            continue
        v = X[:, j] * np.sign(X[:, j] @ V[:, j])
        assert np.linalg.norm(v - V[:, j]) <= vec_tol, (j, w[j] / lam1)
        checked += 1
    # library sign convention: the first component within 1e-6 of the largest magnitude is positive
    for j in range(nm):
        a = np.abs(X[:, j])
        i = int(np.argmax(a >= a.max() * (1 - 1e-6)))
        assert X[i, j] > 0
    return checked


@pytest.mark.parametrize("precision", [0, 1])
def test_radiation_modes_match_eigh(cuda, ctx, plate, precision):
    from inverseacoustics_gb300 import api
    import torch
    x, area = plate.arrays["centres"], plate.params["area"]
    ks = 2 * np.pi * np.array([20.0, 200.0, 1000.0, 2000.0]) / C
    nm = 32
    R = api.sinc_resistance_batch(ctx, T(x, cuda), T(ks, cuda), area)
    lam, modes, info = api.radiation_modes_batch(ctx, R, nm, api.default_config(precision=precision))
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    lam, modes = lam.cpu().numpy(), modes.cpu().numpy()
    vec_tol, res_tol = (1e-9, 1e-12) if precision == 0 else (1e-6, 1e-8)
    checked = 0
    for f, k in enumerate(ks):
        Ro = O.sinc_resistance(x, k, C, RHO, area)
        checked += _check_modes(lam[f], modes[f], Ro, nm, vec_tol, res_tol)
    assert checked >= 20


def test_sound_power_matches_oracle(cuda, ctx, plate):
    from inverseacoustics_gb300 import api
    import torch
    x, area = plate.arrays["centres"], plate.params["area"]
    ks = plate.k[[10, 120, 250]]
    rng = np.random.default_rng(11)
    v = g.complex_normal(rng, (3, 5, x.shape[1]))
    v[:, 0] = plate.params["vel"][[10, 120, 250]]
    R = api.sinc_resistance_batch(ctx, T(x, cuda), T(ks, cuda), area)
    W = api.sound_power_batch(ctx, R, T(v, cuda))
    torch.cuda.synchronize()
    W = W.cpu().numpy()
    for f, k in enumerate(ks):
        Ro = O.sinc_resistance(x, k, C, RHO, area)
        for r in range(5):
            wo = O.sound_power_R(Ro, v[f, r])
            assert abs(W[f, r] - wo) <= 1e-12 * abs(wo)


def test_modal_sound_power(cuda, ctx, plate):
    """With nmodes past the numerical rank, 1/2 sum lambda_j |phi_j^T v|^2
    reproduces 1/2 v^H R v (mixed path)."""
    from inverseacoustics_gb300 import api
    import torch
    x, area = plate.arrays["centres"], plate.params["area"]
    idx = [0, 40, 80]                                   # 20, 329, 638 Hz
    ks = plate.k[idx]
    v = plate.params["vel"][idx][:, None, :]
    R = api.sinc_resistance_batch(ctx, T(x, cuda), T(ks, cuda), area)
    lam, modes, info = api.radiation_modes_batch(ctx, R, 64, api.default_config(precision=1))
    W = api.sound_power_batch(ctx, R, T(v, cuda))
    torch.cuda.synchronize()
    lam, modes, W = lam.cpu().numpy(), modes.cpu().numpy(), W.cpu().numpy()
    for f in range(len(ks)):
        y = modes[f] @ v[f, 0]
        wm = 0.5 * float(np.sum(lam[f] * np.abs(y) ** 2))
        assert abs(wm - W[f, 0]) <= 1e-10 * W[f, 0]


def test_plate_velocity_reconstruction(cuda, ctx, plate):
    """The plate workload end to end: microphone pressures from the Rayleigh
    integral of the modal velocity (+30 dB noise), ESM monopoles at the
    element centres, TSVD (FP64 and mixed) against the oracle's TSVD, then
    the sound power of the reconstruction."""
    from inverseacoustics_gb300 import api
    import torch
    x, area, mics = plate.arrays["centres"], plate.params["area"], plate.arrays["mics"]
    idx = [5, 60, 130, 250]
    ks = plate.k[idx]
    rng = np.random.default_rng(12)
    vel = plate.params["vel"][idx]
    p = np.stack([g.add_noise(rng, g.rayleigh_pressure(mics, x, area, k, vel[f], C, RHO), 30.0)[None, :]
                  for f, k in enumerate(ks)])
    kt = 36                          # s_36 / s_37 >= 1.11 at these bins
    q_ref = []
    for f, k in enumerate(ks):
        G = O.monopole_matrix(mics, x, k)
        U, s, V = O.csvd(G)
        q_ref.append(O.tsvd(U, s, V, p[f, 0], kt))
    R = api.sinc_resistance_batch(ctx, T(x, cuda), T(ks, cuda), area)
    for precision, tol in ((0, 1e-10), (1, 1e-6)):
        cfg = api.default_config(method=1, tsvd_k=kt, precision=precision)
        q, lam, s, info = api.esm_solve_batch(ctx, T(mics, cuda), T(x, cuda), T(ks, cuda), T(p, cuda), cfg)
        W = api.sound_power_batch(ctx, R, q)
        torch.cuda.synchronize()
        assert int(info.abs().sum()) == 0
        q, W = q.cpu().numpy(), W.cpu().numpy()
        for f, k in enumerate(ks):
            assert relerr(q[f, 0], q_ref[f]) < tol
            wo = O.sound_power_R(O.sinc_resistance(x, k, C, RHO, area), q_ref[f])
            assert abs(W[f, 0] - wo) <= 10 * tol * abs(wo)


def test_mixed_tsvd_symmetric_plate_all_bins(cuda, ctx, plate):
    """The full 192-microphone grid is symmetric about the plate centre, so
    G has near-equal singular pairs.  Mixed TSVD against the FP64 path at all
    256 bins: the pairs the first-order eigen-refinement cannot separate are
    rotated apart by the FP64 Jacobi on X^H E X."""
    from inverseacoustics_gb300 import api
    import torch
    x, area, mics = plate.arrays["centres"], plate.params["area"], plate.arrays["mics"]
    rng = np.random.default_rng(3)
    vel = plate.params["vel"]
    p = np.stack([g.add_noise(rng, g.rayleigh_pressure(mics, x, area, k, vel[f], C, RHO), 30.0)[None, :]
                  for f, k in enumerate(plate.k)])
    args = (T(mics, cuda), T(x, cuda), T(plate.k, cuda), T(p, cuda))
    q0, _, _, i0 = api.esm_solve_batch(ctx, *args, api.default_config(method=1, tsvd_k=36))
    q1, _, _, i1 = api.esm_solve_batch(ctx, *args, api.default_config(method=1, tsvd_k=36, precision=1))
    torch.cuda.synchronize()
    assert int(i0.abs().sum()) == 0 and int(i1.abs().sum()) == 0
    err = ((q1 - q0).abs().pow(2).sum((1, 2)).sqrt() / q0.abs().pow(2).sum((1, 2)).sqrt()).cpu().numpy()
    assert err.max() < 1e-8, (int(err.argmax()), float(err.max()))
