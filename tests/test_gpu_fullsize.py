"""GPU parity at the full sizes of the IBEM and HELS workloads, every bin.

IBEM sphere (642 nodes, 1280 triangles, 120 microphones, 64 bins 100-2000
Hz, the inputs the benchmark times): the FP64 path against the oracle (C
assembly, LU solve, Tikhonov-GCV), the reference's ibem() followed by
regtools' csvd/gcv/tikhonov (CUDA/ibem.cuh:424-770, MATLAB/regtools), and the
mixed path against the same oracle.

The oracle bins run on a spawn process pool while nothing else runs on the
host.  Every test prints its measured maximum errors."""
import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from oracle import cpu_pipeline as CP

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


@pytest.fixture(scope="module")
def ibem_case():
    w = g.ibem_sphere(n_freq=64)
    p = g.ibem_sphere_pressures(w)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    ref = CP.map_bins(CP.oracle_ibem_bin, [(nodes, elems, mics, w.k[f], p[f, 0]) for f in range(len(w.k))])
    return w, p, ref


def _errors(x, lam, ref):
    ex = [relerr(x[f, 0], ref[f][0]) for f in range(len(ref))]
    el = [abs(lam[f, 0] - ref[f][1]) / ref[f][1] for f in range(len(ref))]
    return np.array(ex), np.array(el)


def _ibem_run(ctx, cuda, w, p, precision):
    import torch
    from inverseacoustics_gb300 import api
    mesh = api.Mesh(ctx, w.arrays["nodes"], w.arrays["elems"])
    x, lam, s, info = api.ibem_solve_batch(ctx, mesh, T(w.arrays["mics"], cuda), T(w.k, cuda), T(p, cuda),
                                           api.default_config(precision=precision))
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0, info
    out = x.cpu().numpy(), lam.cpu().numpy()
    mesh.close()
    return out


def test_ibem_headline_fp64_every_bin_matches_oracle(cuda, ctx, ibem_case):
    w, p, ref = ibem_case
    x, lam = _ibem_run(ctx, cuda, w, p, 0)
    ex, el = _errors(x, lam, ref)
    print(f"\nIBEM FP64 vs oracle, 64 bins: x max {ex.max():.3e} (bin {ex.argmax()}), "
          f"lambda max {el.max():.3e} (bin {el.argmax()})")
    assert ex.max() < 1e-10
    assert el.max() < 1e-10


def test_ibem_headline_mixed_every_bin_matches_oracle(cuda, ctx, ibem_case):
    w, p, ref = ibem_case
    x, lam = _ibem_run(ctx, cuda, w, p, 1)
    ex, el = _errors(x, lam, ref)
    print(f"\nIBEM mixed vs oracle, 64 bins: x max {ex.max():.3e} (bin {ex.argmax()}), "
          f"lambda max {el.max():.3e} (bin {el.argmax()})")
    assert ex.max() < 1e-6
    assert el.max() < 1e-6


# --------------------------------------------------------------------------
# HELS plane (order 15: 256 terms, 256 microphones, 512 bins 50-3000 Hz, 40
# monopoles, 25 dB): both paths against the oracle (CUDA/hels.cuh:222-323,
# then csvd/gcv/tikhonov).  The lowest bin has kr = 0.137 at the nearest
# microphone, where h_15 is ~1e30: the operators' singular values span 17
# decades (s_p / s_1 ~ 1e-17) and GCV's lambda falls as low as 1e-14 s_1 --
# at FP64 rounding level.  Parity therefore has three tiers:
#  * every bin: no info flag; s within 1e-13 s_1 of LAPACK's; (x, lambda)
#    solves the Tikhonov normal equations (H^H H + lambda^2 I) x = H^H b to
#    within max(1e-12, 100 eps kappa) relative to s_1^2 |x| + s_1 |b|.  The
#    kappa = s_1 / lambda factor is the data-space form's: x = H^H w with
#    w = U (S^2 + lambda^2)^-1 U^H b leaves the residual H^H E w, E ~ eps s_1^2
#    the eigen-decomposition's backward error, |w| ~ |b| / lambda^2 (LAPACK's
#    V-space form has O(eps) here; both have forward errors O(eps kappa));
#  * every bin whose GCV choice the arithmetic determines -- LAPACK's gesdd
#    and gesvd drivers agree on lambda to 1e-8, and the GCV minimum beats the
#    best grid value in the rounding region (lambda < 1e3 16 eps s_1) by 1.5x
#    -- x and lambda within max(1e-10, 100 eps kappa) of the oracle, kappa =
#    s_1 / lambda (the Tikhonov solution's own sensitivity to rounding);
#  * the remaining bins (GCV's choice decided by rounding: the two LAPACK
#    drivers already disagree there) are held to the first tier only.
EPS = np.finfo(float).eps


def _hels_oracle_bin(args):
    import scipy.linalg as sl
    from oracle import ia_oracle as O
    pts, k, order, b = args
    _, He, _ = O.hels(pts, pts, k, order, 343.0, 1.21)
    U, s, V = O.csvd(He)
    lam = O.gcv(U, s, b)
    x = O.tikhonov(U, s, V, b, lam)
    U2, s2, _ = sl.svd(He, lapack_driver="gesvd")
    lam2 = O.gcv(U2, s2, b)
    beta = U.conj().T @ b
    grid = O.gcv_grid(s, 200, None)
    G = np.array([O.gcv_function(s, beta, la, He.shape[0], 0.0, "standard") for la in grid])
    rnd = grid < 1e3 * 16 * EPS * s[0]
    margin = G[rnd].min() / G.min() if rnd.any() else np.inf
    determined = abs(lam - lam2) <= 1e-8 * lam and margin > 1.5
    return x, lam, s, determined


@pytest.fixture(scope="module")
def hels_case():
    w = g.hels_plane(n_freq=512)
    p = g.hels_plane_pressures(w)
    pts = g.cartesian_to_spherical(w.arrays["mics"])
    order = w.params["order"]
    ref = CP.map_bins(_hels_oracle_bin, [(pts, w.k[f], order, p[f, 0]) for f in range(len(w.k))])
    return w, pts, p, ref


def _hels_backward(args):
    """Relative residual of the Tikhonov normal equations for (x, lambda)."""
    from oracle import ia_oracle as O
    pts, k, order, b, x, lam = args
    _, H, _ = O.hels(pts, pts, k, order, 343.0, 1.21)
    s1 = np.linalg.norm(H, 2)
    r = H.conj().T @ (H @ x - b) + lam * lam * x
    return np.linalg.norm(r) / (s1 * s1 * np.linalg.norm(x) + s1 * np.linalg.norm(b))


def _hels_check(w, pts, p, ref, x, lam, s, info, label, mixed_bins=None):
    """The three tiers over the bins the FP64 arithmetic produced; bins left on
    the mixed path (mixed_bins) are checked by the caller instead."""
    F = len(w.k)
    fp64_bins = np.ones(F, bool) if mixed_bins is None else ~mixed_bins
    flagged = np.nonzero(info)[0]
    assert len(flagged) == 0, f"{label}: info flags at bins {flagged[:16]}"
    s_or = np.array([r[2] for r in ref])
    ds = (np.abs(s - s_or).max(axis=1) / s_or[:, 0])
    order = w.params["order"]
    back = np.array(CP.map_bins(_hels_backward, [(pts, w.k[f], order, p[f, 0], x[f, 0], lam[f, 0])
                                                 for f in range(F)]))
    back_bound = np.maximum(1e-12, 100 * EPS * s_or[:, 0] / lam[:, 0])
    det = np.array([r[3] for r in ref]) & fp64_bins
    lam_or = np.array([r[1] for r in ref])
    kappa = s_or[:, 0] / lam_or
    ex = np.array([relerr(x[f, 0], ref[f][0]) for f in range(F)])
    el = np.abs(lam[:, 0] - lam_or) / lam_or
    bound = np.maximum(1e-10, 100 * EPS * kappa)
    r = np.linalg.norm(w.arrays["mics"], axis=0).min()
    print(f"\nHELS N={w.params['order']} {label}, {F} bins (kr {w.k[0] * r:.3f}..{w.k[-1] * r:.2f}): "
          f"{fp64_bins.sum()} FP64 bins: s max {ds[fp64_bins].max():.2e} s_1, normal-equation residual max "
          f"{back[fp64_bins].max():.2e} ({(back / back_bound)[fp64_bins].max():.3f} of its bound; "
          f"{int((back[fp64_bins] < 1e-12).sum())} bins below 1e-12); "
          f"{det.sum()} determined bins: x max {ex[det].max():.2e}, lambda max {el[det].max():.2e}, "
          f"max err / bound {max((ex / bound)[det].max(), (el / bound)[det].max()):.3f}; "
          f"bins with x, lambda within 1e-10: {int(((ex < 1e-10) & (el < 1e-10)).sum())}")
    assert ds[fp64_bins].max() < 1e-13
    assert (back[fp64_bins] < back_bound[fp64_bins]).all()
    assert (ex[det] < bound[det]).all()
    assert (el[det] < bound[det]).all()
    return ex, el, ds


def _hels_run(ctx, cuda, w, pts, p, precision, fallback=1):
    import torch
    from inverseacoustics_gb300 import _lib, api
    x, lam, s, info = api.hels_solve_batch(ctx, T(pts, cuda), w.params["order"], T(w.k, cuda), T(p, cuda),
                                           api.default_config(precision=precision, mixed_fallback=fallback))
    torch.cuda.synchronize()
    fb = _lib.lib().ia_last_fallback_bins(ctx.handle)
    return x.cpu().numpy(), lam.cpu().numpy(), s.cpu().numpy(), info.cpu().numpy(), fb


def test_hels_full_size_fp64_matches_oracle(cuda, ctx, hels_case):
    w, pts, p, ref = hels_case
    x, lam, s, info, fb = _hels_run(ctx, cuda, w, pts, p, 0)
    assert fb == 0
    _hels_check(w, pts, p, ref, x, lam, s, info, "FP64")


def test_hels_full_size_mixed_matches_oracle(cuda, ctx, hels_case):
    """Mixed path.  With the fallback off, the bins that pass its precision
    guard (info 0) must be within 1e-6 of the oracle.  With it on (the
    default), every bin meets the FP64 tiers: the failing bins are solved again
    (FP64, or for a failed trace check first the mixed path with more
    refinement steps).  On this workload almost no bin passes: lambda is
    below 1e-3 s_1 in all but the 32 lowest bins, and there (lambda = s_1, 17
    decades of singular values) the Gram eigensolver loses the spectrum."""
    w, pts, p, ref = hels_case
    x0, lam0, s0, info0, _ = _hels_run(ctx, cuda, w, pts, p, 1, fallback=0)
    passed = info0 == 0
    ex0 = np.array([relerr(x0[f, 0], ref[f][0]) for f in range(len(w.k))])
    el0 = np.array([abs(lam0[f, 0] - ref[f][1]) / ref[f][1] for f in range(len(w.k))])
    s1 = np.array([r[2][0] for r in ref])
    ds0 = np.array([np.abs(s0[f] - ref[f][2]).max() / s1[f] for f in range(len(w.k))])
    pb = passed
    print(f"\nHELS mixed, fallback off: {pb.sum()} bins pass the guard: x max "
          f"{ex0[pb].max() if pb.any() else 0:.2e}, lambda max {el0[pb].max() if pb.any() else 0:.2e}, "
          f"s max {ds0[pb].max() if pb.any() else 0:.2e} s_1; flags {sorted(set(info0.tolist()))}")
    # the mixed eigensolver's s: eigenvalues of H H^H to ~eps s_1^2, so s_i to
    # ~sqrt(eps) s_1 at worst (the smallest)
    assert (ex0[pb] < 1e-6).all() and (el0[pb] < 1e-6).all() and (ds0[pb] < 1e-7).all()
    x, lam, s, info, fb = _hels_run(ctx, cuda, w, pts, p, 1)
    assert fb == int((~passed).sum())
    _hels_check(w, pts, p, ref, x, lam, s, info, f"mixed ({fb} bins solved again)", passed)


# --------------------------------------------------------------------------
# Plate workload (config 4): the ESM velocity reconstruction by TSVD (k = 36)
# from 192 microphones at 0.05 m, 1280 sources, 256 bins 20-2000 Hz.  The
# symmetric array gives near-degenerate singular pairs; at a few bins the
# mixed eigensolver's two Ogita-Aishima steps leave a pair unsettled (s_1 off
# by up to 7e-6 s_1), which its trace check catches (IA_INFO_UNRESOLVED); the
# fallback solves those bins again on the mixed path with three steps.
def test_plate_tsvd_mixed_guard_and_retry(cuda, ctx):
    import torch
    from inverseacoustics_gb300 import _lib, api
    from oracle import ia_oracle as O
    w = g.radiation_plate(n_freq=256)
    x, area, mics = w.arrays["centres"], w.params["area"], w.arrays["mics"]
    rng = np.random.default_rng(3)
    p = np.stack([g.add_noise(rng, g.rayleigh_pressure(mics, x, area, k, w.params["vel"][f]), 30.0)[None, :]
                  for f, k in enumerate(w.k)])
    args = (T(mics, cuda), T(x, cuda), T(w.k, cuda), T(p, cuda))
    so = np.array([np.linalg.svd(O.monopole_matrix(mics, x, k), compute_uv=False)[:36] for k in w.k])

    def run(prec, fallback):
        q, lam, s, info = api.esm_solve_batch(ctx, *args, api.default_config(method=1, tsvd_k=36, precision=prec,
                                                                             mixed_fallback=fallback))
        torch.cuda.synchronize()
        return q.cpu().numpy(), s.cpu().numpy()[:, :36], info.cpu().numpy(), _lib.lib().ia_last_fallback_bins(ctx.handle)

    q0, s0, info0, _ = run(1, 0)
    flagged = np.nonzero(info0)[0]
    es0 = np.abs(s0 - so).max(axis=1) / so[:, 0]
    q, s, info, fb = run(1, 1)
    q64, _, info64, _ = run(0, 1)
    es = np.abs(s - so).max(axis=1) / so[:, 0]
    eq = np.array([relerr(q[f], q64[f]) for f in range(len(w.k))])
    print(f"\nplate TSVD, 256 bins: {len(flagged)} bins flagged {sorted(set(info0[flagged].tolist()))} (s_1..36 "
          f"error there {es0[flagged].max() if len(flagged) else 0:.1e} s_1, elsewhere {np.delete(es0, flagged).max():.1e}); "
          f"after the retry: s_1..36 {es.max():.1e} s_1, x vs FP64 {eq.max():.1e}")
    assert (info0[flagged] == _lib.IA_INFO_UNRESOLVED).all()
    assert np.delete(es0, flagged).max() < 1e-7
    assert fb == len(flagged)
    assert int(np.abs(info).sum()) == 0 and int(np.abs(info64).sum()) == 0
    assert es.max() < 1e-7 and eq.max() < 1e-6
