"""GPU suite: ADMM inversion (ia_admm_batch) against the oracle's restatement
of MATLAB/ADMMG.m, all three norms, wide (dual / Woodbury form, one CTA and
thread-block clusters) and tall (primal form) systems.

Bounds.  With epsilon = 0 every run takes the same number of iterations on
both sides and c agrees to 1e-10 relative in FP64, 1e-9 with double-float
products (the c-update inverse is formed once and applied as a product here,
solved every iteration in the oracle); with a finite epsilon the iteration
counts agree exactly and c to 1e-9 (FP64) / 1e-8 (double-float)."""
import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


def _problems(seed, F, nrhs, l, m, k=4, noise=1e-3):
    rng = np.random.default_rng(seed)
    A = (rng.normal(size=(F, l, m)) + 1j * rng.normal(size=(F, l, m))) / np.sqrt(l)
    X = np.zeros((F, nrhs, m), complex)
    for f in range(F):
        for r in range(nrhs):
            idx = rng.choice(m, k, replace=False)
            X[f, r, idx] = rng.normal(size=k) + 1j * rng.normal(size=k)
    B = np.einsum("flm,frm->frl", A, X) + noise * (rng.normal(size=(F, nrhs, l)) + 1j * rng.normal(size=(F, nrhs, l)))
    lam0 = 0.2 + 0.6 * rng.random((F, nrhs))
    return A, B, lam0


def _run(ctx, cuda, A, B, lam0, acfg, x0=None):
    from inverseacoustics_gb300 import api
    import torch
    H = T(np.ascontiguousarray(A.transpose(0, 2, 1)), cuda)     # (F, m, l): column-major l x m
    c, its, info = api.admm_batch(ctx, H, T(B, cuda), T(lam0, cuda), acfg, x0=None if x0 is None else T(x0, cuda))
    torch.cuda.synchronize()
    return c.cpu().numpy(), its.cpu().numpy(), info.cpu().numpy()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("norm", [1, 2, 3])
@pytest.mark.parametrize("shape", [(24, 80), (40, 16), (32, 300), (120, 642)])
def test_admm_fixed_iterations_match_oracle(cuda, ctx, norm, shape, precision):
    """epsilon = 0: MATLAB's loops run to the end (14 continuation stages x
    Nm for L1 / Lp, Nm for L2).  (120, 642) is the benchmark's shape (clusters
    of 4 CTAs)."""
    from inverseacoustics_gb300 import api
    l, m = shape
    F, nrhs, Nm = (3, 2, 25) if m < 600 else (2, 1, 10)
    A, B, lam0 = _problems(10 + norm, F, nrhs, l, m)
    acfg = api.default_admm_config(norm=norm, max_iters=Nm, rho=4.0, gamma=1.0, epsilon=0.0, p=0.5, gst_iters=4,
                                   precision=precision)
    c, its, info = _run(ctx, cuda, A, B, lam0, acfg)
    tol = 1e-10 if precision == 0 else 1e-9
    for f in range(F):
        for r in range(nrhs):
            co, ito, conv = O.admm(A[f], B[f, r], lam0[f, r], 4.0, 1.0, 0.0, Nm, norm, p=0.5, N=4)
            assert not conv and its[f, r] == ito
            assert relerr(c[f, r], co) < tol, (f, r)
    assert np.all(info == 1)      # IA_INFO_NOCONV: no stage met epsilon = 0


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("norm", [1, 2, 3])
def test_admm_converged_match_oracle(cuda, ctx, norm, precision):
    from inverseacoustics_gb300 import api
    l, m = 24, 80
    F, nrhs, Nm = 4, 1, 3000
    A, B, lam0 = _problems(20 + norm, F, nrhs, l, m)
    acfg = api.default_admm_config(norm=norm, max_iters=Nm, rho=6.0, gamma=1.0, epsilon=1e-8, p=0.7, gst_iters=6,
                                   precision=precision)
    c, its, info = _run(ctx, cuda, A, B, lam0, acfg)
    for f in range(F):
        co, ito, conv = O.admm(A[f], B[f, 0], lam0[f, 0], 6.0, 1.0, 1e-8, Nm, norm, p=0.7, N=6)
        assert conv and its[f, 0] == ito
        assert relerr(c[f, 0], co) < (1e-9 if precision == 0 else 1e-8)
    assert np.all(info == 0)


def test_admm_given_x0_and_batch_independence(cuda, ctx):
    """A caller-supplied starting point (MATLAB's own A \\ b, say) is used as
    is; a system's result is bitwise the same alone and inside a batch."""
    from inverseacoustics_gb300 import api
    l, m = 32, 300
    A, B, lam0 = _problems(31, 4, 1, l, m)
    rng = np.random.default_rng(3)
    x0 = rng.normal(size=(4, 1, m)) + 1j * rng.normal(size=(4, 1, m))
    acfg = api.default_admm_config(norm=3, max_iters=20, rho=3.0, epsilon=0.0, p=0.5, gst_iters=3)
    c, its, _ = _run(ctx, cuda, A, B, lam0, acfg, x0)
    for f in range(4):
        co, ito, _ = O.admm(A[f], B[f, 0], lam0[f, 0], 3.0, 1.0, 0.0, 20, 3, p=0.5, N=3, x0=x0[f, 0])
        assert relerr(c[f, 0], co) < 1e-10
    c1, _, _ = _run(ctx, cuda, A[2:3], B[2:3], lam0[2:3], acfg, x0[2:3])
    assert np.array_equal(c1[0], c[2])


def test_admm_l1_recovers_monopole_sources(cuda, ctx):
    """Sparse equivalent sources: 3 of 162 monopoles on a sphere radiate to 48
    microphones; L1 ADMM on the monopole transfer matrix puts its largest
    entries on the true sources, as the oracle does."""
    from inverseacoustics_gb300 import api
    src, _ = g.icosphere(2, 0.1)
    mics = g.hemisphere_array(np.random.default_rng(4), 48, 0.3)
    ks = 2 * np.pi * np.array([1200.0, 2000.0]) / 343.0
    m = src.shape[1]
    A = np.stack([O.monopole_matrix(mics, src, k) for k in ks])
    A = A / np.linalg.norm(A, axis=(1, 2), keepdims=True) * np.sqrt(48)
    true = np.array([5, 77, 140])
    X = np.zeros((2, 1, m), complex)
    X[:, 0, true] = [1.0, 0.7j, -0.5]
    B = np.einsum("flm,frm->frl", A, X)
    lam0 = np.full((2, 1), 0.01)
    acfg = api.default_admm_config(norm=1, max_iters=200, rho=2.0, epsilon=1e-9)
    c, its, info = _run(ctx, cuda, A, B, lam0, acfg)
    for f in range(2):
        co, ito, _ = O.admm(A[f], B[f, 0], 0.01, 2.0, 1.0, 1e-9, 200, 1)
        assert its[f, 0] == ito
        assert relerr(c[f, 0], co) < 1e-7
        assert set(np.argsort(-np.abs(c[f, 0]))[:3]) == set(true)


def test_admm_and_bem_modes_reject_bad_arguments(cuda, ctx):
    """Invalid configurations come back as IA_ERR_ARG before any device work."""
    from inverseacoustics_gb300 import api
    from inverseacoustics_gb300._lib import IAError
    A, B, lam0 = _problems(40, 1, 1, 8, 20)
    bad = [dict(norm=0), dict(norm=4), dict(rho=0.0), dict(rho=-1.0), dict(max_iters=-1), dict(epsilon=-1e-6),
           dict(norm=3, p=0.0), dict(norm=3, p=1.5), dict(norm=3, gst_iters=-1), dict(precision=2)]
    for kw in bad:
        with pytest.raises(IAError) as e:
            _run(ctx, cuda, A, B, lam0, api.default_admm_config(**kw))
        assert e.value.code == 1, kw
    nodes, elems = g.icosphere(1, 0.1)
    mesh = api.Mesh(ctx, nodes, elems)
    mics, k = T(g.hemisphere_array(np.random.default_rng(1), 8, 0.3), cuda), T(np.array([3.0]), cuda)
    for nm in (0, nodes.shape[1] + 1):
        for cplx in (False, True):
            with pytest.raises(IAError) as e:
                api.bem_modes_batch(ctx, mesh, mics, k, nm, complex_modes=cplx)
            assert e.value.code == 1
    mesh.close()
