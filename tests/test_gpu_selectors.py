"""GPU suite: the other lambda selectors and the damped SVD (L-curve corner,
quasi-optimality, dsvd; MATLAB/regtools/l_curveG.m, lcfunG.m, quasioptG.m,
dsvdG.m) through ia_esm_solve_batch, against the FP64 oracle restatement.
Tall (more microphones than sources: the least-squares residual enters the
L-curve) and wide operators; FP64 and mixed paths.

Bounds: the selectors end with MATLAB's fminbnd (absolute TolX 1e-4), so lambda
is defined by the Brent iterates; identical objective values give identical
iterates.  FP64: lambda 1e-9 and x 1e-9 relative; mixed: lambda and x 1e-6."""
import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu

METHODS = {3: "tikhonov-lcurve", 4: "tikhonov-quasiopt", 5: "dsvd-fixed", 6: "dsvd-lcurve", 7: "dsvd-quasiopt"}


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


@pytest.mark.parametrize("shape", ["tall", "wide"])
@pytest.mark.parametrize("precision", [0, 1])
def test_selectors_match_oracle(cuda, ctx, shape, precision):
    from inverseacoustics_gb300 import api
    import torch
    if shape == "tall" and precision == 1:
        pytest.skip("tall operators take the FP64 SVD in both precisions")
    rng = np.random.default_rng(17)
    mics = g.planar_array(8, 8, 0.03, 0.10)
    src, _ = g.icosphere(1 if shape == "tall" else 2, 0.05)
    ks = 2 * np.pi * np.array([600.0, 1500.0, 3200.0]) / 343.0
    p = np.stack([g.add_noise(rng, O.monopole_matrix(mics, src, k) @ g.complex_normal(rng, src.shape[1]), 25.0)
                  [None, :] for k in ks])
    tol = 1e-9 if precision == 0 else 1e-6
    worst = {}
    for method, name in METHODS.items():
        cfg = api.default_config(method=method, precision=precision, lambda_fixed=0.05)
        x, lam, s, info = api.esm_solve_batch(ctx, T(mics, cuda), T(src, cuda), T(ks, cuda), T(p, cuda), cfg)
        torch.cuda.synchronize()
        assert int(info.abs().sum()) == 0
        for f, k in enumerate(ks):
            G = O.monopole_matrix(mics, src, k)
            xo, lo, _ = O.solve_regularized(G, p[f, 0], name, lam_fixed=0.05)
            el = abs(lam[f, 0].item() - lo) / lo
            ex = relerr(x[f, 0].cpu().numpy(), xo)
            worst[name] = max(worst.get(name, 0.0), el, ex)
            assert el <= tol and ex <= tol, (name, f, el, ex)
    print(shape, precision, {k: f"{v:.1e}" for k, v in worst.items()})
