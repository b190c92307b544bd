"""GPU suite: the differentiable ESM array-design objective and its
hand-written adjoint (ia_esm_design_batch) against the FP64 oracle loss and
gradient, against central finite differences of the GPU loss (h = 1e-6,
bound 1e-5), and driven by torch.optim.Adam through a torch.autograd.Function
that exists only here, in the test harness."""
import math

import numpy as np
import pytest

from inverseacoustics_gb300 import geometry as g
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


def _case(seed, l, subdiv, F, R, fmin=200.0, fmax=4000.0):
    rng = np.random.default_rng(seed)
    surf, _ = g.icosphere(subdiv, 0.10)
    mics = np.stack([rng.uniform(-0.2, 0.2, l), rng.uniform(-0.2, 0.2, l), np.full(l, 0.12)])
    k = 2 * np.pi * np.linspace(fmin, fmax, F) / 343.0
    q = g.complex_normal(rng, (F, surf.shape[1], R))
    src = O.retreat_sources(surf, 0.04)
    noise = np.zeros((F, l, R), complex)
    loglam = np.zeros(F)
    for f in range(F):
        G = O.monopole_matrix(mics, src, k[f])
        p = G @ q[f]
        noise[f] = 10 ** (-30 / 20) * np.linalg.norm(p) / math.sqrt(p.size) * g.complex_normal(rng, (l, R))
        loglam[f] = math.log(0.05 * np.linalg.norm(G) / math.sqrt(l))
    return mics, surf, 0.04, k, loglam, q, noise


def _dev_args(case, dev):
    mics, surf, d, k, ll, q, noise = case
    return (T(mics, dev), T(surf, dev), T(np.array([d]), dev), T(k, dev), T(ll, dev),
            T(np.transpose(q, (0, 2, 1)), dev), T(np.transpose(noise, (0, 2, 1)), dev))


def test_design_matches_oracle(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    case = _case(1, 24, 1, 4, 6)
    mics, surf, d, k, ll, q, noise = case
    err, gm, gd, gl, info = api.esm_design_batch(ctx, *_dev_args(case, cuda))
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    eo = O.esm_design_terms(mics, surf, d, k, ll, q, noise)
    gmo, gdo, glo = O.esm_design_grad(mics, surf, d, k, ll, q, noise)
    assert np.max(np.abs(err.cpu().numpy() - eo)) <= 1e-10 * np.max(eo)
    assert np.max(np.abs(gm.cpu().numpy() - gmo)) <= 1e-9 * np.max(np.abs(gmo))
    assert abs(gd.item() - gdo) <= 1e-9 * abs(gdo)
    assert np.max(np.abs(gl.cpu().numpy() - glo)) <= 1e-9 * np.max(np.abs(glo))


def test_design_full_size_finite_differences(cuda, ctx):
    """128 microphones, 642 sources, 16 fields, 8 of the 128 frequencies:
    adjoint gradient components against central differences of the GPU
    loss, and against the FP64 oracle gradient."""
    from inverseacoustics_gb300 import api
    import torch
    case = _case(4, 128, 3, 8, 16)
    mics, surf, d, k, ll, q, noise = case
    M, S, D, K, LL, Q, N = _dev_args(case, cuda)
    err, gm, gd, gl, info = api.esm_design_batch(ctx, M, S, D, K, LL, Q, N)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    gm, gd, gl = gm.cpu().numpy(), gd.item(), gl.cpu().numpy()

    def loss(M_=M, D_=D, LL_=LL):
        e = api.esm_design_batch(ctx, M_, S, D_, K, LL_, Q, N, grad=False)[0]
        return float(e.mean().item())

    h = 1e-6
    for a, i in ((0, 0), (1, 5), (2, 17), (0, 63), (1, 100), (2, 127)):
        Mp, Mm = M.clone(), M.clone()
        Mp[a, i] += h
        Mm[a, i] -= h
        fd = (loss(M_=Mp) - loss(M_=Mm)) / (2 * h)
        assert abs(fd - gm[a, i]) <= 1e-5 * np.max(np.abs(gm)), (a, i, fd, gm[a, i])
    fd = (loss(D_=D + h) - loss(D_=D - h)) / (2 * h)
    assert abs(fd - gd) <= 1e-5 * abs(gd)
    for f in (0, 3, 7):
        Lp, Lm = LL.clone(), LL.clone()
        Lp[f] += h
        Lm[f] -= h
        fd = (loss(LL_=Lp) - loss(LL_=Lm)) / (2 * h)
        assert abs(fd - gl[f]) <= 1e-5 * np.max(np.abs(gl)), (f, fd, gl[f])
    sel = [0, 7]
    gmo, gdo, glo = O.esm_design_grad(mics, surf, d, k[sel], ll[sel], q[sel], noise[sel])
    e2, gm2, gd2, gl2, _ = api.esm_design_batch(ctx, M, S, D, K[sel].contiguous(), LL[sel].contiguous(),
                                                Q[sel].contiguous(), N[sel].contiguous())
    torch.cuda.synchronize()
    assert np.max(np.abs(gm2.cpu().numpy() - gmo)) <= 1e-9 * np.max(np.abs(gmo))
    assert abs(gd2.item() - gdo) <= 1e-9 * abs(gdo)
    assert np.max(np.abs(gl2.cpu().numpy() - glo)) <= 1e-9 * np.max(np.abs(glo))


def _design_fn(ctx):
    """The test harness's torch.autograd.Function around ia_esm_design_batch."""
    from inverseacoustics_gb300 import api
    import torch

    class EsmDesign(torch.autograd.Function):
        @staticmethod
        def forward(fctx, mics, retreat, loglam, surf, k, q, noise):
            err, gm, gd, gl, _ = api.esm_design_batch(ctx, mics.detach().contiguous(), surf,
                                                      retreat.detach().contiguous(), k, loglam.detach().contiguous(),
                                                      q, noise)
            fctx.save_for_backward(gm, gd, gl)
            return err.mean()

        @staticmethod
        def backward(fctx, gout):
            gm, gd, gl = fctx.saved_tensors
            return gout * gm, gout * gd, gout * gl, None, None, None, None

    return EsmDesign


def _design_problem(cuda):
    """The full design problem: 128 frequencies, 128 mics, 642 sources, 16
    fields; (initial mics, initial log lambda, device tensors S, K, Q, N)."""
    w = g.esm_design(n_freq=128)
    rng = np.random.default_rng(40)
    mics0, surf = w.arrays["mics"], w.arrays["surface"]
    q = w.params["q"]                                      # (F, 642, 16)
    src = O.retreat_sources(surf, 0.04)
    noise = np.zeros((128, 128, 16), complex)
    ll0 = np.zeros(128)
    for f, kk in enumerate(w.k):
        G = O.monopole_matrix(mics0, src, kk)
        p = G @ q[f]
        noise[f] = 10 ** (-30 / 20) * np.linalg.norm(p) / math.sqrt(p.size) * g.complex_normal(rng, (128, 16))
        ll0[f] = math.log(0.05 * np.linalg.norm(G) / math.sqrt(128))
    return (mics0, ll0, T(surf, cuda), T(w.k, cuda), T(np.transpose(q, (0, 2, 1)), cuda),
            T(np.transpose(noise, (0, 2, 1)), cuda))


def _adam(params):
    import torch
    mics, retreat, loglam = params
    return torch.optim.Adam([{"params": [mics, retreat], "lr": 2e-4}, {"params": [loglam], "lr": 2e-2}])


def save_checkpoint(path, params, opt):
    """Parameters and Adam state of the design loop as one .npz."""
    d = {}
    for i, p in enumerate(params):
        st = opt.state[p]
        d[f"param{i}"] = p.detach().cpu().numpy()
        d[f"exp_avg{i}"] = st["exp_avg"].cpu().numpy()
        d[f"exp_avg_sq{i}"] = st["exp_avg_sq"].cpu().numpy()
        d[f"step{i}"] = st["step"].cpu().numpy()
    np.savez(path, **d)


def load_checkpoint(path, params, opt):
    import torch
    z = np.load(path)
    with torch.no_grad():
        for i, p in enumerate(params):
            p.copy_(torch.as_tensor(z[f"param{i}"], device=p.device))
    for i, p in enumerate(params):
        opt.state[p] = {"step": torch.as_tensor(z[f"step{i}"]),
                        "exp_avg": torch.as_tensor(z[f"exp_avg{i}"], device=p.device),
                        "exp_avg_sq": torch.as_tensor(z[f"exp_avg_sq{i}"], device=p.device)}


def test_design_adam_on_device(cuda, ctx, tmp_path):
    """200 Adam steps of the full design problem (128 frequencies) with the
    adjoint behind a torch.autograd.Function; no host round trip inside the
    loop.  The loss must fall.  A checkpoint (parameters and Adam state, .npz)
    written at step 100 and resumed in a fresh optimizer ends bitwise where the
    uninterrupted run ends (the adjoint's reductions are deterministic)."""
    import torch
    EsmDesign = _design_fn(ctx)
    mics0, ll0, S, K, Q, N = _design_problem(cuda)

    def fresh():
        return [T(mics0, cuda).requires_grad_(True), T(np.array([0.04]), cuda).requires_grad_(True),
                T(ll0, cuda).requires_grad_(True)]

    def run(params, opt, steps, ckpt_at=None):
        losses = []
        for step in steps:
            if step == ckpt_at:
                save_checkpoint(tmp_path / "design.npz", params, opt)
            opt.zero_grad()
            L = EsmDesign.apply(params[0], params[1], params[2], S, K, Q, N)
            L.backward()
            opt.step()
            if step in (0, 199):
                losses.append(L.detach())
        return losses

    params = fresh()
    opt = _adam(params)
    losses = run(params, opt, range(200), ckpt_at=100)
    torch.cuda.synchronize()
    l0, l1 = (float(x.item()) for x in losses)
    assert math.isfinite(l1) and l1 < 0.95 * l0, (l0, l1)
    # resume from step 100
    params2 = fresh()
    opt2 = _adam(params2)
    load_checkpoint(tmp_path / "design.npz", params2, opt2)
    run(params2, opt2, range(100, 200))
    torch.cuda.synchronize()
    for p, p2 in zip(params, params2):
        assert torch.equal(p.detach(), p2.detach())
