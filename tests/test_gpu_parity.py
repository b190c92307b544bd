"""GPU suite: every kernel through the C ABI against the oracle and the
reference's golden vectors.  FP64 path tolerance: 1e-10 relative."""
import math

import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from inverseacoustics_gb300 import quadrature as Q
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-10


def T(a, dev, dtype=None):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev, dtype=dtype)


# ------------------------------------------------------------- layer 1 (host)
def test_esm_matches_reference_golden(cuda, golden):
    from inverseacoustics_gb300 import api
    Me, He = api.esm(golden["esm_src"], golden["esm_fld"], float(golden["esm_k"]), float(golden["esm_ri"]))
    assert relerr(Me, golden["esm_Me"]) < TOL
    assert relerr(He, golden["esm_He"]) < TOL


def test_esm_wide_matches_oracle(cuda):
    from inverseacoustics_gb300 import api
    src, _ = g.icosphere(2, 0.05)
    mics = g.planar_array(8, 8, 0.03, 0.10)
    k = 2 * np.pi * 1000 / 343.0
    Me, He = api.esm(src, mics, k, 0.6)
    Mo, Ho = O.esm(src, mics, k, 0.6, 343.0, 1.21)
    assert relerr(Me, Mo) < TOL and relerr(He, Ho) < TOL


@pytest.mark.parametrize("i", [0, 1])
def test_ibem_matches_reference_golden(cuda, golden, i):
    from inverseacoustics_gb300 import api
    Z, H = api.ibem(golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["ks"][i],
                    rules=(golden["rule_regular"], golden["rule_singular"]))
    assert relerr(Z, golden[f"ibem_Z_{i}"]) < TOL
    assert relerr(H, golden[f"ibem_H_{i}"]) < TOL


def test_ibem_chief_matches_reference_golden(cuda, golden):
    from inverseacoustics_gb300 import api
    Z, H = api.ibem(golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["ks"][0], n_ch=2,
                    cp=golden["chief"], rules=(golden["rule_regular"], golden["rule_singular"]))
    assert relerr(Z, golden["ibem_chief_Z"]) < TOL
    assert relerr(H, golden["ibem_chief_H"]) < TOL


def test_ibem_builtin_rules_match_oracle(cuda):
    from inverseacoustics_gb300 import api
    nodes, elems = g.icosphere(2, 0.1)
    mics = g.hemisphere_array(np.random.default_rng(3), 20, 0.3)
    k = 2 * np.pi * 1200 / 343.0
    reg, sing = Q.builtin()
    Z, H = api.ibem(nodes, elems, mics, k)
    Zo, Ho = O.ibem(nodes, elems, mics, k, reg, sing, 343.0, 1.21)
    assert relerr(Z, Zo) < TOL and relerr(H, Ho) < TOL


def _colwise(a, b):
    num = np.linalg.norm(a - b, axis=0)
    den = np.linalg.norm(b, axis=0)
    return float(np.max(num / den))


def test_hels_matches_oracle(cuda):
    from inverseacoustics_gb300 import api
    rng = np.random.default_rng(11)
    S = g.cartesian_to_spherical(g.hemisphere_array(rng, 40, 0.08))
    Hp = g.cartesian_to_spherical(g.planar_array(6, 6, 0.025, 0.15))
    for f in (50.0, 800.0, 3000.0):
        k = 2 * np.pi * f / 343.0
        Me, He, Qe = api.hels(S, Hp, k, 15)
        Mo, Ho, Qo = O.hels(S, Hp, k, 15, 343.0, 1.21)
        assert _colwise(Me, Mo) < TOL and _colwise(He, Ho) < TOL and _colwise(Qe, Qo) < TOL


@pytest.mark.parametrize("shape", [(40, 25), (25, 40), (32, 32), (120, 7), (3, 200)])
def test_csvd(cuda, shape):
    from inverseacoustics_gb300 import api
    rng = np.random.default_rng(sum(shape))
    m, n = shape
    A = g.complex_normal(rng, shape) @ np.diag(np.logspace(0, -8, n))
    U, s, V = api.csvd(A)
    so = np.linalg.svd(A, compute_uv=False)
    assert np.max(np.abs(s - so)) < 1e-13 * so[0]
    assert relerr(U @ np.diag(s) @ V.conj().T, A) < 1e-13
    p = min(m, n)
    assert np.abs(U.conj().T @ U - np.eye(p)).max() < 1e-12
    assert np.abs(V.conj().T @ V - np.eye(p)).max() < 1e-12


def test_tsvd_matches_oracle(cuda):
    from inverseacoustics_gb300 import api
    rng = np.random.default_rng(2)
    A = g.complex_normal(rng, (30, 18))
    b = g.complex_normal(rng, 30)
    U, s, V = O.csvd(A)
    for k in (1, 9, 18):
        assert relerr(api.tsvd(U, s, V, b, k), O.tsvd(U, s, V, b, k)) < 1e-13


def test_pressure_velocity_power(cuda):
    from inverseacoustics_gb300 import api
    rng = np.random.default_rng(4)
    Me = g.complex_normal(rng, (20, 9))
    x = g.complex_normal(rng, 9)
    assert relerr(api.to_pressure(Me, x), Me @ x) < 1e-14
    assert relerr(api.to_velocity(Me, x), Me @ x) < 1e-14
    p, v = g.complex_normal(rng, 20), g.complex_normal(rng, 20)
    assert abs(api.sound_power(p, v, 0.3) - O.sound_power(p, v, 0.3)) < 1e-14 * abs(O.sound_power(p, v, 0.3)) + 1e-300


# ------------------------------------------------------------ layer 2 (batched)
def test_monopole_batch(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    mics = g.planar_array(8, 8, 0.03, 0.10)
    src, _ = g.icosphere(2, 0.05)
    ks = 2 * np.pi * np.array([200.0, 1000.0, 4000.0]) / 343.0
    G = api.monopole_batch(ctx, T(mics, cuda), T(src, cuda), T(ks, cuda))
    torch.cuda.synchronize()
    for f, k in enumerate(ks):
        assert relerr(G[f].cpu().numpy().T, O.monopole_matrix(mics, src, k)) < 1e-14


def _gcv_problem(seed, m, n, F, snr=30.0):
    rng = np.random.default_rng(seed)
    mics = g.planar_array(8, 8, 0.03, 0.10) if m == 64 else g.hemisphere_array(rng, m, 0.3)
    src, _ = g.icosphere(2, 0.05)
    ks = 2 * np.pi * np.linspace(300, 3000, F) / 343.0
    Hs, bs = [], []
    for k in ks:
        G = O.monopole_matrix(mics, src[:, :n], k)
        q = g.complex_normal(rng, n)
        Hs.append(G)
        bs.append(g.add_noise(rng, G @ q, snr))
    return mics, src[:, :n], ks, Hs, bs


@pytest.mark.parametrize("mode", ["standard", "reference"])
def test_solve_batch_matches_oracle(cuda, ctx, mode):
    from inverseacoustics_gb300 import api
    import torch
    _, _, ks, Hs, bs = _gcv_problem(21, 64, 162, 5)
    F = len(Hs)
    Hc = T(np.stack([h.T for h in Hs]), cuda)           # (F, n, m): column-major m x n
    b = T(np.stack([bb[None, :] for bb in bs]), cuda)    # (F, 1, m)
    cfg = api.default_config(gcv_mode=1 if mode == "reference" else 0)
    x, lam, s, info = api.solve_batch(ctx, Hc, 64, 162, b, cfg)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    for f in range(F):
        xo, lo, so = O.solve_tikhonov_gcv(Hs[f], bs[f], mode=mode)
        assert np.max(np.abs(s[f].cpu().numpy() - so)) < 1e-12 * so[0]
        tol = TOL if mode == "standard" else 1e-7
        assert abs(lam[f, 0].item() - lo) < tol * lo
        assert relerr(x[f, 0].cpu().numpy(), xo) < (TOL if mode == "standard" else 1e-6)


def test_solve_batch_cluster_jacobi_is_bitwise_the_one_cta_kernel(cuda, ctx):
    """The FP64 one-sided Jacobi runs over a 4-CTA cluster per bin when the
    clusters fit on the SMs (8 bins) and one CTA per bin otherwise (80 bins):
    the same rotations in the same order, so the first 8 bins of the 80-bin
    call equal the 8-bin call bit for bit (x, lambda, s)."""
    from inverseacoustics_gb300 import api
    import torch
    _, _, _, Hs, bs = _gcv_problem(23, 64, 162, 80)
    Hc = T(np.stack([h.T for h in Hs]), cuda)
    b = T(np.stack([bb[None, :] for bb in bs]), cuda)
    x, lam, s, info = api.solve_batch(ctx, Hc, 64, 162, b)
    x8, lam8, s8, info8 = api.solve_batch(ctx, Hc[:8].contiguous(), 64, 162, b[:8].contiguous())
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0 and int(info8.abs().sum()) == 0
    assert torch.equal(x[:8], x8) and torch.equal(lam[:8], lam8) and torch.equal(s[:8], s8)


def test_esm_pipeline_single_frequency(cuda, ctx):
    """Config 'ESM plain, single frequency' end to end: monopole G, SVD,
    GCV over 200 log-spaced lambda in [1e-8, 1e2], Tikhonov."""
    from inverseacoustics_gb300 import api
    import torch
    w = g.esm_single()
    rng = w.params["rng"]
    mics, src = w.arrays["mics"], w.arrays["sources"]
    k = w.k[0]
    G = O.monopole_matrix(mics, src, k)
    p = g.add_noise(rng, G @ g.complex_normal(rng, src.shape[1]), 30.0)
    cfg = api.default_config(gcv_lo=1e-8, gcv_hi=1e2)
    x, lam, s, info = api.esm_solve_batch(ctx, T(mics, cuda), T(src, cuda), T(w.k, cuda), T(p[None, None, :], cuda),
                                          cfg)
    torch.cuda.synchronize()
    xo, lo, so = O.solve_tikhonov_gcv(G, p, grid=(1e-8, 1e2))
    assert int(info[0]) == 0
    assert abs(lam[0, 0].item() - lo) < TOL * lo
    assert relerr(x[0, 0].cpu().numpy(), xo) < TOL


def test_ibem_transfer_batch_matches_oracle(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    nodes, elems = g.icosphere(2, 0.1)
    mics = g.hemisphere_array(np.random.default_rng(5), 24, 0.3)
    ks = 2 * np.pi * np.array([150.0, 900.0, 1900.0]) / 343.0
    mesh = api.Mesh(ctx, nodes, elems)
    H, info = api.ibem_transfer_batch(ctx, mesh, T(mics, cuda), T(ks, cuda))
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    reg, sing = Q.builtin()
    for f, k in enumerate(ks):
        Ho = O.ibem_transfer(nodes, elems, mics, k, reg, sing, 343.0, 1.21)
        assert relerr(H[f].cpu().numpy().T, Ho) < TOL


def test_ibem_assemble_rows_match_oracle(cuda, ctx, golden):
    from inverseacoustics_gb300 import api
    import torch
    nodes, elems, mics, cp = golden["mesh_nodes"], golden["mesh_elems"], golden["mics"], golden["chief"]
    rules = (golden["rule_regular"], golden["rule_singular"])
    mesh = api.Mesh(ctx, nodes, elems, rules)
    ks = golden["ks"]
    At, Bt, Ah, Bh = api.ibem_assemble_batch(ctx, mesh, T(mics, cuda), T(ks, cuda), cp=T(cp, cuda))
    torch.cuda.synchronize()
    for f, k in enumerate(ks):
        A, B, Ahs, Bhs = O.ibem_assemble(nodes, elems, mics, k, *rules, 343.0, 1.21, cp)
        assert relerr(At[f].cpu().numpy(), A) < 1e-13
        assert relerr(Bt[f].cpu().numpy(), B) < 1e-13
        assert relerr(Ah[f].cpu().numpy(), Ahs) < 1e-13
        assert relerr(Bh[f].cpu().numpy(), Bhs) < 1e-13


def test_ibem_pipeline_matches_oracle_and_is_deterministic(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    nodes, elems = g.icosphere(2, 0.1)
    rng = np.random.default_rng(9)
    mics = g.hemisphere_array(rng, 40, 0.3)
    ks = 2 * np.pi * np.array([300.0, 1200.0]) / 343.0
    p = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in ks])
    mesh = api.Mesh(ctx, nodes, elems)
    args = (ctx, mesh, T(mics, cuda), T(ks, cuda), T(p, cuda))
    x, lam, s, info = api.ibem_solve_batch(*args)
    x2, lam2, _, _ = api.ibem_solve_batch(*args)
    torch.cuda.synchronize()
    assert torch.equal(x, x2) and torch.equal(lam, lam2)
    reg, sing = Q.builtin()
    for f, k in enumerate(ks):
        H = O.ibem_transfer(nodes, elems, mics, k, reg, sing, 343.0, 1.21)
        xo, lo, so = O.solve_tikhonov_gcv(H, p[f, 0])
        assert abs(lam[f, 0].item() - lo) < TOL * lo
        assert relerr(x[f, 0].cpu().numpy(), xo) < TOL


@pytest.mark.parametrize("precision,uniform,nrhs,F", [(0, True, 1, 16), (1, True, 1, 16), (1, False, 2, 16),
                                                       (1, True, 1, 32), (0, False, 1, 32), (1, False, 1, 64)])
def test_ibem_split_pipeline_is_bitwise_the_unsplit_one(cuda, ctx, precision, uniform, nrhs, F):
    """F = 16 runs as two staggered parts of 8, F = 32 as four of 8 and F = 64
    as four of 16, each part on its own stream; every 8 bins equal a plain 8-bin call
    bit for bit (bins stay in their assembly blocks, later kernels work per
    bin) -- evenly spaced bins (phase recurrence in the assembly) and
    scattered ones, one and two right-hand sides."""
    from inverseacoustics_gb300 import api
    import torch
    nodes, elems = g.icosphere(2, 0.1)
    rng = np.random.default_rng(19)
    mics = g.hemisphere_array(rng, 40, 0.3)
    f = np.linspace(200.0, 1800.0, F) if uniform else np.sort(rng.uniform(150.0, 1900.0, F))
    ks = 2 * np.pi * f / 343.0
    p = np.stack([np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0 + r), 30.0)
                            for r in range(nrhs)]) for k in ks])
    mesh = api.Mesh(ctx, nodes, elems)
    cfg = api.default_config(precision=precision)
    md, kd, pd = T(mics, cuda), T(ks, cuda), T(p, cuda)
    x, lam, s, info = api.ibem_solve_batch(ctx, mesh, md, kd, pd, cfg)
    starts = list(range(0, F, 8))
    parts = [api.ibem_solve_batch(ctx, mesh, md, kd[h:h + 8].contiguous(), pd[h:h + 8].contiguous(), cfg)
             for h in starts]
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    for h, (xh, lh, sh, ih) in zip(starts, parts):
        assert torch.equal(x[h:h + 8], xh) and torch.equal(lam[h:h + 8], lh) and torch.equal(s[h:h + 8], sh)
        assert torch.equal(info[h:h + 8], ih)


def test_hels_pipeline_matches_oracle(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    rng = np.random.default_rng(12)
    mics = g.planar_array(8, 8, 0.025, 0.15)
    pts = g.cartesian_to_spherical(mics)
    ks = 2 * np.pi * np.array([500.0, 2500.0]) / 343.0
    src = rng.normal(size=(3, 5)) * 0.03
    p = []
    for k in ks:
        p.append(g.add_noise(rng, O.monopole_matrix(mics, src, k) @ g.complex_normal(rng, 5), 25.0)[None, :])
    p = np.stack(p)
    x, lam, s, info = api.hels_solve_batch(ctx, T(pts, cuda), 6, T(ks, cuda), T(p, cuda))
    torch.cuda.synchronize()
    for f, k in enumerate(ks):
        _, He, _ = O.hels(pts, pts, k, 6, 343.0, 1.21)
        xo, lo, so = O.solve_tikhonov_gcv(He, p[f, 0])
        # lambda sits at a zero of dG/dlog(lambda); summation-order noise moves it
        # by ~ eps / G'' -- the solution is flat there, so x carries the 1e-10 bar.
        assert abs(lam[f, 0].item() - lo) < 1e-7 * lo
        assert relerr(x[f, 0].cpu().numpy(), xo) < TOL


def test_ibem_full_size_transfer(cuda, ctx):
    """Full config size (642 nodes, 1280 triangles, 120 mics): H at two of the
    64 frequencies against the oracle; the rest through size-independent
    properties (finite; H v for the pulsating sphere close to the analytic
    field, away from the interior Dirichlet resonance ka = pi of the sphere,
    where collocation BEM without CHIEF points is ill-posed)."""
    from inverseacoustics_gb300 import api
    import torch
    w = g.ibem_sphere(n_freq=8)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    mesh = api.Mesh(ctx, nodes, elems)
    H, info = api.ibem_transfer_batch(ctx, mesh, T(mics, cuda), T(w.k, cuda))
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    reg, sing = Q.builtin()
    for f in (0, 5):
        Ho = O.ibem_transfer(nodes, elems, mics, w.k[f], reg, sing, 343.0, 1.21)
        assert relerr(H[f].cpu().numpy().T, Ho) < TOL
    v = np.ones(nodes.shape[1])
    for f in range(8):
        Hf = H[f].cpu().numpy().T
        assert np.isfinite(Hf).all()
        if abs(w.k[f] * 0.1 - np.pi) < 0.05 * np.pi:
            continue
        ph = g.pulsating_sphere_pressure(mics, w.k[f], 0.1, 1.0)
        assert relerr(Hf @ v, ph) < 5e-2


def test_nonfinite_input_is_flagged(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    rng = np.random.default_rng(1)
    A = g.complex_normal(rng, (2, 12, 10))
    A[1, 3, 4] = np.nan
    b = g.complex_normal(rng, (2, 1, 10))
    x, lam, s, info = api.solve_batch(ctx, T(A, cuda), 10, 12, T(b, cuda))
    torch.cuda.synchronize()
    assert int(info[0]) == 0
    assert int(info[1]) & 4


def test_bad_rule_and_mesh_rejected(cuda, ctx):
    from inverseacoustics_gb300 import api
    nodes, elems = g.icosphere(1, 0.1)
    reg, sing = Q.builtin()
    bad = reg.copy()
    bad[:, 2] *= 1.5
    with pytest.raises(api.IAError) as e:
        api.Mesh(ctx, nodes, elems, (bad, sing))
    assert e.value.code == 7
    el = elems.copy()
    el[1, 0] = el[0, 0]
    with pytest.raises(api.IAError) as e:
        api.Mesh(ctx, nodes, el)
    assert e.value.code == 1
    # two nodes at one point: equal collocation rows, a singular system
    nd = nodes.copy()
    nd[:, 5] = nd[:, 3]
    with pytest.raises(api.IAError) as e:
        api.Mesh(ctx, nd, elems)
    assert e.value.code == 1
