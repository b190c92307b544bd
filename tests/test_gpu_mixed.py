"""GPU suite: the mixed-precision path (FP32 LU / QR / Jacobi, double-float
refinement and transfer GEMMs, FP64 Tikhonov refinement) against the FP64
oracle.  Stated bound: relative error <= 1e-6 on x; H at FP64 level (1e-11)."""
import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from inverseacoustics_gb300 import quadrature as Q
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-6


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


@pytest.fixture(params=["table", "inline"])
def geom_form(request, monkeypatch):
    """The double-float assembly with its per-call geometry table (the default
    wherever the table fits the size limit) and with the geometry computed
    inline (IA_ASM_GEOM_TABLE=0, the form above the limit)."""
    if request.param == "inline":
        monkeypatch.setenv("IA_ASM_GEOM_TABLE", "0")
    else:
        monkeypatch.delenv("IA_ASM_GEOM_TABLE", raising=False)
    return request.param


def test_mixed_assembly_matches_fp64(cuda, ctx, geom_form):
    """The mixed path assembles in double-float (FP32 pairs, own sin/cos by
    Cody-Waite reduction + Taylor series): rows agree with the FP64 kernel
    (CUDA sincos/rsqrt) to 1e-13, element by element to 1e-12."""
    from inverseacoustics_gb300 import api
    import torch
    w = g.ibem_sphere(n_freq=64)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    ks = w.k[[0, 1, 2, 3, 30, 61, 62, 63]]           # two uniform blocks + a non-uniform block edge
    mesh = api.Mesh(ctx, nodes, elems)
    r64 = api.ibem_assemble_batch(ctx, mesh, T(mics, cuda), T(ks, cuda))
    rmx = api.ibem_assemble_batch(ctx, mesh, T(mics, cuda), T(ks, cuda), api.default_config(precision=1))
    torch.cuda.synchronize()
    for a, b in zip(r64, rmx):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        for f in range(len(ks)):
            assert relerr(b[f], a[f]) < 1e-13
        assert np.max(np.abs(b - a)) < 1e-12 * np.max(np.abs(a))


def test_mixed_assembly_large_arguments(cuda, ctx, geom_form):
    """kr up to ~150: the table-driven double-float sin/cos reduces by pi/512
    exactly for kr < 100 and hands larger arguments to the FP64-reduced series;
    both regimes (and the switch between them inside one row) agree with the
    FP64 kernel to 1e-12."""
    from inverseacoustics_gb300 import api
    import torch
    nodes, elems = g.icosphere(2, 1.0)
    mics = g.hemisphere_array(np.random.default_rng(5), 16, 3.0)
    ks = np.array([20.0, 37.5, 41.0])            # kr_max ~ 4 k (mics at 3 m, surface at 1 m)
    mesh = api.Mesh(ctx, nodes, elems)
    r64 = api.ibem_assemble_batch(ctx, mesh, T(mics, cuda), T(ks, cuda))
    rmx = api.ibem_assemble_batch(ctx, mesh, T(mics, cuda), T(ks, cuda), api.default_config(precision=1))
    torch.cuda.synchronize()
    for a, b in zip(r64, rmx):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        for f in range(len(ks)):
            assert relerr(b[f], a[f]) < 1e-12, f


def test_mixed_assembly_geometry_table_equals_inline(cuda, ctx, monkeypatch):
    """The geometry table holds the r, 1/r and n.(x_q - x_o)/r^2 the rows
    kernel otherwise computes inline, by the same double-float operations:
    the two forms agree to double-float rounding (1e-13 of each row's largest
    entry), surface, CHIEF and field rows, evenly and unevenly spaced
    frequencies."""
    from inverseacoustics_gb300 import api
    import torch
    w = g.ibem_sphere(n_freq=64)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    ks = w.k[[0, 1, 2, 3, 17, 40, 63]]
    cp = np.array([[0.01, -0.02, 0.015], [-0.03, 0.0, 0.02]]).T.copy()
    mesh = api.Mesh(ctx, nodes, elems)
    cfg = api.default_config(precision=1)
    args = (ctx, mesh, T(mics, cuda), T(ks, cuda), cfg)
    monkeypatch.delenv("IA_ASM_GEOM_TABLE", raising=False)
    tab = api.ibem_assemble_batch(*args, cp=T(cp, cuda))
    monkeypatch.setenv("IA_ASM_GEOM_TABLE", "0")
    inl = api.ibem_assemble_batch(*args, cp=T(cp, cuda))
    torch.cuda.synchronize()
    for a, b in zip(tab, inl):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        scale = np.max(np.abs(b), axis=-1, keepdims=True)
        assert np.max(np.abs(a - b) / scale) < 1e-13
    mesh.close()


# FP64-level products of the refinement and the transfer GEMM: the
# double-float CUDA-core GEMM (0) and the tensor-core GEMM on 7 (the default)
# or 8 BF16 slices.  At 7 slices the product's own bound (8e-12 of the row and
# column maxima per term) sets the floor near 5e-11 on these operators.
SLICE_TOL = [(0, 1e-11), (7, 1e-10), (8, 1e-11)]


@pytest.mark.parametrize("slices,tol", SLICE_TOL)
def test_mixed_transfer_is_fp64_accurate(cuda, ctx, slices, tol):
    from inverseacoustics_gb300 import api
    import torch
    w = g.ibem_sphere(n_freq=64)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    ks = w.k[[2, 53, 54, 63]]          # includes the two bins next to ka = pi
    mesh = api.Mesh(ctx, nodes, elems)
    H64, i64 = api.ibem_transfer_batch(ctx, mesh, T(mics, cuda), T(ks, cuda))
    Hmx, imx = api.ibem_transfer_batch(ctx, mesh, T(mics, cuda), T(ks, cuda),
                                       api.default_config(precision=1, refine_steps=2, gemm_slices=slices))
    torch.cuda.synchronize()
    assert int(imx.abs().sum()) == 0
    errs = [relerr(Hmx[f].cpu().numpy(), H64[f].cpu().numpy()) for f in range(len(ks))]
    print(f"\nmixed transfer, {slices} slices: H vs FP64 max {max(errs):.3e}")
    assert max(errs) < tol


@pytest.mark.parametrize("slices,tol", SLICE_TOL)
def test_mixed_transfer_fp32_solve_and_refinement_steps(cuda, ctx, slices, tol):
    """The FP32 LU solve alone (refine_steps = 0) against FP64: H within the
    FP32 level (1e-4, with the sphere's condition numbers); each refinement
    step with FP64-level residuals then gains several digits (1e-8 after one,
    the product's floor after two).  Catches a wrong but refinement-masked
    FP32 solve."""
    from inverseacoustics_gb300 import api
    import torch
    w = g.ibem_sphere(n_freq=64)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    ks = w.k[[2, 30, 54]]
    mesh = api.Mesh(ctx, nodes, elems)
    H64, _ = api.ibem_transfer_batch(ctx, mesh, T(mics, cuda), T(ks, cuda))
    errs = []
    for steps in (0, 1, 2):
        H, info = api.ibem_transfer_batch(ctx, mesh, T(mics, cuda), T(ks, cuda),
                                          api.default_config(precision=1, refine_steps=steps,
                                                             gemm_slices=slices))
        torch.cuda.synchronize()
        assert int(info.abs().sum()) == 0
        errs.append(max(relerr(H[f].cpu().numpy(), H64[f].cpu().numpy()) for f in range(len(ks))))
    assert errs[0] < 1e-4 and errs[1] < 1e-8 and errs[2] < tol, errs
    assert errs[1] < 1e-2 * errs[0]


def test_mixed_ibem_pipeline_full_size(cuda, ctx):
    """Full bench configuration at 8 of its 64 frequencies (two next to the
    interior resonance): mixed x and lambda against the FP64 oracle."""
    from inverseacoustics_gb300 import api
    import torch
    w = g.ibem_sphere(n_freq=64)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    idx = [0, 9, 21, 33, 45, 53, 54, 63]
    ks = w.k[idx]
    rng = np.random.default_rng(7)
    p = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0) +
                              0.5 * g.oscillating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in ks])
    mesh = api.Mesh(ctx, nodes, elems)
    cfg = api.default_config(precision=1)
    x, lam, s, info = api.ibem_solve_batch(ctx, mesh, T(mics, cuda), T(ks, cuda), T(p, cuda), cfg)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    reg, sing = Q.builtin()
    for f in (0, 5, 6, 7):
        H = O.ibem_transfer(nodes, elems, mics, ks[f], reg, sing, 343.0, 1.21)
        xo, lo, so = O.solve_tikhonov_gcv(H, p[f, 0])
        assert abs(lam[f, 0].item() - lo) < 1e-5 * lo
        assert relerr(x[f, 0].cpu().numpy(), xo) < MIXED_TOL


def test_mixed_matches_fp64_path_all_bins(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    nodes, elems = g.icosphere(2, 0.1)
    rng = np.random.default_rng(8)
    mics = g.hemisphere_array(rng, 60, 0.3)
    ks = 2 * np.pi * np.linspace(100, 2000, 16) / 343.0
    p = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in ks])
    mesh = api.Mesh(ctx, nodes, elems)
    x6, l6, _, _ = api.ibem_solve_batch(ctx, mesh, T(mics, cuda), T(ks, cuda), T(p, cuda))
    xm, lm, _, info = api.ibem_solve_batch(ctx, mesh, T(mics, cuda), T(ks, cuda), T(p, cuda),
                                           api.default_config(precision=1))
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    for f in range(len(ks)):
        assert relerr(xm[f, 0].cpu().numpy(), x6[f, 0].cpu().numpy()) < MIXED_TOL


def test_mixed_esm_and_hels_pipelines(cuda, ctx):
    from inverseacoustics_gb300 import api
    import torch
    rng = np.random.default_rng(9)
    mics = g.planar_array(8, 8, 0.03, 0.10)
    src, _ = g.icosphere(2, 0.05)
    ks = 2 * np.pi * np.array([500.0, 1000.0, 3000.0]) / 343.0
    p = np.stack([g.add_noise(rng, O.monopole_matrix(mics, src, k) @ g.complex_normal(rng, 162), 30.0)[None, :]
                  for k in ks])
    cfg = api.default_config(precision=1, gcv_lo=1e-8, gcv_hi=1e2)
    x, lam, s, info = api.esm_solve_batch(ctx, T(mics, cuda), T(src, cuda), T(ks, cuda), T(p, cuda), cfg)
    torch.cuda.synchronize()
    for f, k in enumerate(ks):
        xo, lo, _ = O.solve_tikhonov_gcv(O.monopole_matrix(mics, src, k), p[f, 0], grid=(1e-8, 1e2))
        assert relerr(x[f, 0].cpu().numpy(), xo) < MIXED_TOL
    pts = g.cartesian_to_spherical(g.planar_array(10, 10, 0.025, 0.15))
    mic_xyz = g.planar_array(10, 10, 0.025, 0.15)
    mono = rng.normal(size=(3, 6)) * 0.03
    p = np.stack([g.add_noise(rng, O.monopole_matrix(mic_xyz, mono, k) @ g.complex_normal(rng, 6), 25.0)[None, :]
                  for k in ks])
    x, lam, s, info = api.hels_solve_batch(ctx, T(pts, cuda), 8, T(ks, cuda), T(p, cuda),
                                           api.default_config(precision=1))
    torch.cuda.synchronize()
    for f, k in enumerate(ks):
        _, He, _ = O.hels(pts, pts, k, 8, 343.0, 1.21)
        xo, lo, _ = O.solve_tikhonov_gcv(He, p[f, 0])
        assert relerr(x[f, 0].cpu().numpy(), xo) < MIXED_TOL
