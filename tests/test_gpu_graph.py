"""GPU suite: CUDA graph capture and replay of a whole batched IBEM solve
(ia_capture_begin / ia_capture_end / ia_graph_launch)."""
import numpy as np
import pytest

from inverseacoustics_gb300 import geometry as g

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_matches_direct_calls(cuda, precision):
    from inverseacoustics_gb300 import api
    import torch
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ctx = api.Context(0, stream)
        nodes, elems = g.icosphere(2, 0.1)
        rng = np.random.default_rng(21)
        mics = g.hemisphere_array(rng, 60, 0.3)
        ks = 2 * np.pi * np.linspace(150, 1800, 12) / 343.0
        p1 = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in ks])
        p2 = np.stack([g.add_noise(rng, g.oscillating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :]
                       for k in ks])
        mesh = api.Mesh(ctx, nodes, elems)
        M, K, P = T(mics, cuda), T(ks, cuda), T(p1, cuda)
        cfg = api.default_config(precision=precision)
        ref1 = api.ibem_solve_batch(ctx, mesh, M, K, P, cfg)          # also sizes the workspace
        ref2 = api.ibem_solve_batch(ctx, mesh, M, K, T(p2, cuda), cfg)
        out = api.ibem_solve_outputs(mesh, M, K, P)
        n0 = ctx.launches()
        graph = ctx.capture(lambda: api.ibem_solve_batch(ctx, mesh, M, K, P, cfg, out=out))
        assert ctx.launches() - n0 == graph.kernel_count() > 20
        graph.launch()
        stream.synchronize()
        for a, b in zip(out, ref1):
            assert torch.equal(a, b)
        P.copy_(T(p2, cuda))
        graph.launch()
        graph.launch()
        stream.synchronize()
        for a, b in zip(out, ref2):
            assert torch.equal(a, b)
        graph.close()
        mesh.close()
        ctx.close()


def test_capture_refuses_to_grow_workspace(cuda):
    from inverseacoustics_gb300 import api
    from inverseacoustics_gb300._lib import IAError
    import torch
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ctx = api.Context(0, stream)
        rng = np.random.default_rng(22)
        mics = g.planar_array(8, 8, 0.03, 0.10)
        src, _ = g.icosphere(1, 0.05)
        ks = np.array([2 * np.pi * 1000 / 343.0])
        M, S, K = T(mics, cuda), T(src, cuda), T(ks, cuda)
        P = T(g.complex_normal(rng, (1, 1, 64)), cuda)
        out = (torch.empty((1, 1, 42), dtype=torch.complex128, device=cuda),
               torch.empty((1, 1), dtype=torch.float64, device=cuda),
               torch.empty((1, 42), dtype=torch.float64, device=cuda), torch.zeros(1, dtype=torch.int32, device=cuda))
        with pytest.raises(IAError) as ei:
            ctx.capture(lambda: api.esm_solve_batch(ctx, M, S, K, P, out=out))
        assert ei.value.code == 9
        x, lam, s, info = api.esm_solve_batch(ctx, M, S, K, P)      # usable afterwards
        stream.synchronize()
        assert int(info.item()) == 0 and torch.isfinite(torch.view_as_real(x)).all()
        ctx.close()
