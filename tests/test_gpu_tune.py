"""GPU suite: the kernel-variant autotuner.  Tuned and untuned runs of the
mixed IBEM pipeline must agree bit for bit (variants differ only in the
thread mapping), the table must fill, and a tuning file must round-trip.
The mixed pipeline's tuned GEMMs are its FP32 LU trailing updates (its
FP64-level products run on the tensor-core GEMM, which is not tuned)."""
import os

import numpy as np
import pytest

from inverseacoustics_gb300 import geometry as g

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


def test_tuned_equals_untuned(cuda, ctx, tmp_path, monkeypatch):
    from inverseacoustics_gb300 import _lib, api
    import torch
    L = _lib.lib()
    nodes, elems = g.icosphere(2, 0.1)
    rng = np.random.default_rng(31)
    mics = g.hemisphere_array(rng, 50, 0.3)
    ks = 2 * np.pi * np.linspace(200, 1500, 6) / 343.0
    p = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in ks])
    mesh = api.Mesh(ctx, nodes, elems)
    args = (T(mics, cuda), T(ks, cuda), T(p, cuda))
    cfg = api.default_config(precision=1)
    tune_file = tmp_path / "tune.txt"
    monkeypatch.setenv("IA_TUNE", "1")
    monkeypatch.setenv("IA_TUNE_FILE", str(tune_file))
    L.ia_tune_reset()
    tuned = api.ibem_solve_batch(ctx, mesh, *args, cfg)
    torch.cuda.synchronize()
    n = L.ia_tune_table_size()
    # one entry per GEMM shape of the 162-node LU's trailing updates
    assert n >= 4
    lines = tune_file.read_text().split("\n")
    assert len([x for x in lines if x.strip()]) == n
    monkeypatch.setenv("IA_TUNE", "0")
    monkeypatch.delenv("IA_TUNE_FILE")
    L.ia_tune_reset()
    plain = api.ibem_solve_batch(ctx, mesh, *args, cfg)
    torch.cuda.synchronize()
    assert L.ia_tune_table_size() == 0
    for a, b in zip(tuned, plain):
        assert torch.equal(a, b)
    # the file restores the table without timing anything
    monkeypatch.setenv("IA_TUNE_FILE", str(tune_file))
    L.ia_tune_reset()
    again = api.ibem_solve_batch(ctx, mesh, *args, cfg)
    torch.cuda.synchronize()
    assert L.ia_tune_table_size() == n
    for a, b in zip(tuned, again):
        assert torch.equal(a, b)
    monkeypatch.delenv("IA_TUNE_FILE")
    monkeypatch.setenv("IA_TUNE", "1")
    L.ia_tune_reset()
    mesh.close()


@pytest.mark.parametrize("precision,kernel_id,variant", [(1, 2, 3), (1, 2, 4), (0, 1, 3)])
def test_staged_panel_gemm_is_bitwise_the_generic_gemm(cuda, ctx, tmp_path, monkeypatch, precision, kernel_id,
                                                       variant):
    """The rank-32 updates (LU trailing updates, blocked solves; FP32 in the
    mixed path, FP64 in the FP64 path) forced onto each staged-panel variant
    through a tuning file give the untuned (variant 0) results bit for bit."""
    from inverseacoustics_gb300 import _lib, api
    import torch
    L = _lib.lib()
    nodes, elems = g.icosphere(2, 0.1)
    rng = np.random.default_rng(37)
    mics = g.hemisphere_array(rng, 50, 0.3)
    ks = 2 * np.pi * np.linspace(200, 1500, 5) / 343.0
    p = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in ks])
    mesh = api.Mesh(ctx, nodes, elems)
    args = (T(mics, cuda), T(ks, cuda), T(p, cuda))
    cfg = api.default_config(precision=precision)
    # record the keys of this workload's GEMMs
    tune_file = tmp_path / "tune.txt"
    monkeypatch.setenv("IA_TUNE", "1")
    monkeypatch.setenv("IA_TUNE_FILE", str(tune_file))
    L.ia_tune_reset()
    api.ibem_solve_batch(ctx, mesh, *args, cfg)
    torch.cuda.synchronize()
    forced, rows = 0, []
    for line in tune_file.read_text().split("\n"):
        f = line.split()
        if not f:
            continue
        kernel, opa, opb, kdim = int(f[0]), int(f[2]), int(f[3]), int(f[6])
        if kernel == kernel_id and opa == 0 and opb == 0 and kdim <= 32:   # complex, N/N, K <= 32
            f[-1] = str(variant)
            forced += 1
        rows.append(" ".join(f))
    assert forced >= 4
    forced_file = tmp_path / "forced.txt"
    forced_file.write_text("\n".join(rows) + "\n")
    monkeypatch.setenv("IA_TUNE_FILE", str(forced_file))
    L.ia_tune_reset()
    panel = api.ibem_solve_batch(ctx, mesh, *args, cfg)
    torch.cuda.synchronize()
    monkeypatch.setenv("IA_TUNE", "0")
    monkeypatch.delenv("IA_TUNE_FILE")
    L.ia_tune_reset()
    plain = api.ibem_solve_batch(ctx, mesh, *args, cfg)
    torch.cuda.synchronize()
    for a, b in zip(panel, plain):
        assert torch.equal(a, b)
    monkeypatch.setenv("IA_TUNE", "1")
    L.ia_tune_reset()
    mesh.close()
