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
