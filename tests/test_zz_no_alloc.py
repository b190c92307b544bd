"""GPU suite, collected last: ia_solve_batch_noalloc, the allocation-free
variant of the batched SVD / GCV / Tikhonov solve.

It exists for callers that may not allocate device memory -- a real-time
acquisition loop, or code recording the solve into a CUDA graph -- and works
in a fixed static device array instead.  Two calls in a row through the C ABI
must agree with ia_solve_batch (which uses the context's allocated
workspace) within the FP64 tolerance of the other tests, and a problem larger
than the array must be refused."""
import ctypes as C

import numpy as np
import pytest

from conftest import relerr
from inverseacoustics_gb300 import geometry as g
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _problem(F=4, seed=31):
    rng = np.random.default_rng(seed)
    mics = g.planar_array(8, 8, 0.03, 0.10)
    src, _ = g.icosphere(2, 0.05)
    ks = 2 * np.pi * np.linspace(400, 2400, F) / 343.0
    H = np.stack([O.monopole_matrix(mics, src, k).T for k in ks])          # (F, n, m): column-major m x n
    b = np.stack([g.add_noise(rng, O.monopole_matrix(mics, src, k) @ g.complex_normal(rng, 162), 30.0)[None, :]
                  for k in ks])
    return np.ascontiguousarray(H), np.ascontiguousarray(b)


def _noalloc(ctx, Hd, bd, m, n, cfg):
    import torch
    from inverseacoustics_gb300 import _lib
    F, nrhs = bd.shape[0], bd.shape[1]
    x = torch.empty((F, nrhs, n), dtype=torch.complex128, device=Hd.device)
    lam = torch.empty((F, nrhs), dtype=torch.float64, device=Hd.device)
    s = torch.empty((F, min(m, n)), dtype=torch.float64, device=Hd.device)
    info = torch.zeros(F, dtype=torch.int32, device=Hd.device)
    st = _lib.lib().ia_solve_batch_noalloc(ctx.handle, m, n, F, Hd.data_ptr(), nrhs, bd.data_ptr(), C.byref(cfg),
                                           x.data_ptr(), lam.data_ptr(), s.data_ptr(), info.data_ptr())
    return st, x, lam, s, info


def test_noalloc_matches_allocating_solve_twice(cuda, ctx):
    import torch
    from inverseacoustics_gb300 import api
    H, b = _problem()
    Hd, bd = torch.as_tensor(H, device=cuda), torch.as_tensor(b, device=cuda)
    cfg = api.default_config()
    x0, l0, s0, i0 = api.solve_batch(ctx, Hd, 64, 162, bd, cfg)
    for _ in range(2):
        st, x, lam, s, info = _noalloc(ctx, Hd, bd, 64, 162, cfg)
        torch.cuda.synchronize()
        assert st == 0
        assert int(info.abs().sum()) == 0
        assert relerr(x.cpu().numpy(), x0.cpu().numpy()) < TOL
        assert relerr(lam.cpu().numpy(), l0.cpu().numpy()) < TOL
        assert relerr(s.cpu().numpy(), s0.cpu().numpy()) < TOL


def _pool_bytes(dev=0):
    """(reserved, used) bytes of the device's stream-ordered memory pool, the
    pool every cudaMallocAsync of this library draws from."""
    rt = None
    with open("/proc/self/maps") as fh:
        paths = sorted({ln.split()[-1] for ln in fh if "libcudart.so" in ln})
    for name in paths + ["libcudart.so.13", "libcudart.so.12", "libcudart.so"]:
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            continue
    assert rt is not None, "no CUDA runtime library to query the memory pool"
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), C.c_int(dev)) == 0
    out = []
    for attr in (0x5, 0x7):     # cudaMemPoolAttrReservedMemCurrent, cudaMemPoolAttrUsedMemCurrent
        v = C.c_uint64()
        assert rt.cudaMemPoolGetAttribute(pool, C.c_int(attr), C.byref(v)) == 0
        out.append(v.value)
    return tuple(out)


def test_noalloc_first_call_of_a_shape_inside_a_callers_capture(cuda, ctx):
    """A caller records the solve into its own CUDA graph, and the shape is one
    this process has never solved (the autotuner's table is emptied first):
    the capture must succeed without touching the memory pool or the tuner,
    and the replay must match the allocating entry point."""
    import torch
    from inverseacoustics_gb300 import _lib, api
    L = _lib.lib()
    cfg = api.default_config()
    H1, b1 = _problem()
    st, *_ = _noalloc(ctx, torch.as_tensor(H1, device=cuda), torch.as_tensor(b1, device=cuda), 64, 162, cfg)
    torch.cuda.synchronize()
    assert st == 0                  # the device's array address is known before the capture
    H, b = _problem(F=3, seed=47)
    b = np.ascontiguousarray(np.concatenate([b, 0.5 * b[:, :, ::-1]], axis=1))      # 2 right-hand sides
    Hd, bd = torch.as_tensor(H, device=cuda), torch.as_tensor(b, device=cuda)
    F, nrhs, m, n = 3, 2, 64, 162
    x = torch.empty((F, nrhs, n), dtype=torch.complex128, device=cuda)
    lam = torch.empty((F, nrhs), dtype=torch.float64, device=cuda)
    s = torch.empty((F, m), dtype=torch.float64, device=cuda)
    info = torch.zeros(F, dtype=torch.int32, device=cuda)
    L.ia_tune_reset()
    n_table = L.ia_tune_table_size()
    torch.cuda.synchronize()
    pool0 = _pool_bytes()
    stream = torch.cuda.Stream()
    cap = api.Context(0, stream=stream)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
        st = L.ia_solve_batch_noalloc(cap.handle, m, n, F, Hd.data_ptr(), nrhs, bd.data_ptr(), C.byref(cfg),
                                      x.data_ptr(), lam.data_ptr(), s.data_ptr(), info.data_ptr())
    assert st == 0
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        assert L.ia_tune_table_size() == n_table
        assert _pool_bytes() == pool0
        assert int(info.abs().sum()) == 0
        x0, l0, s0, _ = api.solve_batch(ctx, Hd, m, n, bd, cfg)
        torch.cuda.synchronize()
        assert relerr(x.cpu().numpy(), x0.cpu().numpy()) < TOL
        assert relerr(lam.cpu().numpy(), l0.cpu().numpy()) < TOL
        assert relerr(s.cpu().numpy(), s0.cpu().numpy()) < TOL
        # the allocating call may grow the pool and tune the shape; the next replay may do neither
        pool0 = _pool_bytes()
        n_table = L.ia_tune_table_size()
    cap.close()
    del g


def test_noalloc_refuses_problems_above_its_array(cuda, ctx):
    import torch
    from inverseacoustics_gb300 import api
    F, m, n = 64, 120, 642          # ~90 MB of scratch, above the 16 MiB array
    Hd = torch.zeros((F, n, m), dtype=torch.complex128, device=cuda)
    bd = torch.zeros((F, 1, m), dtype=torch.complex128, device=cuda)
    st, *_ = _noalloc(ctx, Hd, bd, m, n, api.default_config())
    assert st == 8
