"""Frequency sharding over ranks, run as world_size-2 gloo process groups on
the CPU.  The per-rank compute stands in for the GPU kernels with the oracle
(the kernels need a GPU); what is under test is the host logic: the
contiguous blocks, the gather in rank order, and the weighted all-reduce of
the design gradients, which must reproduce the unsharded result."""
import os
import socket

import numpy as np
import pytest

from inverseacoustics_gb300.shard import freq_block


def test_freq_block_partition():
    for F in (0, 1, 7, 64, 129):
        for world in (1, 2, 3, 8):
            blocks = [freq_block(F, world, r) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == F
            assert all(blocks[r][1] == blocks[r + 1][0] for r in range(world - 1))
            sizes = [b - a for a, b in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        freq_block(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, queue):
    import torch
    import torch.distributed as dist
    from inverseacoustics_gb300.shard import design_grad_allreduce, freq_block, gather_blocks
    from tests.test_oracle import _design_case
    from oracle import ia_oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mics, surf, d, k, ll, q, noise = _design_case(seed=3, l=10, subdiv=1, F=5, R=3)
        F = len(k)
        lo, hi = freq_block(F, world, rank)
        sl = slice(lo, hi)
        err = torch.tensor(O.esm_design_terms(mics, surf, d, k[sl], ll[sl], q[sl], noise[sl]))
        gm, gd, gl = O.esm_design_grad(mics, surf, d, k[sl], ll[sl], q[sl], noise[sl])
        loss, gm_t, gd_t, gl_t = design_grad_allreduce(err, torch.tensor(gm), torch.tensor([gd], dtype=torch.float64),
                                                       torch.tensor(gl), F)
        all_err = gather_blocks(err, F)
        all_gl = gather_blocks(gl_t, F)
        if rank == 0:
            queue.put((float(loss.item()), gm_t.numpy(), float(gd_t.item()), all_gl.numpy(), all_err.numpy()))
    finally:
        dist.destroy_process_group()


def test_sharded_design_gradient_matches_unsharded():
    import torch.multiprocessing as mp
    from oracle import ia_oracle as O
    from tests.test_oracle import _design_case
    world = 2
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        loss, gm, gd, gl, err = queue.get(timeout=120)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    mics, surf, d, k, ll, q, noise = _design_case(seed=3, l=10, subdiv=1, F=5, R=3)
    e0 = O.esm_design_terms(mics, surf, d, k, ll, q, noise)
    gm0, gd0, gl0 = O.esm_design_grad(mics, surf, d, k, ll, q, noise)
    assert abs(loss - e0.mean()) <= 1e-14 * e0.mean()
    assert np.allclose(err, e0, rtol=1e-14, atol=0)
    assert np.allclose(gm, gm0, rtol=1e-12, atol=1e-14 * np.abs(gm0).max())
    assert abs(gd - gd0) <= 1e-12 * abs(gd0)
    assert np.allclose(gl, gl0, rtol=1e-12, atol=0)
