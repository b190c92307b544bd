"""Frequency sharding across ranks (one process per GPU).

Every frequency bin is an independent problem, so a batch of F bins splits
into contiguous blocks, one per rank, with no collective on the solve path;
results come back to rank 0 by a host-side gather.  The one exchange is in the
differentiable ESM design: the microphone and retreat gradients of the global
mean loss are the sums over ranks of each rank's block gradient weighted by
its share of the terms (an all-reduce of 3 l + 2 doubles); the per-frequency
log-lambda gradients stay on the rank that owns the bin.
"""
from __future__ import annotations


def freq_block(F: int, world: int, rank: int) -> tuple[int, int]:
    """[start, stop) of rank's contiguous block; the first F % world ranks
    take one extra bin."""
    if world < 1 or not 0 <= rank < world or F < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(F, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_blocks(t, F: int, group=None):
    """Concatenate each rank's block of a per-frequency tensor (leading dim =
    its block length) along dim 0 on every rank, in rank order."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = freq_block(F, world, rank)
    if t.shape[0] != hi - lo:
        raise ValueError("tensor does not hold this rank's block")
    rows = max(freq_block(F, world, r)[1] - freq_block(F, world, r)[0] for r in range(world))
    pad = torch.zeros((rows,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    pad[: hi - lo] = t
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    out = [parts[r][: freq_block(F, world, r)[1] - freq_block(F, world, r)[0]] for r in range(world)]
    return torch.cat(out, 0)


def design_grad_allreduce(err, grad_mics, grad_retreat, grad_loglam, F: int, group=None):
    """Turn one rank's block results of the ESM design objective (err
    (F_block, R) and the gradients of its block mean) into the global mean
    loss and its gradients: returns (loss, grad_mics, grad_retreat,
    grad_loglam_block).  Tensors are modified in place where possible."""
    import torch.distributed as dist
    fb = err.shape[0]
    w = fb / float(F)
    loss = err.sum().reshape(1) / float(F * err.shape[1])
    grad_mics.mul_(w)
    grad_retreat.mul_(w)
    dist.all_reduce(loss, group=group)
    dist.all_reduce(grad_mics, group=group)
    dist.all_reduce(grad_retreat, group=group)
    return loss, grad_mics, grad_retreat, grad_loglam * w
