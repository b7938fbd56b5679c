"""Orientation sharding across processes (one GPU each).

Orientations of a powder grid are independent (kernel/contexts/powder.m:226
runs them in a parfor); the only cross-orientation operation is the weighted
sum of the FIDs (powder.m:280-287).  A multi-process run therefore gives each
rank a contiguous block of the grid, runs it on its own GPU, and combines the
per-rank weighted partial sums on the host in rank order (FP64).  No data-path
collective is needed on the device; the host reduction goes through
``torch.distributed`` (gloo) when a process group exists.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n_orient: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous block [lo, hi) of orientations owned by ``rank`` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError('bad rank/world')
    base, extra = divmod(n_orient, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def shard_grid(grid, rank: int, world: int):
    """The (alphas, betas, gammas, weights) arrays of one rank's block."""
    al, be, ga, w = (np.asarray(a) for a in grid)
    lo, hi = shard_bounds(al.size, rank, world)
    return al[lo:hi], be[lo:hi], ga[lo:hi], w[lo:hi]


def combine_partial_fids(partial: np.ndarray, group=None) -> np.ndarray:
    """Sum every rank's weighted partial FID (complex128) in rank order.

    All ranks receive the result.  Partials are gathered, then added 0, 1, 2, ...
    so the FP64 rounding does not depend on arrival order."""
    import torch
    import torch.distributed as dist
    part = np.ascontiguousarray(partial, dtype=np.complex128)
    if not dist.is_available() or not dist.is_initialized():
        return part.copy()
    world = dist.get_world_size(group)
    t = torch.from_numpy(part.view(np.float64).copy())
    bufs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(bufs, t, group=group)
    out = np.zeros_like(part)
    for b in bufs:
        out = out + b.numpy().view(np.complex128)
    return out


def max_over_ranks(seconds: float, group=None) -> float:
    """Slowest rank's time (the whole-job time of a weakly scaled run)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t[0])
