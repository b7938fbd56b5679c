"""Multi-process orientation sharding on CPU (gloo, world size 2): each rank
computes its block of the grid (here with the FP64 oracle standing in for the
per-rank GPU), the host combines the weighted partials in rank order, and the
result equals the single-process powder sum (kernel/contexts/powder.m:280-287)."""
import os
import socket

import numpy as np
import pytest

from spinach_gb300.shard import combine_partial_fids, max_over_ranks, shard_bounds, shard_grid


def test_shard_bounds_cover_grid():
    for n in (1, 7, 200, 1001):
        for world in (1, 2, 3, 8):
            blocks = [shard_bounds(n, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(blocks[i][1] == blocks[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in blocks]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        from spinach_gb300 import workloads as W
        from oracle_cases import oracle_powder
        w = W.c0()
        grid = W.zcwn_grid(11)
        sub = shard_grid(grid, rank, world)
        fids = oracle_powder(w, sub, nsteps=40, sum_up=False)
        partial = sum(wi * f for wi, f in zip(sub[3], fids))
        total = combine_partial_fids(partial)
        slow = max_over_ranks(0.5 + rank)
        np.save(os.path.join(out_dir, f'rank{rank}.npy'), total)
        np.save(os.path.join(out_dir, f'slow{rank}.npy'), np.array([slow]))
    finally:
        dist.destroy_process_group()


def test_two_rank_powder_equals_single_process(tmp_path):
    torch = pytest.importorskip('torch')
    import torch.multiprocessing as tmp
    port = _free_port()
    tmp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    from spinach_gb300 import workloads as W
    from oracle_cases import oracle_powder
    ref = oracle_powder(W.c0(), W.zcwn_grid(11), nsteps=40)
    for r in range(2):
        got = np.load(tmp_path / f'rank{r}.npy')
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-13
        assert float(np.load(tmp_path / f'slow{r}.npy')[0]) == 1.5
    del torch
