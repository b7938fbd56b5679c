"""Batched uneven systems in one CUDA graph, and the autotuner."""
import numpy as np
import pytest

from oracle_cases import rel_err

pytestmark = pytest.mark.gpu


def _systems():
    from spinach_gb300 import workloads as W
    ws = W.c2()
    # one system of every dimension present (64, 256, 1024, 1156, 1789, 4096)
    seen, out = set(), []
    for w in ws:
        key = (len(w.isotopes), w.approximation)
        if key not in seen:
            seen.add(key)
            out.append(w)
    return out


def test_batch_graph_matches_single_runs(engine_lib):
    import torch
    from spinach_gb300 import batched as B, engine as E
    ws = _systems()
    bp = B.prepare(ws, n_orient=24, nsteps=96, tune=False, precision=E.FP64)
    try:
        assert sorted(set(bp.dims)) == [64, 256, 1024, 1156, 1789, 4096]
        batch = B.capture(bp, precision=E.FP64)
        for _ in range(2):                       # a graph can be replayed
            batch.launch()
            ms = batch.synchronize()
            assert ms > 0
        got = B.powder_fids(bp)
        for eng, g, dt, ns, f in zip(bp.engines, bp.grids, bp.dts, bp.nsteps, got):
            ref = eng.run(*[a.cpu().numpy() for a in g], dt, ns, precision=E.FP64).fid
            assert rel_err(f, ref) <= 1e-13
        # FP32 graph against the FP64 one
        for f in bp.fids:
            f.zero_()
        B.capture(bp, precision=E.FP32)
        bp.batch.launch()
        bp.batch.synchronize()
        for f32, f64 in zip(B.powder_fids(bp), got):
            assert rel_err(f32, f64) <= 1e-5
    finally:
        bp.close()
        torch.cuda.synchronize()


def test_autotune_keeps_results(engine_lib):
    from spinach_gb300 import batched as B, engine as E, workloads as W
    w = [x for x in _systems() if len(x.isotopes) == 5][0]          # dim 1024 full basis
    bp = B.prepare([w], n_orient=64, nsteps=256, tune=False, precision=E.FP64)
    try:
        eng, g = bp.engines[0], bp.grids[0]
        grid = [a.cpu().numpy() for a in g]
        ref = eng.run(*grid, w.dt, 256, precision=E.FP64).fid
        best = eng.autotune(g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(), 64, w.dt, 256, E.FP64)
        assert best['cluster'] in (1, 2, 4, 8) and 32 <= best['threads'] <= 512
        res = eng.run(*grid, w.dt, 256, precision=E.FP64)
        assert res.stats['cluster'] == best['cluster'] and res.stats['threads'] == best['threads']
        assert rel_err(res.fid, ref) <= 1e-10
        # the cache answers a second tuning of the same shape
        again = eng.autotune(g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(), 64, w.dt, 256, E.FP64)
        assert again == best
    finally:
        bp.close()
