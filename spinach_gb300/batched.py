"""Batched powders of many spin systems of uneven Liouville dimension.

Every system gets its own engine handle (uploaded Liouvillian, device-resident
grid and output).  The autotuner (spx_autotune) picks each system's launch
shape -- CTAs per orientation, warps, series length per chunk -- once per
system shape, and one CUDA graph (spx_batch_*) holds every system's launches
on parallel branches, so a whole batch is one graph launch.  The reference
runs such systems one powder() call at a time (kernel/contexts/powder.m).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import engine as E
from . import workloads as W


@dataclass
class BatchedPowders:
    engines: list
    grids: list                 # per system: (alphas, betas, gammas, weights) on the device (torch)
    fids: list                  # per system: device output (torch float64, 2*(nsteps+1))
    dts: list
    nsteps: list
    dims: list
    tuned: list = field(default_factory=list)
    setup_s: float = 0.0
    tune_s: float = 0.0
    batch: object = None

    def close(self):
        if self.batch is not None:
            self.batch.close()
            self.batch = None
        for e in self.engines:
            e.close()


def prepare(workloads, n_orient=None, nsteps=None, device: int = 0, tune: bool = True,
            precision: int = E.FP32, builder: str = 'gpu') -> BatchedPowders:
    """Build, upload and (optionally) autotune every system.  ``builder``
    'gpu' constructs I and Q on the device (Engine.build_system), 'host' with
    the host builder (Engine.upload)."""
    import torch
    if builder not in ('gpu', 'host'):
        raise ValueError("builder must be 'gpu' or 'host'")
    dev = torch.device('cuda', device)
    t0 = time.perf_counter()
    engines, grids, fids, dts, nss, dims = [], [], [], [], [], []
    for w in workloads:
        eng = E.Engine(device)
        if builder == 'gpu':
            L = W.build_spec(w)
            eng.build_system(L.monomials, L.r_diag, L.rho0, L.coil)
        else:
            L = W.build(w)
            eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
        no = n_orient or w.n_orient
        ns = nsteps or w.nsteps
        g = torch.tensor(np.stack(W.zcwn_grid(no)), dtype=torch.float64, device=dev).contiguous()
        engines.append(eng)
        grids.append(g)
        fids.append(torch.zeros(2 * (ns + 1), dtype=torch.float64, device=dev))
        dts.append(w.dt)
        nss.append(ns)
        dims.append(L.dim)
    setup = time.perf_counter() - t0
    tuned = []
    t0 = time.perf_counter()
    if tune:
        for eng, g, dt, ns in zip(engines, grids, dts, nss):
            tuned.append(eng.autotune(g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(), g.shape[1], dt, ns,
                                      precision))
    return BatchedPowders(engines, grids, fids, dts, nss, dims, tuned, setup, time.perf_counter() - t0)


def capture(bp: BatchedPowders, precision: int = E.FP32) -> E.Batch:
    """One graph over every system (replaces a previous one)."""
    if bp.batch is not None:
        bp.batch.close()
    runs = [(eng, g.shape[1], g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(), g[3].data_ptr(), dt, ns,
             f.data_ptr(), precision)
            for eng, g, f, dt, ns in zip(bp.engines, bp.grids, bp.fids, bp.dts, bp.nsteps)]
    bp.batch = E.Batch(runs)
    return bp.batch


def powder_fids(bp: BatchedPowders) -> list:
    """Host copies of every system's powder FID (complex128)."""
    return [f.cpu().numpy().view(np.complex128).copy() for f in bp.fids]
