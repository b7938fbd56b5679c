"""GPU parity on the configurations the metric is quoted on, against the FP64
oracle fixtures of tests/golden/make_golden.py ('wide'):

* c1 (IK-0(3), dim 1156, T1/T2, 2048 steps): the whole 1000-orientation powder
  FID and 32 per-orientation FIDs spread over the grid (Krylov branch,
  kernel/krylov.m + step.m, summed in grid order as powder.m:280-287);
* c1 against the reference's DEFAULT propagator branch (propagator.m:64-201,
  then P*rho, evolution.m:563-566) run with prop_chop = eps, the 'paranoia'
  tolerances of kernel/utilities/tolerances.m:97-100, at two orientations: the
  chop quantisation is then below the bar, so the propagator branch itself is
  held to 1e-10;
* c4 (EPR radical, IK-1(3), dim 2736, 4096 steps): the whole 4000-orientation
  powder FID and 24 orientations;
* c2: four orientations of one system of every dimension (64, 256, 1024,
  1156, 1789, 4096), and the whole 400-orientation powder of each of those
  six systems through the batched graph with on-GPU construction.

Bars (relative 2-norm error, tests/lib/test_close.m metric): FP64 <= 1e-10,
FP32 <= 1e-5.
"""
import os

import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import rel_err

GOLD = os.path.join(os.path.dirname(__file__), 'golden')
FP64_TOL = 1e-10
FP32_TOL = 1e-5

pytestmark = pytest.mark.gpu


def _upload(eng, w):
    L = W.build(w)
    eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    return L


def _check_orientations(eng, w, gold, label):
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = gold['sel']
    wt = np.full(sel.size, 1.0 / sel.size)
    for prec, tol in ((E.FP64, FP64_TOL), (E.FP32, FP32_TOL)):
        res = eng.run(al[sel], be[sel], ga[sel], wt, w.dt, int(gold['nsteps']), precision=prec, per_orientation=True)
        errs = [rel_err(res.fids[i], gold['fids'][i]) for i in range(sel.size)]
        assert max(errs) <= tol, (label, prec, int(np.argmax(errs)), max(errs))


def test_c1_whole_powder_vs_oracle(gpu_engine):
    """The number the metric is about: the 1000-orientation c1 powder FID."""
    w = W.c1()
    _upload(gpu_engine, w)
    gold = np.load(os.path.join(GOLD, 'c1_powder_krylov_fp64.npz'))
    g = W.zcwn_grid(w.n_orient)
    r64 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64)
    assert rel_err(r64.fid, gold['fid']) <= FP64_TOL
    r32 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP32)
    assert rel_err(r32.fid, gold['fid']) <= FP32_TOL
    assert r64.stats['orientations_failed'] == 0 and r32.stats['orientations_failed'] == 0


def test_c1_thirty_two_orientations(gpu_engine):
    w = W.c1()
    _upload(gpu_engine, w)
    _check_orientations(gpu_engine, w, np.load(os.path.join(GOLD, 'c1_powder_krylov_fp64.npz')), 'c1')


def test_c1_default_propagator_branch_at_paranoia_chop(gpu_engine):
    """propagator.m's chopped Taylor + squaring branch with prop_chop = eps:
    the GPU's FP64 FIDs are within 1e-10 of it (with the default prop_chop =
    1e-10 the branch itself moves the FID by 3e-7, see test_gpu_parity)."""
    w = W.c1()
    _upload(gpu_engine, w)
    _check_orientations(gpu_engine, w, np.load(os.path.join(GOLD, 'c1_orient_propagator_paranoia_fp64.npz')),
                        'c1 propagator branch')


def test_c4_whole_powder_vs_oracle(gpu_engine):
    """Config 4's powder FID (4000 orientations x 4096 steps)."""
    w = W.c4()
    _upload(gpu_engine, w)
    gold = np.load(os.path.join(GOLD, 'c4_powder_krylov_fp64.npz'))
    g = W.zcwn_grid(w.n_orient)
    r64 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64)
    assert rel_err(r64.fid, gold['fid']) <= FP64_TOL
    r32 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP32)
    assert rel_err(r32.fid, gold['fid']) <= FP32_TOL


def test_c4_twenty_four_orientations(gpu_engine):
    w = W.c4()
    _upload(gpu_engine, w)
    _check_orientations(gpu_engine, w, np.load(os.path.join(GOLD, 'c4_orients_krylov_fp64.npz')), 'c4')


C2_DIMS = [64, 256, 1024, 1156, 1789, 4096]


@pytest.mark.parametrize('dim', C2_DIMS)
def test_c2_every_dimension_four_orientations(gpu_engine, dim):
    gold = np.load(os.path.join(GOLD, f'c2_dim{dim}_krylov_fp64.npz'))
    w = W.c2()[int(gold['system'])]
    L = _upload(gpu_engine, w)
    assert L.dim == dim
    _check_orientations(gpu_engine, w, gold, f'c2 dim {dim}')


def test_c2_whole_powders_through_the_batched_graph(engine_lib):
    """The c2 path itself (on-GPU construction of I and Q, one CUDA graph over
    the systems) against the oracle's whole 400-orientation powders of one
    system of every dimension, FP64 and FP32."""
    import torch
    from spinach_gb300 import batched as B
    golds = [np.load(os.path.join(GOLD, f'c2_dim{d}_krylov_fp64.npz')) for d in C2_DIMS]
    ws = W.c2()
    bp = B.prepare([ws[int(g['system'])] for g in golds], tune=False, precision=E.FP64)
    try:
        assert bp.dims == C2_DIMS
        for prec, tol in ((E.FP64, FP64_TOL), (E.FP32, FP32_TOL)):
            for f in bp.fids:
                f.zero_()
            B.capture(bp, precision=prec)
            bp.batch.launch()
            bp.batch.synchronize()
            for d, f, g in zip(bp.dims, B.powder_fids(bp), golds):
                assert rel_err(f, g['fid']) <= tol, (d, prec, rel_err(f, g['fid']))
    finally:
        bp.close()
        torch.cuda.synchronize()
