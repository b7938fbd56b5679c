"""Every FP32 result states its error against FP64: spx_run_powder and
spx_run_powder_device re-run two orientations of an FP32 run in FP64 on a
second stream and report the measured per-orientation error and the error it
implies for the powder FID; above half of 1e-5 (the bar of the metric, with a
margin for an estimate drawn from two orientations) spx_run_powder returns an
FP64 re-run of the whole grid instead.

FP32's error grows with the length of an undamped acquisition (the rounding of
the stored vectors acts like a small frequency error): the c0 system (no
relaxation) crosses 1e-5 near 16k steps, while the relaxing c1 system stays
near 2e-7 at its own 2048 steps.
"""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import rel_err

pytestmark = pytest.mark.gpu


def _upload(eng, w):
    L = W.build(w)
    eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)


def test_c1_states_its_error_and_keeps_fp32(gpu_engine):
    w = W.c1()
    _upload(gpu_engine, w)
    g = W.zcwn_grid(w.n_orient)
    r32 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP32)
    st = r32.stats
    assert st['fp32_checked'] == 2 and st['promoted_fp64'] == 0 and st['precision'] == E.FP32
    r64 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64)
    actual = rel_err(r32.fid, r64.fid)
    assert actual <= 1e-6
    # the stated powder error is of the right size, and below the bar
    assert 0.2 * actual <= st['fp32_powder_error'] <= 5 * actual + 1e-8, (st['fp32_powder_error'], actual)
    assert st['fp32_powder_error'] < 0.5 * E.FP32_ERROR_BAR and st['fp32_rel_error'] < E.FP32_ERROR_BAR


@pytest.mark.parametrize('nsteps', [1024, 4096])
def test_c0_stated_error_tracks_the_measured_one(gpu_engine, nsteps):
    w = W.c0()
    _upload(gpu_engine, w)
    g = W.zcwn_grid(w.n_orient)
    r32 = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP32, promote=False)
    r64 = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP64)
    actual = rel_err(r32.fid, r64.fid)
    est = r32.stats['fp32_powder_error']
    assert 0.5 * actual <= est <= 2 * actual, (est, actual)


def test_c0_long_undamped_run_is_promoted_to_fp64(gpu_engine):
    """16384 undamped steps: FP32 misses the bar, so the returned powder FID
    is the FP64 one."""
    w = W.c0()
    _upload(gpu_engine, w)
    g = W.zcwn_grid(w.n_orient)
    nsteps = 16384
    r64 = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP64)
    kept = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP32, promote=False)
    actual = rel_err(kept.fid, r64.fid)
    assert kept.stats['promoted_fp64'] == 0 and actual > 1e-5
    assert 0.5 * actual <= kept.stats['fp32_powder_error'] <= 2 * actual
    res = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP32)
    assert res.stats['promoted_fp64'] == 1 and res.stats['precision'] == E.FP64
    assert res.stats['fp32_powder_error'] > 0.5 * E.FP32_ERROR_BAR
    assert rel_err(res.fid, r64.fid) <= 1e-13


def test_check_can_be_switched_off_and_runs_on_device_buffers(gpu_engine):
    import torch
    w = W.c0()
    _upload(gpu_engine, w)
    grid = W.zcwn_grid(w.n_orient)
    off = gpu_engine.run(*grid, w.dt, 512, precision=E.FP32, fp32_check=False)
    assert off.stats['fp32_checked'] == 0 and off.stats['fp32_rel_error'] == 0.0
    on = gpu_engine.run(*grid, w.dt, 512, precision=E.FP32)
    assert np.array_equal(on.fid, off.fid)            # the check leaves the FP32 result as it is
    dev = torch.device('cuda', 0)
    g = torch.tensor(np.stack(grid), dtype=torch.float64, device=dev).contiguous()
    out = torch.zeros(2 * 513, dtype=torch.float64, device=dev)
    gpu_engine.run_device(*[g[i].data_ptr() for i in range(4)], w.n_orient, w.dt, 512, out.data_ptr(),
                          precision=E.FP32)
    st = gpu_engine.stats()
    assert st['fp32_checked'] == 2 and 0 < st['fp32_powder_error'] < 1e-5
    assert np.array_equal(out.cpu().numpy().view(np.complex128), on.fid)
