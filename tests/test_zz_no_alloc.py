"""spx_run_powder_noalloc: the entry point for callers that cannot allocate
device memory while they run (hosts that reserve all GPU memory up front, code
that must avoid the device-wide synchronisation of cudaMalloc/cudaFree).  Its
intermediates live in the library's static device array.  These tests check
its FIDs against the allocating entry point on two calls in a row (one
channel, two channels, per-orientation initial states), that repeated calls
leave the device's free memory unchanged, and that a run larger than the array
is refused before any work is queued.
"""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W

pytestmark = pytest.mark.gpu

TOL = {E.FP64: 1e-10, E.FP32: 1e-5}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _device_grid(grid):
    import torch
    g = torch.tensor(np.stack(grid), dtype=torch.float64, device=torch.device('cuda', 0)).contiguous()
    return g, [g[i].data_ptr() for i in range(4)]


def _noalloc(eng, ptr, n_orient, dt, nsteps, nchan, prec):
    import torch
    out = torch.full((2 * (nsteps + 1) * nchan,), float('nan'), dtype=torch.float64,
                     device=torch.device('cuda', 0))
    torch.cuda.synchronize()
    eng.run_noalloc(ptr[0], ptr[1], ptr[2], ptr[3], n_orient, dt, nsteps, out.data_ptr(), precision=prec)
    fid = out.cpu().numpy().view(np.complex128)
    return fid.reshape(nchan, nsteps + 1) if nchan > 1 else fid


def _check_two_calls(eng, grid, dt, nsteps, nchan=1):
    g, ptr = _device_grid(grid)
    n = len(grid[0])
    for prec in (E.FP64, E.FP32):
        ref = eng.run(*grid, dt, nsteps, precision=prec).fid
        for call in range(2):
            fid = _noalloc(eng, ptr, n, dt, nsteps, nchan, prec)
            assert np.all(np.isfinite(fid)), (prec, call)
            assert _rel(fid, ref) <= TOL[prec], (prec, call, _rel(fid, ref))


def test_noalloc_matches_allocating_entry_point():
    w = W.c0()
    L = W.build(w)
    eng = E.Engine(0)
    try:
        eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
        _check_two_calls(eng, W.zcwn_grid(w.n_orient), w.dt, w.nsteps)
    finally:
        eng.close()


def test_noalloc_two_channels_and_per_orientation_states():
    from spinach_gb300 import spin_system as S
    w = W.c0()
    L = W.build(w)
    ss = W.spin_system_of(w)
    fac = S.factory_for(ss, S.build_basis(ss, w.approximation, w.level))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([3, 40, 99, 150, 180])
    grid = (al[sel], be[sel], ga[sel], np.array([0.1, 0.3, 0.2, 0.25, 0.15]))
    eng = E.Engine(0)
    try:
        eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
        eng.upload_coils([fac.state('L+', '13C'), fac.state('Lx', '13C')])
        _check_two_calls(eng, grid, w.dt, 300, nchan=2)
        eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
        states = np.cos(grid[1])[:, None] * fac.state('Lx', '13C') + np.sin(grid[2])[:, None] * fac.state('Lz', '1H')
        eng.set_initial_states(states)
        _check_two_calls(eng, grid, w.dt, 300)
    finally:
        eng.close()


def test_noalloc_leaves_free_device_memory_unchanged():
    import torch
    w = W.c0()
    L = W.build(w)
    grid = W.zcwn_grid(w.n_orient)
    eng = E.Engine(0)
    try:
        eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
        g, ptr = _device_grid(grid)
        out = torch.zeros(2 * (w.nsteps + 1), dtype=torch.float64, device=torch.device('cuda', 0))
        torch.cuda.synchronize()
        eng.run_noalloc(ptr[0], ptr[1], ptr[2], ptr[3], w.n_orient, w.dt, w.nsteps, out.data_ptr(),
                        precision=E.FP32)                   # warm-up: module and kernel loading
        free0 = torch.cuda.mem_get_info(0)[0]
        for prec in (E.FP32, E.FP64, E.FP32):
            eng.run_noalloc(ptr[0], ptr[1], ptr[2], ptr[3], w.n_orient, w.dt, w.nsteps, out.data_ptr(),
                            precision=prec)
        assert torch.cuda.mem_get_info(0)[0] == free0
    finally:
        eng.close()


def test_noalloc_refuses_runs_beyond_its_scratch():
    import torch
    w = W.c0()
    L = W.build(w)
    eng = E.Engine(0)
    try:
        eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
        n = 40000                     # 40000 orientations x 2049 points do not fit 64 MiB
        dev = torch.device('cuda', 0)
        g = torch.zeros((4, n), dtype=torch.float64, device=dev)
        out = torch.zeros(2 * 2049, dtype=torch.float64, device=dev)
        with pytest.raises(E.SpxError) as err:
            eng.run_noalloc(g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(), g[3].data_ptr(), n,
                            w.dt, 2048, out.data_ptr(), precision=E.FP64)
        assert 'bytes of scratch' in str(err.value)
    finally:
        eng.close()
