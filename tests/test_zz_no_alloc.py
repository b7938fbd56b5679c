"""spx_run_powder_noalloc: the entry point for callers that cannot allocate device
memory while they run (hosts that reserve all GPU memory up front, code that
must avoid the device-wide synchronisation of cudaMalloc/cudaFree).  Its
intermediates live in the library's static device array; this test checks its
FID against the allocating entry point on two calls in a row, and that a run
larger than the array is refused before any work is queued.
"""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W

pytestmark = pytest.mark.gpu

TOL = {E.FP64: 1e-10, E.FP32: 1e-5}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_allocating_entry_point():
    import torch
    w = W.c0()
    L = W.build(w)
    grid = W.zcwn_grid(w.n_orient)
    eng = E.Engine(0)
    try:
        eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
        dev = torch.device('cuda', 0)
        g = torch.tensor(np.stack(grid), dtype=torch.float64, device=dev).contiguous()
        ptr = [g[i].data_ptr() for i in range(4)]
        for prec in (E.FP64, E.FP32):
            ref = eng.run(*grid, w.dt, w.nsteps, precision=prec).fid
            for call in range(2):
                out = torch.full((2 * (w.nsteps + 1),), float('nan'), dtype=torch.float64, device=dev)
                torch.cuda.synchronize()
                eng.run_noalloc(ptr[0], ptr[1], ptr[2], ptr[3], w.n_orient, w.dt, w.nsteps,
                                out.data_ptr(), precision=prec)
                fid = out.cpu().numpy().view(np.complex128)
                assert np.all(np.isfinite(fid)), (prec, call)
                assert _rel(fid, ref) <= TOL[prec], (prec, call, _rel(fid, ref))
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
