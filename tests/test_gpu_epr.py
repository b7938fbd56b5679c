"""GPU parity on an X-band radical ('esr' assumptions: secular electron, full
nuclear Zeeman, z* hyperfine; complex off-diagonal Liouvillian values and
electron T2) against the oracle's exact (step.m/krylov.m) branch."""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_powder, rel_err

pytestmark = pytest.mark.gpu


def test_small_radical_fp64_fp32(gpu_engine):
    w = W.c4_small()
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    g = W.zcwn_grid(w.n_orient)
    ref = oracle_powder(w, g, krylov=True)
    r64 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64)
    assert r64.stats['real_offdiag'] == 0
    assert rel_err(r64.fid, ref) <= 1e-10
    r32 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP32)
    assert rel_err(r32.fid, ref) <= 1e-5
