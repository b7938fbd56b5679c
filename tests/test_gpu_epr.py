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


def test_radical_with_14n_quadratic_coupling(gpu_engine):
    """The nitrogen's quadratic coupling in full ('strong' under 'esr': five
    T(2,m) terms) on the small radical, built on the host and on the GPU."""
    w = W.c4_small()
    w.coupling_eigs = dict(w.coupling_eigs)
    w.coupling_euler = dict(w.coupling_euler)
    w.coupling_eigs[(1, 1)] = [-0.4e6, -0.6e6, 1.0e6]
    w.coupling_euler[(1, 1)] = [0.2, 0.9, 1.7]
    g = W.zcwn_grid(w.n_orient)
    ref = oracle_powder(w, g, krylov=True)
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    assert rel_err(gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64).fid, ref) <= 1e-10
    assert rel_err(gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP32).fid, ref) <= 1e-5
    bs = W.build_spec(w)
    gpu_engine.build_system(bs.monomials, bs.r_diag, bs.rho0, bs.coil)
    assert rel_err(gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64).fid, ref) <= 1e-10
