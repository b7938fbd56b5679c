"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances (relative 2-norm error of the FID, the metric of the reference's
tests/lib/test_close.m): FP64 path <= 1e-10, FP32 path <= 1e-5.
"""
import os

import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_powder, rel_err

GOLD = os.path.join(os.path.dirname(__file__), 'golden')
FP64_TOL = 1e-10
FP32_TOL = 1e-5

pytestmark = pytest.mark.gpu


def _upload(eng, w):
    L = W.build(w)
    eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    return L


def test_c0_full_powder_fp64_and_fp32(gpu_engine):
    """Config c0 (dim 64, 200 orientations, 1024 steps) vs the oracle's expm branch."""
    w = W.c0()
    _upload(gpu_engine, w)
    g = W.zcwn_grid(w.n_orient)
    ref = np.load(os.path.join(GOLD, 'c0_powder_fp64.npz'))['fid']
    r64 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64)
    assert rel_err(r64.fid, ref) <= FP64_TOL
    r32 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP32)
    assert rel_err(r32.fid, ref) <= FP32_TOL
    assert r64.stats['orientations_failed'] == 0 and r32.stats['matvecs'] > 0


def test_deuterium_powder_fp64_and_fp32(gpu_engine):
    """Static 2H powder pattern (quadratic coupling T(2,0), dim 144, 400
    orientations, 1024 steps) vs the oracle's expm branch."""
    w = W.deuterium()
    _upload(gpu_engine, w)
    g = W.zcwn_grid(w.n_orient)
    ref = np.load(os.path.join(GOLD, 'deuterium_powder_fp64.npz'))['fid']
    r64 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP64)
    assert rel_err(r64.fid, ref) <= FP64_TOL
    r32 = gpu_engine.run(*g, w.dt, w.nsteps, precision=E.FP32)
    assert rel_err(r32.fid, ref) <= FP32_TOL


def test_c1_orientations_vs_krylov_branch(gpu_engine):
    """Config c1 (IK-0(3), dim 1156, T1/T2, 2048 steps), per orientation, vs step.m/krylov.m."""
    w = W.c1()
    _upload(gpu_engine, w)
    gold = np.load(os.path.join(GOLD, 'c1_orient_krylov_fp64.npz'))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = gold['sel']
    wt = np.full(sel.size, 1.0 / sel.size)
    for prec, tol in ((E.FP64, FP64_TOL), (E.FP32, FP32_TOL)):
        res = gpu_engine.run(al[sel], be[sel], ga[sel], wt, w.dt, w.nsteps, precision=prec, per_orientation=True)
        for i in range(sel.size):
            assert rel_err(res.fids[i], gold['fids'][i]) <= tol, (prec, i)
        assert rel_err(res.fid, gold['fids'].mean(axis=0)) <= tol


def test_c1_vs_default_propagator_branch(gpu_engine):
    """The reference's default (chopped) propagator branch differs from the exact
    branches by its prop_chop quantisation; the GPU result sits within 1e-6 of it."""
    w = W.c1()
    _upload(gpu_engine, w)
    gold = np.load(os.path.join(GOLD, 'c1_orient_propagator_fp64.npz'))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    s = gold['sel']
    res = gpu_engine.run(al[s], be[s], ga[s], np.ones(1), w.dt, w.nsteps, precision=E.FP64)
    assert rel_err(res.fid, gold['fids'][0]) <= 1e-6


def test_per_orientation_outputs_and_weights(gpu_engine):
    """sum_up=false outputs (powder.m:291-297) and the weighted sum (powder.m:280-287)."""
    w = W.c0()
    _upload(gpu_engine, w)
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([3, 17, 101, 150, 199])
    wt = np.array([0.1, 0.3, 0.2, 0.25, 0.15])
    ref = oracle_powder(w, (al[sel], be[sel], ga[sel], wt), nsteps=300, sum_up=False)
    res = gpu_engine.run(al[sel], be[sel], ga[sel], wt, w.dt, 300, precision=E.FP64, per_orientation=True)
    for i in range(sel.size):
        assert rel_err(res.fids[i], ref[i]) <= FP64_TOL
    assert rel_err(res.fid, sum(wi * f for wi, f in zip(wt, ref))) <= FP64_TOL


@pytest.mark.parametrize('nsteps', [0, 1, 2, 7, 63, 64, 65])
def test_step_counts_and_chunk_edges(gpu_engine, nsteps):
    """Ragged chunk edges: nsteps+1 not a multiple of the chunk length."""
    w = W.c0()
    _upload(gpu_engine, w)
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([5, 77])
    ref = oracle_powder(w, (al[sel], be[sel], ga[sel], np.array([0.5, 0.5])), nsteps=nsteps)
    res = gpu_engine.run(al[sel], be[sel], ga[sel], np.array([0.5, 0.5]), w.dt, nsteps,
                         precision=E.FP64, chunk_steps=16)
    assert res.fid.shape == (nsteps + 1,)
    assert rel_err(res.fid, ref) <= FP64_TOL


def test_zero_hamiltonian_constant_fid(gpu_engine):
    """tests/kernel/test_liquid_single_spin_fid.m: a zero-offset spin has a constant FID."""
    import scipy.sparse as sp
    from spinach_gb300 import spin_system as S
    ss = S.make_spin_system(['1H'], 14.1)
    b = S.build_basis(ss)
    f = S.OperatorFactory(ss, b)
    H = S.rotational_hamiltonian(ss, b, 'nmr', f)
    rho = f.state('L+', '1H')
    gpu_engine.upload(H.iso, H.aniso, None, rho, rho)
    res = gpu_engine.run([0.0], [0.0], [0.0], [1.0], 1e-3, 7, precision=E.FP64)
    assert np.allclose(res.fid, res.fid[0] * np.ones(8), rtol=1e-12, atol=1e-12)
    assert abs(res.fid[0] - np.vdot(rho, rho)) < 1e-12
    del sp


def test_invalid_inputs_raise(gpu_engine):
    w = W.c0()
    _upload(gpu_engine, w)
    with pytest.raises(E.SpxError):
        gpu_engine.run([0.0], [np.nan], [0.0], [1.0], w.dt, 4)
    with pytest.raises(E.SpxError):
        gpu_engine.run([0.0], [0.1], [0.0], [1.0], -1.0, 4)
    with pytest.raises(E.SpxError):
        gpu_engine.run([0.0], [0.1], [0.0], [1.0], 1e3, 4)    # |L dt| too large


def test_frequency_offsets(gpu_engine):
    """powder.m's frqoffset: offsets on both isotopes, host and GPU builders."""
    import copy
    w = copy.deepcopy(W.c0())
    w.extra['offset'] = {'13C': 1500.0, '1H': -300.0}
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([2, 50, 123, 177])
    g = (al[sel], be[sel], ga[sel], np.full(sel.size, 0.25))
    ref = oracle_powder(w, g, nsteps=400)
    _upload(gpu_engine, w)
    assert rel_err(gpu_engine.run(*g, w.dt, 400, precision=E.FP64).fid, ref) <= FP64_TOL
    assert rel_err(gpu_engine.run(*g, w.dt, 400, precision=E.FP32).fid, ref) <= FP32_TOL
    bs = W.build_spec(w)
    gpu_engine.build_system(bs.monomials, bs.r_diag, bs.rho0, bs.coil)
    assert rel_err(gpu_engine.run(*g, w.dt, 400, precision=E.FP64).fid, ref) <= FP64_TOL


def test_isotropic_damping(gpu_engine):
    """relaxation.m 'damp' with T1/T2 on the c0 system."""
    import copy
    w = copy.deepcopy(W.c0())
    rng = np.random.default_rng(4)
    w.r1, w.r2 = list(rng.uniform(1, 5, 3)), list(rng.uniform(5, 20, 3))
    w.extra['damp_rate'] = 37.0
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([9, 88, 140])
    g = (al[sel], be[sel], ga[sel], np.full(sel.size, 1 / 3))
    ref = oracle_powder(w, g, nsteps=600)
    _upload(gpu_engine, w)
    assert rel_err(gpu_engine.run(*g, w.dt, 600, precision=E.FP64).fid, ref) <= FP64_TOL
    assert rel_err(gpu_engine.run(*g, w.dt, 600, precision=E.FP32).fid, ref) <= FP32_TOL


@pytest.mark.parametrize('extra', [{'decouple': ['1H']}, {'homodec': ('Lx', '1H', 2500.0)}])
def test_acquire_options(gpu_engine, extra):
    """acquire.m's decoupling (:51, as a smaller basis) and homodecoupling (:54-62)."""
    import copy
    w = copy.deepcopy(W.c0())
    w.extra.update(extra)
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([4, 77, 150])
    g = (al[sel], be[sel], ga[sel], np.full(sel.size, 1 / 3))
    ref = oracle_powder(w, g, nsteps=300)
    _upload(gpu_engine, w)
    assert rel_err(gpu_engine.run(*g, w.dt, 300, precision=E.FP64).fid, ref) <= FP64_TOL
    assert rel_err(gpu_engine.run(*g, w.dt, 300, precision=E.FP32).fid, ref) <= FP32_TOL
    bs = W.build_spec(w)
    gpu_engine.build_system(bs.monomials, bs.r_diag, bs.rho0, bs.coil)
    assert rel_err(gpu_engine.run(*g, w.dt, 300, precision=E.FP64).fid, ref) <= FP64_TOL


def test_dead_time_as_a_program(gpu_engine):
    """acquire.m:65-67 (rho0 <- step(L, rho0, dead_time)) as a silent one-step segment."""
    from oracle_cases import oracle_system
    from oracle import spinach_ref as R
    w = W.c0()
    ss, I, Q = oracle_system(w)
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([11, 99])
    g = (al[sel], be[sel], ga[sel], np.array([0.4, 0.6]))
    dead = 23.7e-6
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=201, dead_time=dead)
    ref = sum(g[3][i] * R.powder_orientation_fid(ss, I, Q, par, (g[0][i], g[1][i], g[2][i])) for i in range(2))
    _upload(gpu_engine, w)
    res = gpu_engine.run_sequence(*g, [], [('evolve', 1, dead, False), ('evolve', 200, w.dt)], precision=E.FP64)
    assert rel_err(res.fid, ref) <= FP64_TOL
