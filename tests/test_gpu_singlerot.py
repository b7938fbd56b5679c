"""Magic-angle spinning (kernel/contexts/singlerot.m, Fokker-Planck, and
kernel/contexts/floquet.m) through the engine: the rotor-space and Floquet
Liouvillians in upload form run on the same kernels, with acquire and with
the hard-pulse sequences."""
import math

import numpy as np
import pytest

from spinach_gb300 import engine as E, singlerot as SR, workloads as W
from oracle_cases import oracle_system, rel_err
from oracle import spinach_ref as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('max_rank,rate', [(3, 12.5e3), (5, 5e3)])
def test_mas_powder_matches_oracle(gpu_engine, max_rank, rate):
    w = W.c0()
    L = W.build(w)
    axis = (1.0, 1.0, 1.0)
    I_fp, terms, R_fp, rho0, coil = SR.fokker_planck(L.I, L.terms, L.R, L.rho0, L.coil, max_rank, rate, axis)
    ss, I, Q = oracle_system(w, krylov=True)
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([7, 66, 131])
    g = (al[sel], be[sel], ga[sel], np.array([0.25, 0.35, 0.4]))
    nsteps = 160
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=nsteps + 1,
               rate=rate, axis=axis, max_rank=max_rank)
    ref = sum(g[3][i] * R.singlerot_orientation_fid(ss, I, Q, par, (g[0][i], g[1][i], g[2][i]))
              for i in range(sel.size))
    gpu_engine.upload(I_fp, terms, R_fp, rho0, coil)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run(*g, w.dt, nsteps, precision=prec)
        assert res.stats['dim'] == (2 * max_rank + 1) * L.dim
        assert rel_err(res.fid, ref) <= tol, prec


def test_reference_single_crystal_case(gpu_engine):
    """tests/kernel/test_ctx_singlerot_acquire.m through the engine."""
    from spinach_gb300 import spin_system as S
    ss = S.make_spin_system(['1H'], 14.1, zeeman_eigs=[[-2.0, -2.0, 4.0]], zeeman_euler=[[0.0, 0.0, 0.0]])
    basis = S.build_basis(ss, 'none', 0, projections=[1])
    fac = S.factory_for(ss, basis)
    H = S.rotational_hamiltonian(ss, basis, 'nmr', fac)
    rho0 = fac.state('L+', '1H')
    I_fp, terms, _, r0, cl = SR.fokker_planck(H.iso, H.aniso, None, rho0, rho0, 1, 1000.0, (1, 1, 1),
                                             single_crystal=True)
    gpu_engine.upload(I_fp, terms, None, r0, cl)
    fid = gpu_engine.run(np.zeros(1), np.zeros(1), np.zeros(1), np.ones(1), 1 / 2000.0, 2, precision=E.FP64).fid
    assert fid.shape == (3,)
    assert abs(fid[0] - np.vdot(rho0, rho0)) <= 1e-12
    assert np.all(np.isfinite(fid))


def _rotor_frame_angles(angles, axis):
    """Euler angles of the rotation whose Wigner matrix is
    D(angles) * D_rot2lab: floquet.m moves the crystallite into the rotor
    frame with a trailing D_rot2lab that singlerot.m does not apply, so the
    same crystallite carries these angles in singlerot.m."""
    phi, theta = SR.rotor_axis_angles(axis)
    D = SR.wigner_d(1, *angles) @ SR.wigner_d(1, phi, theta, 0.0).conj().T
    b = math.acos(max(-1.0, min(1.0, D[1, 1].real)))
    d = SR.wigner_d(1, 0.0, b, 0.0)
    return -np.angle(D[0, 1] / d[0, 1]), b, -np.angle(D[1, 0] / d[1, 0])


def test_floquet_mas_matches_oracle_and_fokker_planck(gpu_engine):
    """floquet.m (Fourier components) on the engine against the oracle's
    restatement, and against the Fokker-Planck rotor grid of singlerot.m for
    the same crystallites, which describes the same spinning sample."""
    w = W.c0()
    L = W.build(w)
    axis, rate = (1.0, 1.0, 1.0), 12.5e3
    ss, I, Q = oracle_system(w, krylov=True)
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([7, 66, 131])
    g = (al[sel], be[sel], ga[sel], np.array([0.25, 0.35, 0.4]))
    nsteps = 160
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=nsteps + 1,
               rate=rate, axis=axis, max_rank=4)
    ref = sum(g[3][i] * R.floquet_orientation_fid(ss, I, Q, par, (g[0][i], g[1][i], g[2][i])) for i in range(3))
    gpu_engine.upload(*SR.floquet_system(L.I, L.terms, L.R, L.rho0, L.coil, 4, rate, axis))
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        assert rel_err(gpu_engine.run(*g, w.dt, nsteps, precision=prec).fid, ref) <= tol, prec
    # both MAS treatments, converged in the rotor rank, give the same signal
    gpu_engine.upload(*SR.floquet_system(L.I, L.terms, L.R, L.rho0, L.coil, 12, rate, axis))
    f_fl = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP64).fid
    mapped = np.array([_rotor_frame_angles((g[0][i], g[1][i], g[2][i]), axis) for i in range(3)])
    gpu_engine.upload(*SR.fokker_planck(L.I, L.terms, L.R, L.rho0, L.coil, 12, rate, axis))
    f_fp = gpu_engine.run(mapped[:, 0], mapped[:, 1], mapped[:, 2], g[3], w.dt, nsteps, precision=E.FP64).fid
    assert rel_err(f_fl, f_fp) <= 1e-5


@pytest.mark.parametrize('context,sequence', [('singlerot', 'hp_acquire'), ('floquet', 'cpmg'),
                                              ('singlerot', 'cpmg'), ('floquet', 'hp_acquire')])
def test_mas_contexts_with_pulse_sequences(gpu_engine, context, sequence):
    """singlerot.m / floquet.m with @hp_acquire (echo) and @cpmg: pulses
    projected into the rotor or Fourier space, kron(speye(spc_dim), op)
    (hp_acquire.m:57,69, cpmg.m:33), on the engine against the oracle."""
    from spinach_gb300 import contexts as X
    sys_ = dict(isotopes=['13C', '1H'], magnet=14.1)
    inter = dict(zeeman=dict(eigs=[[10.0, 70.0, 180.0], [1.0, 3.0, 8.0]], euler=[[0.1, 0.7, 1.9], [0, 0, 0]]),
                 coupling=dict(scalar={(0, 1): 140.0}))
    spin_system = X.basis(X.create(sys_, inter), dict(approximation='none'))
    al, be, ga = np.zeros(3), np.array([0.4, 1.3, 2.5]), np.array([0.3, 2.0, 4.1])
    w = np.array([0.2, 0.5, 0.3])
    base = dict(rate=8e3, axis=(1, 1, 1), max_rank=3, grid=(al, be, ga, w))
    if sequence == 'hp_acquire':
        seq = dict(pulse_op=('Ly', '13C'), pulse_angle=np.pi / 2, echo_time=3e-5, echo_oper=('Lx', '13C'),
                   echo_angle=np.pi, sweep=2e4, npoints=40)
    else:
        seq = dict(pulse_op=('Ly', '13C'), timestep=5e-5, npoints=16, nloops=2)
    parameters = dict(base, rho0=('Lz', '13C'), coil=('L+', '13C'), **seq)
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(approximation='none', level=0, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(base, rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, 'L+', '13C'))
    for k in ('pulse_op', 'echo_oper'):
        if k in seq:
            par[k] = R.operator(ss, seq[k][0], seq[k][1])
    par.update({k: v for k, v in seq.items() if k not in ('pulse_op', 'echo_oper')})
    one = R.singlerot_orientation_fid if context == 'singlerot' else R.floquet_orientation_fid
    ref = sum(w[i] * one(ss, I, Q, par, (al[i], be[i], ga[i]), sequence=sequence) for i in range(3))
    assert np.abs(ref).max() > 0.05
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        fid, _ = getattr(X, context)(spin_system, sequence, parameters, 'nmr', engine=gpu_engine, precision=prec)
        assert rel_err(fid, ref) <= tol, prec
