"""CPMG echo trains on the evolution core (experiments/cpmg.m in the powder
context): hard pulses between propagation segments that continue from each
orientation's final state."""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_system, rel_err
from oracle import spinach_ref as R

pytestmark = pytest.mark.gpu


def _case(w, krylov):
    from spinach_gb300 import spin_system as S
    L = W.build(w)
    ss_b = W.spin_system_of(w)
    fac = S.factory_for(ss_b, S.build_basis(ss_b, w.approximation, w.level))
    ss, I, Q = oracle_system(w, krylov=krylov)
    carbons = [i for i, iso in enumerate(w.isotopes) if iso == '13C']
    pulse = sum(fac.operator([('Ly', s)]) for s in carbons)
    pulse_o = R.operator(ss, 'Ly', '13C')
    assert abs(pulse - pulse_o).max() < 1e-14
    rho0 = fac.state('Lz', '13C')
    assert np.allclose(rho0, R.state(ss, 'Lz', '13C'), atol=1e-14)
    return L, ss, I, Q, pulse, pulse_o, rho0


def _oracle(w, ss, I, Q, pulse_o, g, npoints, nloops):
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, *w.coil), pulse_op=pulse_o, timestep=w.dt,
               npoints=npoints, nloops=nloops)
    return sum(g[3][i] * R.powder_orientation_cpmg(ss, I, Q, par, (g[0][i], g[1][i], g[2][i]))
               for i in range(g[0].size))


@pytest.mark.parametrize('wname,sel,npoints,nloops', [('c0', [3, 40, 99, 150, 180], 48, 2),
                                                       ('c1', [4, 611], 24, 2)])
def test_cpmg_matches_oracle(gpu_engine, wname, sel, npoints, nloops):
    w = getattr(W, wname)()
    L, ss, I, Q, pulse, pulse_o, rho0 = _case(w, krylov=(wname != 'c0'))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array(sel)
    g = (al[sel], be[sel], ga[sel], np.linspace(0.1, 0.4, sel.size))
    ref = _oracle(w, ss, I, Q, pulse_o, g, npoints, nloops)
    assert np.abs(ref).max() > 0.05
    gpu_engine.upload(L.I, L.terms, L.R, rho0, L.coil)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run_cpmg(*g, w.dt, npoints, nloops, pulse, precision=prec)
        assert res.fid.shape == (npoints * (1 + 2 * nloops),)
        assert rel_err(res.fid, ref) <= tol, prec
        # the half-echo alone is the pulsed acquisition
        assert rel_err(res.fid[:npoints], ref[:npoints]) <= tol


def test_cpmg_on_a_cluster_matches_one_cta(gpu_engine):
    w = W.c1()
    L, ss, I, Q, pulse, pulse_o, rho0 = _case(w, krylov=True)
    g = W.zcwn_grid(16)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, L.coil)
    a = gpu_engine.run_cpmg(*g, w.dt, 100, 3, pulse, precision=E.FP64, cluster=1)
    b = gpu_engine.run_cpmg(*g, w.dt, 100, 3, pulse, precision=E.FP64, cluster=2)
    assert b.stats['cluster'] == 2
    assert rel_err(b.fid, a.fid) <= 1e-12


def test_cpmg_argument_checks(gpu_engine):
    w = W.c0()
    L, ss, I, Q, pulse, pulse_o, rho0 = _case(w, krylov=False)
    g = W.zcwn_grid(8)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, L.coil)
    with pytest.raises(E.SpxError):                      # cpmg.m: nloops a positive integer
        gpu_engine.run_cpmg(*g, w.dt, 16, 0, pulse)
    with pytest.raises(E.SpxError):
        gpu_engine.run_cpmg(*g, w.dt, 0, 1, pulse)
    gpu_engine.upload_coils([L.coil, L.coil])
    with pytest.raises(E.SpxError):                      # one detection channel
        gpu_engine.run_cpmg(*g, w.dt, 16, 1, pulse)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, L.coil)
    res = gpu_engine.run_cpmg(*g, w.dt, 16, 1, pulse, precision=E.FP64)
    assert np.all(np.isfinite(res.fid))
    # with a zero pulse the half-echo is the plain acquisition, and a plain
    # run afterwards is unaffected by the pulse-sequence buffers
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    pre = gpu_engine.run_cpmg(*g, w.dt, 16, 1, 0 * pulse, precision=E.FP64)
    plain = gpu_engine.run(*g, w.dt, 46, precision=E.FP64)
    assert np.abs(plain.fid).max() > 0.05
    assert rel_err(pre.fid, plain.fid[list(range(16)) + list(range(15, 47))]) <= 1e-13


@pytest.mark.parametrize('wname,spin', [('c0', '13C'), ('c4_small', 'E')])
def test_hp_acquire_echo_program_matches_oracle(gpu_engine, wname, spin):
    """experiments/hp_acquire.m with an echo (pulse, echo_time, echo pulse,
    echo_time, acquisition) as a pulse program."""
    from spinach_gb300 import spin_system as S
    w = getattr(W, wname)()
    L = W.build(w)
    ss_b = W.spin_system_of(w)
    fac = S.factory_for(ss_b, S.build_basis(ss_b, w.approximation, w.level))
    ss, I, Q = oracle_system(w, krylov=(wname != 'c0'))
    spins = [i for i, iso in enumerate(w.isotopes) if iso == spin]
    Py = sum(fac.operator([('Ly', s)]) for s in spins)
    Px = sum(fac.operator([('Lx', s)]) for s in spins)
    echo = 37 * w.dt
    npoints = 64
    par = dict(rho0=R.state(ss, 'Lz', spin), coil=R.state(ss, 'L+', spin), pulse_op=R.operator(ss, 'Ly', spin),
               pulse_angle=np.pi / 2, echo_time=echo, echo_oper=R.operator(ss, 'Lx', spin), echo_angle=np.pi,
               sweep=1 / w.dt, npoints=npoints)
    g = W.zcwn_grid(6)
    g = (g[0], g[1], g[2], np.linspace(0.1, 0.3, 6))
    ref = sum(g[3][i] * R.powder_orientation_hp_acquire(ss, I, Q, par, (g[0][i], g[1][i], g[2][i]))
              for i in range(6))
    assert np.abs(ref).max() > 0.05
    gpu_engine.upload(L.I, L.terms, L.R, fac.state('Lz', spin), fac.state('L+', spin))
    prog = [('pulse', 0, np.pi / 2), ('evolve', 1, echo, False), ('pulse', 1, np.pi), ('evolve', 1, echo, False),
            ('evolve', npoints - 1, w.dt)]
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run_sequence(*g, [Py, Px], prog, precision=prec)
        assert res.fid.shape == (npoints,)
        assert rel_err(res.fid, ref) <= tol, prec
    with pytest.raises(E.SpxError):                          # pulse index out of range
        gpu_engine.run_sequence(*g, [Py], prog)


def test_program_identities(gpu_engine):
    """A zero-step segment and a zero-angle pulse leave the state alone: the
    program's recorded segments tile the plain acquisition."""
    w = W.c0()
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    g = W.zcwn_grid(10)
    plain = gpu_engine.run(*g, w.dt, 40, precision=E.FP64).fid
    P = L.I * 0 + L.terms[sorted(L.terms)[0]]              # any operator: used with angle 0
    prog = [('evolve', 0, w.dt), ('pulse', 0, 0.0), ('evolve', 15, w.dt), ('evolve', 25, w.dt)]
    res = gpu_engine.run_sequence(*g, [P], prog, precision=E.FP64)
    assert res.fid.shape == (1 + 16 + 26,)
    want = np.concatenate([plain[:1], plain[:16], plain[15:41]])
    assert rel_err(res.fid, want) <= 1e-13


def test_cpmg_per_orientation_fids(gpu_engine):
    w = W.c0()
    L, ss, I, Q, pulse, pulse_o, rho0 = _case(w, krylov=False)
    g = W.zcwn_grid(7)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, L.coil)
    res = gpu_engine.run_cpmg(*g, w.dt, 16, 2, pulse, precision=E.FP64, per_orientation=True)
    assert res.fids.shape == (7, 80)
    assert np.abs((g[3][:, None] * res.fids).sum(axis=0) - res.fid).max() <= 1e-12 * np.abs(res.fid).max()
