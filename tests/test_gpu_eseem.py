"""Two-pulse echo (experiments/esr_dipolar/eseem.m) in the powder context:
forward and adjoint trajectories of the evolution core, joined by the
180-degree pulse in one bilinear form per orientation and step."""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_system, rel_err
from oracle import spinach_ref as R

pytestmark = pytest.mark.gpu


def _case(w, spin, krylov):
    from spinach_gb300 import spin_system as S
    L = W.build(w)
    ss_b = W.spin_system_of(w)
    fac = S.factory_for(ss_b, S.build_basis(ss_b, w.approximation, w.level))
    ss, I, Q = oracle_system(w, krylov=krylov)
    spins = [i for i, iso in enumerate(w.isotopes) if iso == spin]
    pulse = sum(fac.operator([('Ly', s)]) for s in spins)
    assert abs(pulse - R.operator(ss, 'Ly', spin)).max() < 1e-14
    return L, ss, I, Q, pulse, fac.state('Lz', spin), fac.state('L+', spin)


@pytest.mark.parametrize('wname,spin,timestep,npoints', [('c0', '13C', 20e-6, 64),
                                                         ('c4_small', 'E', 10e-9, 48)])
def test_eseem_matches_oracle(gpu_engine, wname, spin, timestep, npoints):
    w = getattr(W, wname)()
    L, ss, I, Q, pulse, rho0, coil = _case(w, spin, krylov=(wname != 'c0'))
    g = W.zcwn_grid(5)
    g = (g[0], g[1], g[2], np.array([0.1, 0.3, 0.2, 0.25, 0.15]))
    par = dict(rho0=R.state(ss, 'Lz', spin), coil=R.state(ss, 'L+', spin), pulse_op=R.operator(ss, 'Ly', spin),
               timestep=timestep, npoints=npoints)
    ref = sum(g[3][i] * R.powder_orientation_eseem(ss, I, Q, par, (g[0][i], g[1][i], g[2][i])) for i in range(5))
    assert np.abs(ref).max() > 0.05
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run_eseem(*g, timestep, npoints, pulse, precision=prec)
        assert res.fid.shape == (npoints,)
        assert rel_err(res.fid, ref) <= tol, prec
    # the plain acquisition afterwards is untouched by the echo buffers
    plain = gpu_engine.run(*g, w.dt, 32, precision=E.FP64)
    assert np.all(np.isfinite(plain.fid))


def test_eseem_on_clusters_of_two_and_four(gpu_engine):
    w = W.c4()
    L, ss, I, Q, pulse, rho0, coil = _case(w, 'E', krylov=True)
    g = W.zcwn_grid(6)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    a = gpu_engine.run_eseem(*g, 16e-9, 24, pulse, precision=E.FP64, cluster=2)
    b = gpu_engine.run_eseem(*g, 16e-9, 24, pulse, precision=E.FP64, cluster=4)
    assert a.stats['cluster'] == 2 and b.stats['cluster'] == 4
    assert rel_err(b.fid, a.fid) <= 1e-12
    assert np.abs(a.fid).max() > 0.01


def test_eseem_argument_checks(gpu_engine):
    w = W.c0()
    L, ss, I, Q, pulse, rho0, coil = _case(w, '13C', krylov=False)
    g = W.zcwn_grid(4)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    with pytest.raises(E.SpxError):
        gpu_engine.run_eseem(*g, 1e-5, 0, pulse)
    with pytest.raises(E.SpxError):
        gpu_engine.run_eseem(*g, -1e-5, 8, pulse)
    gpu_engine.upload_coils([coil, coil])
    with pytest.raises(E.SpxError):
        gpu_engine.run_eseem(*g, 1e-5, 8, pulse)


def test_eseem_per_orientation_echoes(gpu_engine):
    w = W.c0()
    L, ss, I, Q, pulse, rho0, coil = _case(w, '13C', krylov=False)
    g = W.zcwn_grid(9)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    res = gpu_engine.run_eseem(*g, 20e-6, 40, pulse, precision=E.FP64, per_orientation=True)
    assert res.fids.shape == (9, 40)
    assert np.abs((g[3][:, None] * res.fids).sum(axis=0) - res.fid).max() <= 1e-12 * np.abs(res.fid).max()


@pytest.mark.parametrize('wname,spin,timestep,npoints', [('c0', '13C', 20e-6, 48),
                                                         ('c4_small', 'E', 10e-9, 32)])
def test_oopeseem_matches_oracle(gpu_engine, wname, spin, timestep, npoints):
    """experiments/esr_dipolar/oopeseem.m: the echo core with a 45-degree
    first pulse (spx_run_oopeseem)."""
    w = getattr(W, wname)()
    L, ss, I, Q, pulse, rho0, coil = _case(w, spin, krylov=(wname != 'c0'))
    g = W.zcwn_grid(4)
    g = (g[0], g[1], g[2], np.array([0.1, 0.4, 0.3, 0.2]))
    par = dict(rho0=R.state(ss, 'Lz', spin), coil=R.state(ss, 'L+', spin), pulse_op=R.operator(ss, 'Ly', spin),
               timestep=timestep, npoints=npoints)
    ref = sum(g[3][i] * R.powder_orientation_sequence(ss, I, Q, par, (g[0][i], g[1][i], g[2][i]), R.oopeseem)
              for i in range(4))
    assert np.abs(ref).max() > 0.05
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run_eseem(*g, timestep, npoints, pulse, precision=prec, out_of_phase=True)
        assert rel_err(res.fid, ref) <= tol, prec
