"""Three-pulse DEER with hard pulses (experiments/esr_dipolar/deer_3p_hard_deer.m)
in the powder context: an adjoint run and pulse give each orientation's
detection side, whose adjoint trajectory, read backwards, meets the forward
trajectory through the pump pulse in one bilinear form per orientation and
pump position."""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_system, rel_err
from oracle import spinach_ref as R

pytestmark = pytest.mark.gpu


def _case(w, probe, pump, krylov):
    from spinach_gb300 import spin_system as S
    L = W.build(w)
    ss_b = W.spin_system_of(w)
    fac = S.factory_for(ss_b, S.build_basis(ss_b, w.approximation, w.level))
    ss, I, Q = oracle_system(w, krylov=krylov)

    def ly(iso):
        return sum(fac.operator([('Ly', s)]) for s, i in enumerate(w.isotopes) if i == iso)
    assert abs(ly(probe) - R.operator(ss, 'Ly', probe)).max() < 1e-14
    return L, ss, I, Q, ly(probe), ly(pump), fac.state('Lz', probe), fac.state('L+', probe)


@pytest.mark.parametrize('wname,probe,pump,stepsize,nsteps', [('c0', '13C', '1H', 10e-6, 40),
                                                              ('c4_small', 'E', '1H', 10e-9, 24)])
def test_deer_matches_oracle(gpu_engine, wname, probe, pump, stepsize, nsteps):
    w = getattr(W, wname)()
    L, ss, I, Q, Xprob, Xpump, rho0, coil = _case(w, probe, pump, krylov=(wname != 'c0'))
    g = W.zcwn_grid(5)
    g = (g[0], g[1], g[2], np.array([0.1, 0.3, 0.2, 0.25, 0.15]))
    par = dict(rho0=R.state(ss, 'Lz', probe), coil_prob=R.state(ss, 'L+', probe),
               ex_prob=R.operator(ss, 'Ly', probe), ex_pump=R.operator(ss, 'Ly', pump), stepsize=stepsize,
               nsteps=nsteps)
    ref = sum(g[3][i] * R.powder_orientation_deer(ss, I, Q, par, (g[0][i], g[1][i], g[2][i])) for i in range(5))
    assert np.abs(ref).max() > 0.05
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run_deer(*g, stepsize, nsteps, Xprob, Xpump, precision=prec, per_orientation=True)
        assert res.fid.shape == (nsteps + 1,) and res.fids.shape == (5, nsteps + 1)
        assert rel_err(res.fid, ref) <= tol, prec
        assert np.abs((g[3][:, None] * res.fids).sum(axis=0) - res.fid).max() <= 1e-12 * np.abs(res.fid).max()


def test_deer_identities_and_checks(gpu_engine):
    """A zero pump leaves every point the same echo (the pump position no
    longer matters), and the argument checks of deer_3p_hard_deer.m."""
    w = W.c0()
    L, ss, I, Q, Xprob, Xpump, rho0, coil = _case(w, '13C', '1H', krylov=False)
    g = W.zcwn_grid(7)
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    res = gpu_engine.run_deer(*g, 10e-6, 16, Xprob, 0 * Xpump, precision=E.FP64)
    assert np.abs(res.fid[0]) > 0.01
    assert np.abs(res.fid - res.fid[0]).max() <= 1e-11 * np.abs(res.fid[0])
    with pytest.raises(E.SpxError):                      # nsteps a positive integer
        gpu_engine.run_deer(*g, 10e-6, 0, Xprob, Xpump)
    with pytest.raises(E.SpxError):                      # stepsize positive
        gpu_engine.run_deer(*g, 0.0, 8, Xprob, Xpump)
    gpu_engine.upload_coils([L.coil, L.coil])
    with pytest.raises(E.SpxError):                      # one detection channel
        gpu_engine.run_deer(*g, 10e-6, 8, Xprob, Xpump)


def test_deer_echo_program_matches_oracle(gpu_engine):
    """experiments/esr_dipolar/deer_3p_hard_echo.m as a pulse program on the
    c4 radical (probe E, pump 1H): three hard pulses, three silent delays and
    the echo over tc."""
    w = W.c4_small()
    L, ss, I, Q, Xprob, Xpump, rho0, coil = _case(w, 'E', '1H', krylov=True)
    ta, tb, tc, n = 200e-9, 60e-9, 120e-9, 24
    g = W.zcwn_grid(4)
    g = (g[0], g[1], g[2], np.array([0.3, 0.2, 0.4, 0.1]))
    par = dict(rho0=R.state(ss, 'Lz', 'E'), coil=R.state(ss, 'L+', 'E'), ex_prob=R.operator(ss, 'Ly', 'E'),
               ex_pump=R.operator(ss, 'Ly', '1H'), ta=ta, tb=tb, tc=tc, nsteps=n)
    ref = sum(g[3][i] * R.powder_orientation_sequence(ss, I, Q, par, (g[0][i], g[1][i], g[2][i]),
                                                      R.deer_3p_hard_echo) for i in range(4))
    assert np.abs(ref).max() > 0.02
    gpu_engine.upload(L.I, L.terms, L.R, rho0, coil)
    prog = [('pulse', 0, np.pi / 2), ('evolve', 1, tb, False), ('pulse', 1, np.pi), ('evolve', 1, ta - tb, False),
            ('pulse', 0, np.pi), ('evolve', 1, ta - 0.5 * tc, False), ('evolve', n, tc / n)]
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run_sequence(*g, [Xprob, Xpump], prog, precision=prec)
        assert res.fid.shape == (n + 1,)
        assert rel_err(res.fid, ref) <= tol, prec
