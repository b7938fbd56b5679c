"""Per-orientation initial states (kernel/contexts/powder.m:244-254: 'aniso_eq'
or a function-handle rho0 evaluated at every grid point)."""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_system, rel_err
from oracle import spinach_ref as R

pytestmark = pytest.mark.gpu


def test_per_orientation_initial_states_match_oracle(gpu_engine):
    from spinach_gb300 import spin_system as S
    w = W.c0()
    L = W.build(w)
    ss_b = W.spin_system_of(w)
    fac = S.factory_for(ss_b, S.build_basis(ss_b, w.approximation, w.level))
    ss, I, Q = oracle_system(w)
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([3, 40, 99, 150, 180])
    g = (al[sel], be[sel], ga[sel], np.full(sel.size, 0.2))
    nsteps = 300
    # rho0(Omega) = cos(beta) Lx(13C) + sin(gamma) Lz(1H): a stand-in for a
    # function-handle initial condition
    bx, bz = fac.state('Lx', '13C'), fac.state('Lz', '1H')
    ox, oz = R.state(ss, 'Lx', '13C'), R.state(ss, 'Lz', '1H')
    assert np.allclose(bx, ox, atol=1e-14) and np.allclose(bz, oz, atol=1e-14)
    coef = np.stack([np.cos(g[1]), np.sin(g[2])], 1)
    states = coef[:, :1] * bx + coef[:, 1:] * bz
    ref = []
    for i in range(sel.size):
        par = dict(rho0=coef[i, 0] * ox + coef[i, 1] * oz, coil=R.state(ss, *w.coil), sweep=1 / w.dt,
                   npoints=nsteps + 1)
        ref.append(R.powder_orientation_fid(ss, I, Q, par, (g[0][i], g[1][i], g[2][i])))
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    gpu_engine.set_initial_states(states)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run(*g, w.dt, nsteps, precision=prec, per_orientation=True)
        for i in range(sel.size):
            assert rel_err(res.fids[i], ref[i]) <= tol, (prec, i)
        assert rel_err(res.fid, 0.2 * sum(ref)) <= tol
    with pytest.raises(E.SpxError):                 # the grid must match the states
        gpu_engine.run(*[a[:3] for a in g], w.dt, nsteps)
    gpu_engine.set_initial_states(None)             # back to the single rho0
    res = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP64, per_orientation=True)
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=nsteps + 1)
    assert rel_err(res.fids[0], R.powder_orientation_fid(ss, I, Q, par, (g[0][0], g[1][0], g[2][0]))) <= 1e-10
