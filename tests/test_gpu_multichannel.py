"""Several detection channels in one run (kernel/evolution.m 'multichannel':
one FID row per coil column)."""
import copy

import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_powder, rel_err

pytestmark = pytest.mark.gpu


def _system():
    from spinach_gb300 import spin_system as S
    w = W.c1()
    ss = W.spin_system_of(w)
    basis = S.build_basis(ss, w.approximation, w.level)
    fac = S.factory_for(ss, basis)
    L = W.build(w)
    # two 13C observables (proton coherence stays exactly zero here: the
    # heteronuclear couplings are secular under 'nmr')
    coils = [fac.state('L+', '13C'), fac.state('Lx', '13C')]
    return w, L, coils


def test_two_channels_match_single_channel_runs_and_oracle(gpu_engine):
    w, L, coils = _system()
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([4, 250, 611])
    g = (al[sel], be[sel], ga[sel], np.array([0.2, 0.5, 0.3]))
    nsteps = 200
    single = []
    for c in coils:
        gpu_engine.upload(L.I, L.terms, L.R, L.rho0, c)
        single.append({p: gpu_engine.run(*g, w.dt, nsteps, precision=p, per_orientation=True) for p in (E.FP64, E.FP32)})
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, coils[0])
    gpu_engine.upload_coils(coils)
    for p, tol in ((E.FP64, 1e-13), (E.FP32, 1e-6)):
        res = gpu_engine.run(*g, w.dt, nsteps, precision=p, per_orientation=True)
        assert res.fid.shape == (2, nsteps + 1) and res.fids.shape == (3, 2, nsteps + 1)
        assert res.stats['channels'] == 2
        for c in range(2):
            assert rel_err(res.fid[c], single[c][p].fid) <= tol, (p, c)
            for i in range(3):
                assert rel_err(res.fids[i, c], single[c][p].fids[i]) <= tol, (p, c, i)
    # the second channel against the oracle (exact step.m branch)
    w1 = copy.deepcopy(w)
    w1.coil = ('Lx', '13C')
    ref = oracle_powder(w1, g, nsteps=nsteps, krylov=True)
    res = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP64)
    assert rel_err(res.fid[1], ref) <= 1e-10


def test_channels_on_a_cluster(gpu_engine):
    w, L, coils = _system()
    g = W.zcwn_grid(12)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, coils[0])
    gpu_engine.upload_coils(coils)
    a = gpu_engine.run(*g, w.dt, 300, precision=E.FP64, cluster=1)
    b = gpu_engine.run(*g, w.dt, 300, precision=E.FP64, cluster=2)
    assert b.stats['cluster'] == 2
    for c in range(2):
        assert rel_err(b.fid[c], a.fid[c]) <= 1e-12


def test_channel_limits(gpu_engine):
    w, L, coils = _system()
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, coils[0])
    dense = np.random.default_rng(0).normal(size=L.dim) + 0j
    with pytest.raises(E.SpxError):
        gpu_engine.upload_coils([coils[0], dense])        # more than 32 non-zeros over two channels
    with pytest.raises(E.SpxError):
        gpu_engine.upload_coils([coils[0]] * 9)           # at most 8 channels
