"""Parity of the thread-block-cluster kernels (one orientation shared by 2-8
CTAs that exchange state rows through distributed shared memory) against the
FP64 oracle fixtures, and of clustered runs against single-CTA runs."""
import os

import numpy as np
import pytest

from oracle_cases import rel_err

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')


def _engine(w):
    from spinach_gb300 import engine as E, workloads as W
    L = W.build(w)
    eng = E.Engine(0)
    eng.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    return eng


@pytest.mark.parametrize('cluster', [2, 4, 8])
def test_c1_forced_clusters_match_oracle(engine_lib, cluster):
    from spinach_gb300 import engine as E, workloads as W
    w = W.c1()
    gold = np.load(os.path.join(GOLD, 'c1_orient_krylov_fp64.npz'))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = gold['sel']
    wt = np.full(sel.size, 1.0 / sel.size)
    eng = _engine(w)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = eng.run(al[sel], be[sel], ga[sel], wt, w.dt, w.nsteps, precision=prec, per_orientation=True,
                      cluster=cluster)
        assert res.stats['cluster'] == cluster
        for i in range(sel.size):
            assert rel_err(res.fids[i], gold['fids'][i]) <= tol, (prec, cluster, i)


def test_cluster_matches_single_cta(engine_lib):
    """Same orientations with 1 and 2 CTAs each: the row split must not change
    the arithmetic beyond reduction order."""
    from spinach_gb300 import engine as E, workloads as W
    w = W.c1()
    al, be, ga, wt = W.zcwn_grid(40)
    eng = _engine(w)
    for prec, tol in ((E.FP64, 1e-12), (E.FP32, 1e-6)):
        a = eng.run(al, be, ga, wt, w.dt, 512, precision=prec, cluster=1)
        b = eng.run(al, be, ga, wt, w.dt, 512, precision=prec, cluster=2)
        assert a.stats['cluster'] == 1 and b.stats['cluster'] == 2
        assert rel_err(b.fid, a.fid) <= tol, prec


def test_c4_full_basis_dim2736(engine_lib):
    """EPR radical (e + 14N + 10 1H, IK-1(3), dim 2736, complex off-diagonal
    values): FP32 fits one SM, FP64 needs a cluster; both shapes checked."""
    from spinach_gb300 import engine as E, workloads as W
    w = W.c4()
    gold = np.load(os.path.join(GOLD, 'c4_orient_krylov_fp64.npz'))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = gold['sel']
    wt = np.full(sel.size, 1.0 / sel.size)
    eng = _engine(w)
    for prec, tol, cluster in ((E.FP64, 1e-10, 0), (E.FP32, 1e-5, 0), (E.FP32, 1e-5, 2)):
        res = eng.run(al[sel], be[sel], ga[sel], wt, w.dt, w.nsteps, precision=prec, per_orientation=True,
                      cluster=cluster)
        assert res.stats['real_offdiag'] == 0
        if cluster:
            assert res.stats['cluster'] == cluster
        for i in range(sel.size):
            assert rel_err(res.fids[i], gold['fids'][i]) <= tol, (prec, cluster, i)
        assert rel_err(res.fid, gold['fids'].mean(axis=0)) <= tol


def test_c2_dim4096_system(engine_lib):
    """A 6-spin full-basis system of the batched workload (dim 4096)."""
    from spinach_gb300 import engine as E, workloads as W
    gold = np.load(os.path.join(GOLD, 'c2_dim4096_orient_krylov_fp64.npz'))
    w = W.c2()[int(gold['system'])]
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = gold['sel']
    wt = np.full(sel.size, 1.0 / sel.size)
    eng = _engine(w)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = eng.run(al[sel], be[sel], ga[sel], wt, w.dt, w.nsteps, precision=prec, per_orientation=True)
        assert res.stats['cluster'] > 1 and res.stats['dim'] == 4096
        for i in range(sel.size):
            assert rel_err(res.fids[i], gold['fids'][i]) <= tol, (prec, i)
