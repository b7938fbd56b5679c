"""Launch shapes the engine picks for the benchmark systems, and parity across
the shapes a system can run with.

FP32 runs of 33-46 slices per CTA use the 768-thread 2-row kernel (one warp
per two slices plus two); 5-6 rows per lane use the 6-row kernel with the
low parts folded into the Kahan sums; cluster launches of real FP32 values
use the packed layout (value and column in 8 bytes), which puts c2's
dim-4096 systems on 4-CTA clusters.  Every shape of one system must give the
same FID within the FP32 bar, and FP64 must keep its 16-warp shapes.
"""
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


def test_c1_fp32_runs_twenty_warps_and_every_warp_count_agrees(engine_lib):
    from spinach_gb300 import engine as E, workloads as W
    w = W.c1()
    eng = _engine(w)
    g = W.zcwn_grid(w.n_orient)
    sel = slice(0, 152)
    grid = [a[sel] for a in g]
    r64 = eng.run(*grid, w.dt, w.nsteps, precision=E.FP64)
    assert r64.stats['threads'] == 512 and r64.stats['cluster'] == 1
    default = eng.run(*grid, w.dt, w.nsteps, precision=E.FP32, fp32_check=False)
    assert default.stats['threads'] == 640 and default.stats['cluster'] == 1      # 37 slices: 20 warps
    assert rel_err(default.fid, r64.fid) <= 1e-6
    for threads in (512, 576, 704, 768):
        r = eng.run(*grid, w.dt, w.nsteps, precision=E.FP32, fp32_check=False, threads=threads)
        assert r.stats['threads'] == threads
        assert rel_err(r.fid, r64.fid) <= 1e-6, threads
    eng.close()


def test_c4_fp32_one_cta_six_rows_matches_oracle(engine_lib):
    from spinach_gb300 import engine as E, workloads as W
    w = W.c4()
    gold = np.load(os.path.join(GOLD, 'c4_orient_krylov_fp64.npz'))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    s = gold['sel']
    eng = _engine(w)
    res = eng.run(al[s], be[s], ga[s], np.full(s.size, 1.0 / s.size), w.dt, w.nsteps, precision=E.FP32,
                  per_orientation=True, fp32_check=False)
    assert res.stats['cluster'] == 1 and res.stats['threads'] == 512          # 86 slices: 6 rows per lane
    for i in range(s.size):
        assert rel_err(res.fids[i], gold['fids'][i]) <= 1e-5, i
    eng.close()


def test_c2_dim4096_packed_clusters_of_four(engine_lib):
    from spinach_gb300 import engine as E, workloads as W
    gold = np.load(os.path.join(GOLD, 'c2_dim4096_orient_krylov_fp64.npz'))
    w = W.c2()[int(gold['system'])]
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    s = gold['sel']
    eng = _engine(w)
    wt = np.full(s.size, 1.0 / s.size)
    res = eng.run(al[s], be[s], ga[s], wt, w.dt, w.nsteps, precision=E.FP32, per_orientation=True,
                  fp32_check=False)
    assert res.stats['cluster'] == 4 and res.stats['threads'] > 512          # packed values, wide kernel
    for i in range(s.size):
        assert rel_err(res.fids[i], gold['fids'][i]) <= 1e-5, i
    # the 8-CTA clusters (plain layout) and 16-warp 4-CTA clusters agree
    for cluster, threads in ((8, 0), (4, 512)):
        r = eng.run(al[s], be[s], ga[s], wt, w.dt, w.nsteps, precision=E.FP32, fp32_check=False,
                    cluster=cluster, threads=threads)
        assert r.stats['cluster'] == cluster
        assert rel_err(r.fid, res.fid) <= 2e-6, (cluster, threads)
    eng.close()


def test_forced_shapes_of_the_six_row_and_wide_kernels(engine_lib):
    """Shapes the defaults do not reach on the benchmark systems: c1 on 7 and 9
    warps (6 rows per lane: low parts folded into the Kahan sums, t_{k-2} read
    back from shared memory) and a complex EPR system (18 slices) on 20 and 24
    warps (the wide kernel with one row per lane), each against FP64."""
    from spinach_gb300 import engine as E, workloads as W
    for w, shapes in ((W.c1(), (224, 288)), (W.c4_small(n_protons=2), (640, 768))):
        eng = _engine(w)
        g = [a[:64] for a in W.zcwn_grid(w.n_orient)]
        r64 = eng.run(*g, w.dt, w.nsteps, precision=E.FP64)
        for threads in shapes:
            r = eng.run(*g, w.dt, w.nsteps, precision=E.FP32, fp32_check=False, threads=threads)
            assert r.stats['threads'] == threads and r.stats['cluster'] == 1, (threads, r.stats['cluster'])
            assert rel_err(r.fid, r64.fid) <= 1e-5, threads
        eng.close()


@pytest.mark.parametrize('scale', [1e-4, 1e4])
def test_packed_cluster_values_at_any_magnitude(engine_lib, scale):
    """The packed cluster layout stores each value's low part as a half in
    units set by the system's bound on its entries: the c1 Liouvillian scaled
    by 1e4 (EPR-sized entries, ~1e9 rad/s) or 1e-4, with the time step scaled
    the other way, is the same dynamics and must give the same FIDs on 2- and
    4-CTA clusters as on one CTA."""
    from spinach_gb300 import engine as E, workloads as W
    w = W.c1()
    L = W.build(w)
    eng = E.Engine(0)
    eng.upload(L.I * scale, {k: q * scale for k, q in L.terms.items()}, L.R * scale, L.rho0, L.coil)
    g = [a[:48] for a in W.zcwn_grid(w.n_orient)]
    dt = w.dt / scale
    ref = eng.run(*g, dt, w.nsteps, precision=E.FP64)
    one = eng.run(*g, dt, w.nsteps, precision=E.FP32, fp32_check=False, cluster=1)
    assert rel_err(one.fid, ref.fid) <= 1e-6
    for cluster in (2, 4):
        r = eng.run(*g, dt, w.nsteps, precision=E.FP32, fp32_check=False, cluster=cluster)
        assert r.stats['cluster'] == cluster and r.stats['real_offdiag'] == 1
        assert rel_err(r.fid, ref.fid) <= 1e-6, cluster
    eng.close()
