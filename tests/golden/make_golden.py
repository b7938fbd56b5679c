"""Generate the FP64 oracle fixtures used by the GPU parity tests.

Run from the repository root:  python tests/golden/make_golden.py
(``python tests/golden/make_golden.py large`` for the cluster-sized
systems, ``... deuterium`` for the quadratic-coupling workload, ``... grids``
to copy the reference's 14-point Lebedev grid out of its grid file, which
needs the reference source tree).  Writes tests/golden/*.npz.  Inputs are the seeded workloads of
spinach_gb300.workloads; FIDs come from the oracle (oracle/spinach_ref.py).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from spinach_gb300 import workloads as W  # noqa: E402
from oracle_cases import oracle_powder  # noqa: E402


def save(name, **kw):
    np.savez_compressed(os.path.join(HERE, name), **kw)
    print('wrote', name, {k: getattr(v, 'shape', v) for k, v in kw.items()})


def large_systems():
    """Systems whose share of L needs a cluster of CTAs on the GPU."""
    # c4 EPR radical, IK-1(3) basis dim 2736, Krylov branch, 3 orientations x 4096 steps
    w = W.c4()
    al, be, ga, wt = W.zcwn_grid(w.n_orient)
    sel = np.array([0, 1234, 3210])
    sub = (al[sel], be[sel], ga[sel], np.full(sel.size, 1.0 / sel.size))
    fk = oracle_powder(w, sub, krylov=True, sum_up=False)
    save('c4_orient_krylov_fp64.npz', sel=sel, fids=np.array(fk), seed=w.seed, nsteps=w.nsteps)
    # the first dim-4096 system of the batched workload (6 spins, full basis), 2 orientations x 1024 steps
    ws = W.c2()
    idx = next(i for i, x in enumerate(ws) if len(x.isotopes) == 6)
    w = ws[idx]
    al, be, ga, wt = W.zcwn_grid(w.n_orient)
    sel = np.array([7, 211])
    sub = (al[sel], be[sel], ga[sel], np.full(sel.size, 1.0 / sel.size))
    fk = oracle_powder(w, sub, krylov=True, sum_up=False)
    save('c2_dim4096_orient_krylov_fp64.npz', system=idx, sel=sel, fids=np.array(fk), seed=w.seed,
         nsteps=w.nsteps)


def deuterium():
    """Static 2H powder pattern (quadratic coupling), dim 144 < 200: expm branch, full grid."""
    w = W.deuterium()
    g = W.zcwn_grid(w.n_orient)
    fid = oracle_powder(w, g)
    save('deuterium_powder_fp64.npz', fid=fid, seed=w.seed, nsteps=w.nsteps, n_orient=w.n_orient)


def grids():
    """kernel/grids/leb_2ang_rank_5.mat of the reference (the grid of
    tests/kernel/test_ctx_powder_average.m) as arrays."""
    from spinach_gb300 import contexts as X
    al, be, ga, w = X.load_grid('/root/reference/kernel/grids/leb_2ang_rank_5.mat')
    save('grid_leb_2ang_rank_5.npz', alphas=al, betas=be, gammas=ga, weights=w)


def main():
    if 'grids' in sys.argv[1:]:
        return grids()
    if 'large' in sys.argv[1:]:
        return large_systems()
    if 'deuterium' in sys.argv[1:]:
        return deuterium()
    t = time.time()
    # c0: full 200-point grid, 1024 steps, default tolerances (expm branch, dim < 200)
    w = W.c0()
    g = W.zcwn_grid(w.n_orient)
    fid = oracle_powder(w, g)
    save('c0_powder_fp64.npz', fid=fid, seed=w.seed, nsteps=w.nsteps, n_orient=w.n_orient)
    # c1: three orientations, 2048 steps; Krylov branch (step.m) and propagator branch
    w = W.c1()
    al, be, ga, wt = W.zcwn_grid(w.n_orient)
    sel = np.array([0, 333, 777])
    sub = (al[sel], be[sel], ga[sel], np.full(sel.size, 1.0 / sel.size))
    fk = oracle_powder(w, sub, krylov=True, sum_up=False)
    save('c1_orient_krylov_fp64.npz', sel=sel, fids=np.array(fk), seed=w.seed, nsteps=w.nsteps)
    fp = oracle_powder(w, (sub[0][:1], sub[1][:1], sub[2][:1], np.ones(1)), krylov=False, sum_up=False)
    save('c1_orient_propagator_fp64.npz', sel=sel[:1], fids=np.array(fp), seed=w.seed, nsteps=w.nsteps)
    large_systems()
    print('done in', round(time.time() - t, 1), 's')


if __name__ == '__main__':
    main()
