"""Generate the FP64 oracle fixtures used by the GPU parity tests.

Run from the repository root:  python tests/golden/make_golden.py
(``python tests/golden/make_golden.py large`` for the cluster-sized
systems, ``... deuterium`` for the quadratic-coupling workload,
``... sequences`` for the pulse sequences and MAS contexts, ``... grids``
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


SEQ_SEL = np.array([7, 66, 131, 180])
SEQ_W = np.array([0.1, 0.4, 0.3, 0.2])


def sequence_cases():
    """The c0 system (13C + 2 1H, dim 64) at four zcwn orientations with
    every restated pulse sequence and both MAS contexts: name -> (function of
    (ss, I, Q, angles), parameters).  Shared with the regression test."""
    from oracle import spinach_ref as R
    from oracle_cases import oracle_system
    w = W.c0()
    ss, I, Q = oracle_system(w)
    Ly = R.operator(ss, 'Ly', '13C')
    base = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, 'L+', '13C'))
    cases = {
        'hp_acquire': (R.hp_acquire, dict(base, pulse_op=Ly, pulse_angle=np.pi / 2, echo_time=37 * w.dt,
                                          echo_oper=R.operator(ss, 'Lx', '13C'), echo_angle=np.pi,
                                          sweep=1 / w.dt, npoints=64)),
        'cpmg': (R.cpmg, dict(base, pulse_op=Ly, timestep=w.dt, npoints=24, nloops=2)),
        'eseem': (R.eseem, dict(base, pulse_op=Ly, timestep=2 * w.dt, npoints=48)),
        'oopeseem': (R.oopeseem, dict(base, pulse_op=Ly, timestep=2 * w.dt, npoints=48)),
        'deer_3p_hard_deer': (R.deer_3p_hard, dict(base, coil_prob=base['coil'], ex_prob=Ly,
                                                   ex_pump=R.operator(ss, 'Ly', '1H'), stepsize=w.dt,
                                                   nsteps=40)),
        'deer_3p_hard_echo': (R.deer_3p_hard_echo, dict(base, ex_prob=Ly, ex_pump=R.operator(ss, 'Ly', '1H'),
                                                        ta=60 * w.dt, tb=20 * w.dt, tc=40 * w.dt, nsteps=40)),
    }
    out = {k: (lambda f, p: (lambda a: R.powder_orientation_sequence(ss, I, Q, p, a, f)))(f, p)
           for k, (f, p) in cases.items()}
    mas = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=161,
               rate=12.5e3, axis=(1.0, 1.0, 1.0), max_rank=4)
    out['singlerot'] = lambda a: R.singlerot_orientation_fid(ss, I, Q, mas, a)
    out['floquet'] = lambda a: R.floquet_orientation_fid(ss, I, Q, mas, a)
    return w, out


def sequences():
    w, cases = sequence_cases()
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    res = {}
    for name, f in cases.items():
        res[name] = sum(SEQ_W[i] * f((al[j], be[j], ga[j])) for i, j in enumerate(SEQ_SEL))
    save('c0_sequences_fp64.npz', sel=SEQ_SEL, weights=SEQ_W, seed=w.seed, **res)


def main():
    if 'sequences' in sys.argv[1:]:
        return sequences()
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
