"""Generate the FP64 oracle fixtures used by the GPU parity tests.

Run from the repository root:  python tests/golden/make_golden.py
(``python tests/golden/make_golden.py large`` for the cluster-sized
systems, ``... deuterium`` for the quadratic-coupling workload,
``... sequences`` for the pulse sequences and MAS contexts, ``... wide``
for the full c1 powder, many c1/c4 orientations, every c2 dimension and the
paranoia-mode propagator branch (parallel over the host cores), ``... powders``
for the whole c4 powder and the remaining c2 whole powders (about an hour on
8 cores), ``... grids
<reference root>`` to copy the reference's 14-point Lebedev grid out of its
grid file, which needs the reference source tree; the root can also come
from the SPINACH_ROOT environment variable).  Writes tests/golden/*.npz.  Inputs are the seeded workloads of
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


def grids(root):
    """kernel/grids/leb_2ang_rank_5.mat of the reference (the grid of
    tests/kernel/test_ctx_powder_average.m) as arrays; ``root`` is the
    reference's source tree."""
    from spinach_gb300 import contexts as X
    if not root:
        raise SystemExit('give the reference source tree: make_golden.py grids <root> (or SPINACH_ROOT)')
    al, be, ga, w = X.load_grid(os.path.join(root, 'kernel', 'grids', 'leb_2ang_rank_5.mat'))
    save('grid_leb_2ang_rank_5.npz', alphas=al, betas=be, gammas=ga, weights=w)


_SYSTEMS = {}


def _workload(kind, idx):
    if kind == 'c2':
        return W.c2()[idx]
    return {'c1': W.c1, 'c4': W.c4}[kind]()


def _orient_fids(task):
    """Worker: per-orientation FP64 FIDs of grid points ``sel`` of a workload
    (one oracle setup per worker and system)."""
    from oracle import spinach_ref as R
    from oracle_cases import oracle_system
    kind, idx, sel, tol_mode, krylov = task
    w = _workload(kind, idx)
    key = (kind, idx, tol_mode, krylov)
    if key not in _SYSTEMS:
        _SYSTEMS[key] = oracle_system(w, tol_mode, krylov)
    ss, I, Q = _SYSTEMS[key]
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.asarray(sel)
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=w.nsteps + 1)
    grid = (al[sel], be[sel], ga[sel], np.ones(sel.size))
    return sel, np.array(R.powder(ss, par, w.assumptions, grid, setup=(I, Q), sum_up=False))


def _pool_fids(pool, kind, idx, sel, tol_mode='default', krylov=True, chunk=8):
    """Per-orientation FIDs of the grid points ``sel``, computed in parallel,
    returned in the order of ``sel``."""
    sel = np.asarray(sel)
    tasks = [(kind, idx, sel[i:i + chunk].tolist(), tol_mode, krylov) for i in range(0, sel.size, chunk)]
    out = {}
    for s, f in pool.imap_unordered(_orient_fids, tasks):
        for j, fj in zip(s, f):
            out[int(j)] = fj
    return np.array([out[int(j)] for j in sel])


def wide():
    """Wide parity fixtures, parallel over the host cores (spawned workers,
    one BLAS thread each):
      * c1: the whole 1000-orientation powder FID (Krylov branch, summed in
        grid order as powder.m:280-287 does) and 32 per-orientation FIDs;
      * c1: two orientations of the default propagator branch with
        prop_chop = eps ('paranoia', kernel/utilities/tolerances.m:97-100);
      * c4: 24 per-orientation FIDs (Krylov branch);
      * c2: four orientations of the first system of every dimension, and the
        whole 400-orientation powder of the dim-64, -256 and -1024 systems."""
    import multiprocessing as mp
    for v in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[v] = '1'
    t0 = time.time()
    with mp.get_context('spawn').Pool(os.cpu_count()) as pool:
        w = W.c1()
        fids = _pool_fids(pool, 'c1', 0, np.arange(w.n_orient), chunk=20)
        _, _, _, wt = W.zcwn_grid(w.n_orient)
        fid = wt[0] * fids[0]
        for n in range(1, w.n_orient):
            fid = fid + wt[n] * fids[n]
        sel = np.linspace(0, w.n_orient - 1, 32).round().astype(int)
        save('c1_powder_krylov_fp64.npz', fid=fid, sel=sel, fids=fids[sel], seed=w.seed, nsteps=w.nsteps,
             n_orient=w.n_orient)
        print('c1 powder', round(time.time() - t0, 1), 's')
        psel = np.array([0, 611])
        fp = _pool_fids(pool, 'c1', 0, psel, tol_mode='paranoia', krylov=False, chunk=1)
        save('c1_orient_propagator_paranoia_fp64.npz', sel=psel, fids=fp, seed=w.seed, nsteps=w.nsteps)
        print('c1 paranoia', round(time.time() - t0, 1), 's')
        w = W.c4()
        sel = np.linspace(7, w.n_orient - 1, 24).round().astype(int)
        save('c4_orients_krylov_fp64.npz', sel=sel, fids=_pool_fids(pool, 'c4', 0, sel, chunk=1), seed=w.seed,
             nsteps=w.nsteps)
        print('c4', round(time.time() - t0, 1), 's')
        ws = W.c2()
        dims = {}
        for i, x in enumerate(ws):
            d = W.build(x).dim
            dims.setdefault(d, i)
        for d, i in sorted(dims.items()):
            x = ws[i]
            sel = np.array([13, 111, 257, 389])
            kw = dict(system=i, dim=d, sel=sel, fids=_pool_fids(pool, 'c2', i, sel, chunk=1), seed=x.seed,
                      nsteps=x.nsteps)
            if d <= 1024:
                _, _, _, wt = W.zcwn_grid(x.n_orient)
                f = _pool_fids(pool, 'c2', i, np.arange(x.n_orient), chunk=10)
                p = wt[0] * f[0]
                for n in range(1, x.n_orient):
                    p = p + wt[n] * f[n]
                kw['fid'] = p
            save(f'c2_dim{d}_krylov_fp64.npz', **kw)
            print('c2 dim', d, round(time.time() - t0, 1), 's')


def wide_powders():
    """The whole powder FIDs the 'wide' fixtures leave out, parallel over the
    host cores: config 4's 4000-orientation powder (Krylov branch, summed in
    grid order) and the 400-orientation powders of the c2 systems of
    dimension 1156, 1789 and 4096 (added to their c2_dim*_krylov_fp64.npz)."""
    import multiprocessing as mp
    for v in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[v] = '1'
    t0 = time.time()
    with mp.get_context('spawn').Pool(os.cpu_count()) as pool:
        ws = W.c2()
        for d in (1156, 1789, 4096):
            name = f'c2_dim{d}_krylov_fp64.npz'
            old = dict(np.load(os.path.join(HERE, name)))
            i = int(old['system'])
            x = ws[i]
            _, _, _, wt = W.zcwn_grid(x.n_orient)
            f = _pool_fids(pool, 'c2', i, np.arange(x.n_orient), chunk=4)
            p = wt[0] * f[0]
            for n in range(1, x.n_orient):
                p = p + wt[n] * f[n]
            old['fid'] = p
            save(name, **old)
            print('c2 dim', d, round(time.time() - t0, 1), 's', flush=True)
        w = W.c4()
        _, _, _, wt = W.zcwn_grid(w.n_orient)
        f = _pool_fids(pool, 'c4', 0, np.arange(w.n_orient), chunk=10)
        fid = wt[0] * f[0]
        for n in range(1, w.n_orient):
            fid = fid + wt[n] * f[n]
        save('c4_powder_krylov_fp64.npz', fid=fid, seed=w.seed, nsteps=w.nsteps, n_orient=w.n_orient)
        print('c4 powder', round(time.time() - t0, 1), 's', flush=True)


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
        rest = sys.argv[sys.argv.index('grids') + 1:]
        return grids(rest[0] if rest else os.environ.get('SPINACH_ROOT'))
    if 'wide' in sys.argv[1:]:
        return wide()
    if 'powders' in sys.argv[1:]:
        return wide_powders()
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
