"""Oracle-side construction of the workloads (test helper)."""
import numpy as np

from oracle import spinach_ref as R


def oracle_system(w, tol_mode='default', krylov=False):
    inter = dict(zeeman=dict(eigs=w.zeeman_eigs, euler=w.zeeman_euler))
    if w.coordinates is not None:
        inter['coordinates'] = w.coordinates
    if w.coupling_eigs is not None:
        inter['coupling'] = dict(eigs=w.coupling_eigs, euler=w.coupling_euler or {})
    if w.extra.get('damp_rate'):
        inter.setdefault('relaxation', []).append('damp')
        inter['damp_rate'] = w.extra['damp_rate']
    if w.r1 is not None:
        inter.setdefault('relaxation', []).append('t1_t2')
        inter['r1_rates'] = w.r1
        inter['r2_rates'] = w.r2
    sys_ = dict(isotopes=w.isotopes, magnet=w.magnet, enable=['krylov'] if krylov else [])
    ss = R.create(sys_, inter, tol_mode)
    ss = R.basis(ss, dict(approximation=w.approximation, level=w.level, space_level=1))
    ss, I, Q = R.powder_setup(ss, w.assumptions)
    if w.extra.get('offset'):                   # powder.m:157, frqoffset.m
        spins = list(w.extra['offset'])
        I = R.frqoffset(ss, I, spins, [w.extra['offset'][s] for s in spins])
    return ss, I, Q


def oracle_powder(w, grid, nsteps=None, tol_mode='default', krylov=False, sum_up=True):
    ss, I, Q = oracle_system(w, tol_mode, krylov)
    nsteps = w.nsteps if nsteps is None else nsteps
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=nsteps + 1)
    if w.extra.get('decouple'):
        par['decouple'] = list(w.extra['decouple'])
    if w.extra.get('homodec'):
        op, iso, pwr = w.extra['homodec']
        par['homodec_oper'] = R.operator(ss, op, iso)
        par['homodec_pwr'] = pwr
    return R.powder(ss, par, w.assumptions, grid, setup=(I, Q), sum_up=sum_up)


def rel_err(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))
