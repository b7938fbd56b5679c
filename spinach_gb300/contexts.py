"""Spinach's calling convention on the GPU engine.

``create(sys, inter)`` and ``basis(spin_system, bas)`` take the reference's
input structures (kernel/create.m, kernel/basis.m) as dicts, with 0-based spin
indices in the coupling keys; ``state`` and ``operator`` build Liouville
vectors and commutation superoperators (kernel/state.m, kernel/operator.m);
``powder(spin_system, pulse_sequence, parameters, assumptions)``,
``crystal(...)``, ``singlerot(...)`` and ``floquet(...)`` run the contexts
(kernel/contexts/powder.m, crystal.m, singlerot.m, floquet.m) with the pulse
sequences ``'acquire'``, ``'hp_acquire'``, ``'cpmg'``, ``'eseem'``,
``'oopeseem'``, ``'deer_3p_hard_deer'``, ``'deer_3p_hard_echo'`` and
``'inv_rec'`` (experiments/*.m; the two MAS contexts run acquire,
hp_acquire and cpmg), the parameters named as there.  Every orientation runs
on the GPU; the host only prepares the system.

Supported fields.  sys: isotopes, magnet.  inter: zeeman.eigs/euler (ppm, or
g for electrons), coordinates (Angstrom), coupling.eigs/euler/scalar (Hz,
keys (a, b); (a, a) is a quadratic coupling), relaxation (['t1_t2'],
['damp']), r1_rates, r2_rates, damp_rate, temperature.  bas: approximation
('none', 'IK-0', 'IK-1'), level, projections.  parameters: grid (alphas,
betas, gammas, weights, a grid file, or 'single_crystal'), rho0 / coil
(vectors, or (operator, isotope) pairs; rho0 may be a function of (alpha,
beta, gamma)), sweep, npoints, spins + offset, decouple, homodec_oper +
homodec_pwr, dead_time, needs (['iso_eq'] or ['aniso_eq'], with inter
temperature), sum_up, pulse_op, pulse_angle, echo_time, echo_oper,
echo_angle, nloops, timestep; DEER: ex_prob, ex_pump, coil_prob, stepsize,
nsteps, output ('brief'), ta, tb, tc; inv_rec: n_delays, max_delay;
crystal: orientation; singlerot and floquet: rate, axis, max_rank.
``engine`` (an Engine) and ``precision`` (engine.FP64 or FP32) are optional
keyword arguments.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

from . import engine as E
from . import singlerot as SR
from . import spin_system as S


@dataclass
class System:
    """A spin system with its basis (the reference's ``spin_system`` after
    create() and basis())."""
    ss: S.SpinSystem
    basis: S.Basis | None = None
    damp_rate: float = 0.0
    temperature: float | None = None

    @property
    def isotopes(self) -> list:
        return self.ss.isotopes

    def factory(self) -> S.OperatorFactory:
        if self.basis is None:
            raise ValueError('call basis() before building states or operators')
        return S.factory_for(self.ss, self.basis)


def create(sys: dict, inter: dict) -> System:
    """kernel/create.m: interaction tensors from the sys / inter structures."""
    isotopes = list(sys['isotopes'])
    z = inter.get('zeeman', {})
    cpl = inter.get('coupling', {})
    rl = list(inter.get('relaxation', []))
    unknown = [t for t in rl if t not in ('t1_t2', 'damp')]
    if unknown:
        raise ValueError(f'relaxation theories {unknown} are not supported')
    r1 = inter.get('r1_rates') if 't1_t2' in rl else None
    r2 = inter.get('r2_rates') if 't1_t2' in rl else None
    ss = S.make_spin_system(isotopes, float(sys['magnet']), zeeman_eigs=z.get('eigs'),
                            zeeman_euler=z.get('euler'), coordinates=inter.get('coordinates'),
                            coupling_scalar=cpl.get('scalar'), coupling_eigs=cpl.get('eigs'),
                            coupling_euler=cpl.get('euler'), r1=r1, r2=r2)
    damp = float(np.mean(np.diag(np.atleast_2d(inter.get('damp_rate', 0.0))))) if 'damp' in rl else 0.0
    return System(ss, None, damp, inter.get('temperature'))


def basis(spin_system: System, bas: dict) -> System:
    """kernel/basis.m: the spherical-tensor Liouville basis."""
    b = S.build_basis(spin_system.ss, bas.get('approximation', 'none'), int(bas.get('level', 0)),
                      projections=bas.get('projections'))
    return System(spin_system.ss, b, spin_system.damp_rate, spin_system.temperature)


def state(spin_system: System, op: str, isotope: str) -> np.ndarray:
    """kernel/state.m: sum over the spins of an isotope of op, as a Liouville vector."""
    return spin_system.factory().state(op, isotope)


def operator(spin_system: System, op: str, isotope: str) -> sp.csr_matrix:
    """kernel/operator.m ('comm'): the commutation superoperator of sum_s op(s)."""
    spins = [i for i, x in enumerate(spin_system.isotopes) if x == isotope]
    if not spins:
        raise ValueError('no such spins in the system')
    f = spin_system.factory()
    return sum(f.operator([(op, s)]) for s in spins)


def _vector(spin_system: System, v) -> np.ndarray:
    if isinstance(v, (tuple, list)) and len(v) == 2 and isinstance(v[0], str):
        return state(spin_system, v[0], v[1])
    return np.asarray(v, complex)


def _matrix(spin_system: System, m):
    if isinstance(m, (tuple, list)) and len(m) == 2 and isinstance(m[0], str):
        return operator(spin_system, m[0], m[1])
    return m


def _restrict(spin_system: System, full: System, v: np.ndarray) -> np.ndarray:
    """A vector of the full basis on the decoupled (smaller) basis."""
    if full.basis is spin_system.basis or v.shape[0] == spin_system.basis.dim:
        return v
    idx = np.searchsorted(full.basis.keys, spin_system.basis.keys)
    return v[idx]


def _name(pulse_sequence) -> str:
    return pulse_sequence if isinstance(pulse_sequence, str) else getattr(pulse_sequence, '__name__', '')


def _setup(spin_system: System, parameters: dict, assumptions: str, sequence: str):
    """[I,Q]=hamiltonian(assume(...)), frqoffset (powder.m:148-161), the
    relaxation (powder.m:263), acquire.m's decoupling and homodecoupling."""
    if spin_system.basis is None:
        raise ValueError('call basis() first')
    full = spin_system
    dec = list(parameters.get('decouple') or [])
    # acquire.m decouples (and homodecouples) the whole evolution, which the
    # smaller basis reproduces; hp_acquire.m decouples after its pulses
    if dec and sequence != 'acquire':
        raise ValueError('decoupling is supported for acquire')
    if 'homodec_oper' in parameters and sequence != 'acquire':
        raise ValueError('homodecoupling is part of acquire')
    work = (System(full.ss, S.decoupled_basis(full.ss, full.basis, dec), full.damp_rate, full.temperature)
            if dec else full)
    f = work.factory()
    H = S.rotational_hamiltonian(work.ss, work.basis, assumptions, f)
    iso = H.iso
    spins = list(parameters.get('spins') or [])
    offs = list(np.atleast_1d(parameters.get('offset', np.zeros(len(spins)))))
    if spins:
        if len(offs) != len(spins):
            raise ValueError('parameters.offset must have the same number of elements as parameters.spins')
        seen = {}
        for name, off in zip(spins, offs):
            if name not in work.isotopes:
                raise ValueError('parameters.spins refers to a spin that is not present in the system')
            if name in seen and seen[name] != off:
                raise ValueError('offsets on channels referring to the same spin must be the same')
            seen[name] = off
        for name, off in seen.items():
            if off:
                iso = iso + 2 * math.pi * float(off) * operator(work, 'Lz', name)
    if 'homodec_oper' in parameters:
        iso = iso + 2 * math.pi * float(parameters['homodec_pwr']) * _restrict_matrix(
            work, full, _matrix(full, parameters['homodec_oper']))
    R = sp.diags(S.relaxation_diagonal(work.ss, work.basis, work.damp_rate)).tocsr().astype(complex)
    needs = list(parameters.get('needs') or [])
    if any(n not in ('iso_eq', 'aniso_eq') for n in needs):
        raise ValueError("parameters.needs may contain 'iso_eq' and 'aniso_eq'")
    if needs and 'rho0' in parameters:
        raise ValueError('thermal equilibrium request conflicts with user-specified initial condition.')
    if needs:
        # powder.m:128-147: the lab-frame Hamiltonian as left-side products
        HL = S.rotational_hamiltonian(work.ss, work.basis, 'labframe', work.factory(), kind='left')
        rho0 = S.equilibrium_states(S.RotationalHamiltonian(HL.dim, HL.iso, {}), work.temperature)
    elif callable(parameters['rho0']):
        # powder.m:250-252: a function handle evaluated at every orientation;
        # the single rho0 is a placeholder (the states replace it)
        HL = None
        rho0 = np.zeros(work.basis.dim, complex)
        rho0[0] = 1.0
    else:
        HL = None
        rho0 = _restrict(work, full, _vector(full, parameters['rho0']))
    coil = _restrict(work, full, _vector(full, parameters['coil']))
    return work, full, iso, H.aniso, R, rho0, coil, HL


def _restrict_matrix(work: System, full: System, M):
    if work.basis is full.basis:
        return M
    idx = np.searchsorted(full.basis.keys, work.basis.keys)
    return sp.csr_matrix(M)[idx][:, idx]


def load_grid(path: str):
    """A spherical grid file of the reference (kernel/grids/*.mat, MATLAB v5
    format): (alphas, betas, gammas, weights) as flat float64 arrays."""
    import scipy.io as sio
    try:
        d = sio.loadmat(path)
    except NotImplementedError as e:              # v7.3 (HDF5) files
        raise ValueError(f'{path}: MATLAB v7.3 grid files are not readable here') from e
    missing = [k for k in ('alphas', 'betas', 'gammas', 'weights') if k not in d]
    if missing:
        raise ValueError(f'{path}: no {missing} in the grid file')
    return tuple(np.ascontiguousarray(np.ravel(d[k]), np.float64) for k in ('alphas', 'betas', 'gammas', 'weights'))


def _grid(parameters: dict):
    g = parameters['grid']
    if isinstance(g, str) and g == 'single_crystal':
        # kernel/grids/single_crystal.mat: one orientation at zero Euler angles, unit weight
        return (np.zeros(1), np.zeros(1), np.zeros(1), np.ones(1))
    if isinstance(g, str):
        g = load_grid(g)
    if isinstance(g, dict):
        g = (g['alphas'], g['betas'], g['gammas'], g['weights'])
    return tuple(np.ascontiguousarray(np.ravel(a), np.float64) for a in g)


def _run(eng, pulse_sequence, parameters, work, full, grid, precision, spc_dim: int = 1):
    """Runs the sequence on the uploaded system.  Pulse operators are
    projected into the context's spatial space, kron(speye(spc_dim), op), as
    hp_acquire.m:57,69 and cpmg.m:33 do (spc_dim = 1 for powder.m)."""
    al, be, ga, w = grid
    name = _name(pulse_sequence)

    def op(key):
        P = _restrict_matrix(work, full, _matrix(full, parameters[key]))
        return P if spc_dim == 1 else sp.kron(sp.identity(spc_dim), P, format='csr')

    if name == 'acquire':
        dt, n = 1.0 / float(parameters['sweep']), int(parameters['npoints']) - 1
        if 'dead_time' in parameters:
            prog = [('evolve', 1, float(parameters['dead_time']), False), ('evolve', n, dt)]
            return eng.run_sequence(al, be, ga, w, [], prog, precision=precision,
                                    per_orientation=not parameters.get('sum_up', 1))
        return eng.run(al, be, ga, w, dt, n, precision=precision, per_orientation=not parameters.get('sum_up', 1))
    if name == 'hp_acquire':
        ops = [op('pulse_op')]
        prog = [('pulse', 0, float(parameters['pulse_angle']))]
        if 'echo_time' in parameters:
            ops.append(op('echo_oper'))
            et = float(parameters['echo_time'])
            prog += [('evolve', 1, et, False), ('pulse', 1, float(parameters['echo_angle'])), ('evolve', 1, et, False)]
        prog.append(('evolve', int(parameters['npoints']) - 1, 1.0 / float(parameters['sweep'])))
        return eng.run_sequence(al, be, ga, w, ops, prog, precision=precision,
                                per_orientation=not parameters.get('sum_up', 1))
    if name == 'cpmg':
        P = op('pulse_op')
        return eng.run_cpmg(al, be, ga, w, float(parameters['timestep']), int(parameters['npoints']),
                            int(parameters['nloops']), P, precision=precision,
                            per_orientation=not parameters.get('sum_up', 1))
    if name == 'deer_3p_hard_deer':
        if spc_dim != 1:
            raise ValueError('deer_3p_hard_deer runs in the powder context on this engine')
        if parameters.get('output', 'brief') != 'brief':
            raise ValueError("deer_3p_hard_deer runs output='brief' on this engine")
        return eng.run_deer(al, be, ga, w, float(parameters['stepsize']), int(parameters['nsteps']), op('ex_prob'),
                            op('ex_pump'), precision=precision, per_orientation=not parameters.get('sum_up', 1))
    if name == 'inv_rec':
        # one program per recovery delay: the trajectory column k of inv_rec.m
        nd = int(parameters['n_delays'])
        if nd < 1:
            raise ValueError('parameters.n_delays must be a positive integer')
        dd, dt, n = float(parameters['max_delay']) / nd, 1.0 / float(parameters['sweep']), int(parameters['npoints']) - 1
        P = op('pulse_op')
        runs = []
        for k in range(nd + 1):
            prog = ([('pulse', 0, np.pi)] + ([('evolve', k, dd, False)] if k else []) +
                    [('pulse', 0, np.pi / 2), ('evolve', n, dt)])
            runs.append(eng.run_sequence(al, be, ga, w, [P], prog, precision=precision,
                                         per_orientation=not parameters.get('sum_up', 1)))
        return _Stacked(np.stack([r.fid for r in runs], axis=1),
                        None if runs[0].fids is None else np.stack([r.fids for r in runs], axis=-1))
    if name == 'deer_3p_hard_echo':
        # deer_3p_hard_echo.m: three hard pulses, three silent delays, the echo over tc
        ta, tb, tc, n = (float(parameters['ta']), float(parameters['tb']), float(parameters['tc']),
                         int(parameters['nsteps']))
        prog = [('pulse', 0, np.pi / 2), ('evolve', 1, tb, False), ('pulse', 1, np.pi),
                ('evolve', 1, ta - tb, False), ('pulse', 0, np.pi), ('evolve', 1, ta - 0.5 * tc, False),
                ('evolve', n, tc / n)]
        return eng.run_sequence(al, be, ga, w, [op('ex_prob'), op('ex_pump')], prog, precision=precision,
                                per_orientation=not parameters.get('sum_up', 1))
    if name in ('eseem', 'oopeseem'):
        if spc_dim != 1:
            raise ValueError(f'{name} runs in the powder context on this engine')
        P = op('pulse_op')
        return eng.run_eseem(al, be, ga, w, float(parameters['timestep']), int(parameters['npoints']), P,
                             precision=precision, per_orientation=not parameters.get('sum_up', 1),
                             out_of_phase=name == 'oopeseem')
    raise ValueError(f'pulse sequence {pulse_sequence!r} is not supported on this engine')


@dataclass
class _Stacked:
    """Several recorded programs side by side: fid is npoints x columns, fids
    (per orientation) n_orient x npoints x columns."""
    fid: np.ndarray
    fids: np.ndarray | None


def _answer(res, parameters):
    if parameters.get('sum_up', 1):
        return res.fid
    if res.fids is None:
        raise ValueError('no per-orientation outputs for this sequence')
    return list(res.fids)


def powder(spin_system: System, pulse_sequence, parameters: dict, assumptions: str, engine=None,
           precision: int = E.FP64):
    """kernel/contexts/powder.m:99-309: returns (answer, grid), the answer the
    weighted sum of the orientations' outputs (sum_up, default) or their list.
    For deer_3p_hard_deer the answer is the DEER trace (deer.deer_trace of
    the 'brief' output), detected on parameters['coil_prob']."""
    if _name(pulse_sequence) == 'deer_3p_hard_deer':
        parameters = dict(parameters, coil=parameters['coil_prob'])
    if _name(pulse_sequence) == 'inv_rec':
        # inv_rec.m makes its own rho0 (the isotropic equilibrium), coil (L+)
        # and pulse operator (Ly) from parameters.spins{1}
        if 'rho0' in parameters or parameters.get('needs'):
            raise ValueError('inv_rec starts from the isotropic thermal equilibrium')
        spin = list(parameters['spins'])[0]
        parameters = dict(parameters, needs=['iso_eq'], coil=('L+', spin), pulse_op=('Ly', spin))
    work, full, I, Q, R, rho0, coil, HL = _setup(spin_system, parameters, assumptions, _name(pulse_sequence))
    grid = _grid(parameters)
    eng = engine or E.Engine(0)
    try:
        eng.upload(I, Q, R, rho0, coil)
        if 'aniso_eq' in (parameters.get('needs') or []):
            # powder.m:244-248: the equilibrium at every orientation
            eng.set_initial_states(S.equilibrium_states(HL, work.temperature, *grid[:3]))
        elif callable(parameters.get('rho0')):
            f = parameters['rho0']
            eng.set_initial_states(np.array([_restrict(work, full, _vector(full, f(a, b, g)))
                                             for a, b, g in zip(*grid[:3])]))
        try:
            res = _run(eng, pulse_sequence, parameters, work, full, grid, precision)
        finally:
            eng.set_initial_states(None)
    finally:
        if engine is None:
            eng.close()
    return _answer(res, parameters), grid


def crystal(spin_system: System, pulse_sequence, parameters: dict, assumptions: str, engine=None,
            precision: int = E.FP64):
    """kernel/contexts/crystal.m:74-147: the sequence at the single
    orientation parameters['orientation'] (three Euler angles), H Hermitised
    as there; returns the answer alone.  A one-point powder on the engine."""
    o = np.asarray(parameters.get('orientation', []), np.float64).ravel()
    if o.size != 3 or not np.all(np.isfinite(o)):
        raise ValueError('parameters.orientation must be a row vector with three numbers')
    grid = (o[:1].copy(), o[1:2].copy(), o[2:3].copy(), np.ones(1))
    answer, _ = powder(spin_system, pulse_sequence, dict(parameters, grid=grid), assumptions, engine=engine,
                       precision=precision)
    return answer


def _mas_name(pulse_sequence, context: str, parameters: dict) -> str:
    name = _name(pulse_sequence)
    if name not in ('acquire', 'hp_acquire', 'cpmg'):
        raise ValueError(f'{context} runs acquire, hp_acquire or cpmg on this engine')
    if parameters.get('needs'):
        raise ValueError(f'{context} takes an explicit rho0 on this engine')
    return name


def singlerot(spin_system: System, pulse_sequence, parameters: dict, assumptions: str, engine=None,
              precision: int = E.FP64):
    """kernel/contexts/singlerot.m with acquire, hp_acquire or cpmg: the
    Fokker-Planck problem of rate, axis and max_rank, in the engine's upload
    form.  A grid named 'single_crystal' (or single_crystal=True) starts from
    one rotor point."""
    name = _mas_name(pulse_sequence, 'singlerot', parameters)
    work, full, I, Q, R, rho0, coil, _ = _setup(spin_system, parameters, assumptions, name)
    single = bool(parameters.get('single_crystal')) or parameters.get('grid') == 'single_crystal'
    grid = ((np.zeros(1), np.zeros(1), np.zeros(1), np.ones(1)) if parameters.get('grid') == 'single_crystal'
            else _grid(parameters))
    fp = SR.fokker_planck(I, Q, R, rho0, coil, int(parameters['max_rank']), float(parameters['rate']),
                          parameters['axis'], single_crystal=single)
    eng = engine or E.Engine(0)
    try:
        eng.upload(*fp)
        res = _run(eng, name, parameters, work, full, grid, precision, spc_dim=2 * int(parameters['max_rank']) + 1)
    finally:
        if engine is None:
            eng.close()
    return _answer(res, parameters), grid


def floquet(spin_system: System, pulse_sequence, parameters: dict, assumptions: str, engine=None,
            precision: int = E.FP64):
    """kernel/contexts/floquet.m with acquire, hp_acquire or cpmg: the
    Floquet problem of rate, axis and max_rank (Fourier components of the
    rotor-frame Hamiltonian), in the engine's upload form."""
    name = _mas_name(pulse_sequence, 'floquet', parameters)
    work, full, I, Q, R, rho0, coil, _ = _setup(spin_system, parameters, assumptions, name)
    grid = ((np.zeros(1), np.zeros(1), np.zeros(1), np.ones(1)) if parameters.get('grid') == 'single_crystal'
            else _grid(parameters))
    fs = SR.floquet_system(I, Q, R, rho0, coil, int(parameters['max_rank']), float(parameters['rate']),
                           parameters['axis'])
    eng = engine or E.Engine(0)
    try:
        eng.upload(*fs)
        res = _run(eng, name, parameters, work, full, grid, precision, spc_dim=2 * int(parameters['max_rank']) + 1)
    finally:
        if engine is None:
            eng.close()
    return _answer(res, parameters), grid
