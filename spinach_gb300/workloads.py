"""Seeded synthetic spin systems for the powder-FID workloads.

Each workload is a static powder experiment (kernel/contexts/powder.m with
experiments/acquire.m) on a synthetic molecule:
  * ``c0``  13C-1H-1H, full basis (dim 64), 200-point zcwn grid, 1024 steps of 10 us;
  * ``c1``  13C + 6 1H, IK-0 level 3 basis (dim 1156), T1/T2 relaxation,
            1000-point zcwn grid, 2048 steps of 5 us;
  * ``c2``  64 systems of 3-8 spins (full basis up to 4^6 = 4096, IK-0(3) above),
            400 orientations each, 1024 steps of 10 us;
  * ``c4``  X-band EPR radical: electron, 14N and 10 1H hyperfines, IK-1 level 3
            basis on the electron-centred coupling graph.
Interaction draws follow the workload description: isotropic shifts U(0,200)
ppm (13C) and U(0,10) ppm (1H), CSA anisotropy U(-100,100) ppm with asymmetry
U(0,1) and uniformly random orientation, dipolar couplings from Cartesian
coordinates with 1.1 A C-H bonds.  Geometry: the first two protons sit on the
13C; further protons come in CH2 pairs on spinless (12C) carbons 1.53 A away,
every H-H distance at least 1.5 A.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from . import spin_system as ssm


@dataclass
class Workload:
    name: str
    isotopes: list
    magnet: float
    zeeman_eigs: list
    zeeman_euler: list
    coordinates: list | None
    coupling_eigs: dict | None
    coupling_euler: dict | None
    r1: list | None
    r2: list | None
    approximation: str
    level: int
    assumptions: str
    rho0: tuple          # (operator, isotope)
    coil: tuple
    dt: float
    nsteps: int
    n_orient: int
    seed: int
    extra: dict = field(default_factory=dict)


def zcwn_grid(n: int):
    """Two-angle zcwn grid (kernel/grids/grid_fibon.m:70-78) with uniform weights."""
    phi = (1 + math.sqrt(5)) / 2
    k = np.arange(n)
    return (np.zeros(n), np.arccos(2 * (k / n) - 1), 2 * np.pi * k / phi ** 2, np.full(n, 1.0 / n))


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def _geometry(n_h: int, rng) -> list:
    coords = [np.zeros(3)]
    anchors = [np.zeros(3)]
    while len(anchors) < 1 + max(0, (n_h - 1) // 2):
        for _ in range(100000):
            a = 1.53 * _unit(rng)
            if all(np.linalg.norm(a - b) > 2.0 for b in anchors[1:]):
                anchors.append(a)
                break
        else:
            raise RuntimeError('could not place carbon anchors')
    for i in range(n_h):
        anc = anchors[0] if i < 2 else anchors[1 + (i - 2) // 2]
        for _ in range(100000):
            c = anc + 1.1 * _unit(rng)
            if all(np.linalg.norm(c - x) > 1.5 for x in coords[1:]) and \
               all(np.linalg.norm(c - b) > 1.05 for b in anchors if b is not anc):
                coords.append(c)
                break
        else:
            raise RuntimeError('could not place protons')
    return coords


def _csa(rng, iso_range):
    d = rng.uniform(*iso_range)
    a = rng.uniform(-100, 100)
    e = rng.uniform(0, 1)
    eigs = [d + a * (-(1 + e) / 2), d + a * (-(1 - e) / 2), d + a]
    eul = [rng.uniform(0, 2 * np.pi), math.acos(rng.uniform(-1, 1)), rng.uniform(0, 2 * np.pi)]
    return eigs, eul


def nmr_molecule(name, n_spins, seed, approximation, level, dt, nsteps, n_orient, relax):
    rng = np.random.default_rng(seed)
    iso = ['13C'] + ['1H'] * (n_spins - 1)
    coords = _geometry(n_spins - 1, rng)
    eigs, eul = [], []
    for s in iso:
        e, u = _csa(rng, (0, 200) if s == '13C' else (0, 10))
        eigs.append(e)
        eul.append(u)
    r1 = r2 = None
    if relax:
        r1 = list(rng.uniform(1, 50, n_spins))
        r2 = list(rng.uniform(1, 50, n_spins))
    return Workload(name, iso, 14.1, eigs, eul, coords, None, None, r1, r2, approximation, level,
                    'nmr', ('Lx', '13C'), ('L+', '13C'), dt, nsteps, n_orient, seed)


def deuterium(seed: int = 5) -> Workload:
    """Static 2H powder pattern: a C-D group with one proton (2H at 1.09 A from
    the 13C, the proton at 1.09 A on another bond) at 14.1 T, 2H quadratic
    coupling with C_Q about 170 kHz and asymmetry up to 0.2 along the C-D bond,
    13C and 2H shift tensors, dipolar couplings from the geometry; full basis
    (dim 144), 'nmr'; Lx(2H) detected with L+(2H), 400 orientations x 1024
    steps of 2 us."""
    rng = np.random.default_rng(seed)
    cd = _unit(rng)
    ch = _unit(rng)
    while abs(float(cd @ ch)) > 0.5:
        ch = _unit(rng)
    coords = [1.09 * cd, np.zeros(3), 1.09 * ch]
    eigs, eul = [], []
    for rng_iso in ((0, 5), (0, 200), (0, 10)):
        e, u = _csa(rng, rng_iso)
        eigs.append(e)
        eul.append(u)
    cq = rng.uniform(160e3, 180e3)
    eta = rng.uniform(0.0, 0.2)
    # principal axis of the quadratic coupling along the C-D bond
    bet = math.acos(float(np.clip(cd[2], -1, 1)))
    alp = math.atan2(float(cd[1]), float(cd[0]))
    ceigs = {(0, 0): [-(1 - eta) * cq / 6, -(1 + eta) * cq / 6, cq / 3]}
    ceul = {(0, 0): [alp, bet, rng.uniform(0, 2 * np.pi)]}
    return Workload('deuterium', ['2H', '13C', '1H'], 14.1, eigs, eul, coords, ceigs, ceul, None, None, 'none', 0,
                    'nmr', ('Lx', '2H'), ('L+', '2H'), 2e-6, 1024, 400, seed)


def c0(seed: int = 0) -> Workload:
    return nmr_molecule('c0', 3, seed, 'none', 0, 10e-6, 1024, 200, relax=False)


def c1(seed: int = 1) -> Workload:
    return nmr_molecule('c1', 7, seed, 'IK-0', 3, 5e-6, 2048, 1000, relax=True)


def c2(seed: int = 2, n_systems: int = 64) -> list:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_systems):
        ns = int(rng.integers(3, 9))
        full = 4 ** ns <= 4096
        out.append(nmr_molecule(f'c2.{i}', ns, seed * 1000 + i, 'none' if full else 'IK-0',
                                0 if full else 3, 10e-6, 1024, 400, relax=True))
    return out


def c2_4096(seed: int = 2) -> Workload:
    """The first dim-4096 system of c2 (six spins, full basis)."""
    return next(w for w in c2(seed) if len(w.isotopes) == 6)


def c4(seed: int = 4) -> Workload:
    """X-band nitroxide-like radical (0.34 T): electron with an axial g tensor,
    one 14N and ten 1H hyperfine couplings, T2 on the electron."""
    rng = np.random.default_rng(seed)
    iso = ['E', '14N'] + ['1H'] * 10
    giso = 2.006
    dg = rng.uniform(0.002, 0.01)
    geigs = [giso - dg / 3, giso - dg / 3, giso + 2 * dg / 3]
    eul_e = [rng.uniform(0, 2 * np.pi), math.acos(rng.uniform(-1, 1)), rng.uniform(0, 2 * np.pi)]
    aiso = rng.uniform(30e6, 45e6)
    aan = rng.uniform(20e6, 60e6)
    ceigs = {(0, 1): [aiso - aan / 3, aiso - aan / 3, aiso + 2 * aan / 3]}
    ceul = {(0, 1): [rng.uniform(0, 2 * np.pi), math.acos(rng.uniform(-1, 1)), rng.uniform(0, 2 * np.pi)]}
    for h in range(10):
        a = rng.normal(0.0, 3e6)
        ceigs[(0, 2 + h)] = [a, a, a]
    n = len(iso)
    r1 = [0.0] * n
    r2 = [0.0] * n
    r2[0] = 1.0 / rng.uniform(0.2e-6, 2e-6)
    return Workload('c4', iso, 0.34, [geigs] + [None] * (n - 1), [eul_e] + [None] * (n - 1), None,
                    ceigs, ceul, r1, r2, 'IK-1', 3, 'esr', ('Lx', 'E'), ('L+', 'E'), 1e-9, 4096, 4000, seed)


WORKLOADS = {'c0': c0, 'c1': c1, 'c4': c4}


@dataclass
class Liouvillian:
    """Inputs of one powder run in the form the engine uploads."""
    I: sp.csr_matrix
    terms: dict          # (rank, k, m) -> csr
    R: sp.csr_matrix
    rho0: np.ndarray
    coil: np.ndarray
    dim: int


def spin_system_of(w: Workload) -> ssm.SpinSystem:
    return ssm.make_spin_system(w.isotopes, w.magnet, zeeman_eigs=w.zeeman_eigs,
                                zeeman_euler=w.zeeman_euler, coordinates=w.coordinates,
                                coupling_eigs=w.coupling_eigs, coupling_euler=w.coupling_euler,
                                r1=w.r1, r2=w.r2)


def build(w: Workload) -> Liouvillian:
    """Host setup of a workload: I, Q{r}{k,m}, R, rho0, coil."""
    ss = spin_system_of(w)
    basis = ssm.decoupled_basis(ss, ssm.build_basis(ss, w.approximation, w.level), w.extra.get('decouple'))
    fac = ssm.factory_for(ss, basis)
    H = ssm.rotational_hamiltonian(ss, basis, w.assumptions, fac)
    R = sp.diags(ssm.relaxation_diagonal(ss, basis, w.extra.get('damp_rate', 0.0))).tocsr().astype(complex)
    iso = H.iso
    for s, off in _offsets(w):
        iso = iso + 2 * math.pi * off * fac.operator([('Lz', s)])
    if w.extra.get('homodec'):                  # acquire.m:54-62: L + 2*pi*pwr*oper
        op, name, pwr = w.extra['homodec']
        for s in [i for i, x in enumerate(w.isotopes) if x == name]:
            iso = iso + 2 * math.pi * pwr * fac.operator([(op, s)])
    return Liouvillian(iso, H.aniso, R, fac.state(*w.rho0), fac.state(*w.coil), basis.dim)


def _offsets(w: Workload):
    """(spin, offset Hz) of w.extra['offset'] = {isotope: Hz}: the frequency
    offsets of powder.m's frqoffset call (kernel/frqoffset.m)."""
    out = []
    for iso_name, off in (w.extra.get('offset') or {}).items():
        if iso_name not in w.isotopes:
            raise ValueError(f'offset for {iso_name}, which is not in the system')
        if off != 0:
            out += [(s, float(off)) for s, name in enumerate(w.isotopes) if name == iso_name]
    return out


@dataclass
class BuildSpec:
    """Input of the on-GPU construction of a workload (Engine.build_system)."""
    monomials: object                 # spin_system.HamiltonianMonomials
    r_diag: np.ndarray
    rho0: np.ndarray
    coil: np.ndarray
    dim: int


def build_spec(w: Workload) -> BuildSpec:
    """Host half of the on-GPU setup: basis, monomials, relaxation, states."""
    ss = spin_system_of(w)
    basis = ssm.decoupled_basis(ss, ssm.build_basis(ss, w.approximation, w.level), w.extra.get('decouple'))
    fac = ssm.factory_for(ss, basis)
    hm = ssm.hamiltonian_monomials(ss, basis, w.assumptions)
    extra = [(s, 2, 2 * math.pi * o) for s, o in _offsets(w)]          # Lz: code 2
    if w.extra.get('homodec'):
        op, name, pwr = w.extra['homodec']
        for s in [i for i, x in enumerate(w.isotopes) if x == name]:
            extra += [(s, code, 2 * math.pi * pwr * f) for code, f in ssm.OperatorFactory._CODE[op]]
    if extra:                                   # isotropic one-spin monomials
        hm.mono_term = np.concatenate([hm.mono_term, np.zeros(len(extra), np.int32)])
        hm.mono_spins = np.concatenate([hm.mono_spins, np.array([[s, -1] for s, _, _ in extra], np.int32)])
        hm.mono_codes = np.concatenate([hm.mono_codes, np.array([[c, 0] for _, c, _ in extra], np.int32)])
        hm.mono_coefs = np.concatenate([hm.mono_coefs, np.array([v for _, _, v in extra], np.complex128)])
    return BuildSpec(hm, ssm.relaxation_diagonal(ss, basis, w.extra.get('damp_rate', 0.0)), fac.state(*w.rho0), fac.state(*w.coil), basis.dim)


def c4_small(seed: int = 4, n_protons: int = 2) -> Workload:
    """The c4 radical cut to ``n_protons`` protons in the full basis (parity-test size)."""
    w = c4(seed)
    keep = 2 + n_protons
    w.name = f'c4_small{n_protons}'
    w.isotopes = w.isotopes[:keep]
    w.zeeman_eigs = w.zeeman_eigs[:keep]
    w.zeeman_euler = w.zeeman_euler[:keep]
    w.coupling_eigs = {k: v for k, v in w.coupling_eigs.items() if max(k) < keep}
    w.coupling_euler = {k: v for k, v in w.coupling_euler.items() if max(k) < keep}
    w.r1, w.r2 = w.r1[:keep], w.r2[:keep]
    w.approximation, w.level = 'none', 0
    w.nsteps, w.n_orient = 256, 8
    return w
