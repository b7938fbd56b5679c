"""Host-side spin-system setup for the powder-FID engine.

This is the setup the reference runs once per powder call before its
orientation loop (kernel/contexts/powder.m:148-161): interaction tensors
(kernel/create.m), interaction strengths (kernel/assume.m), the spherical-tensor
Liouville basis (kernel/basis.m) and the isotropic part ``I`` plus rotational
basis ``Q{r}{k,m}`` of the Liouvillian (kernel/hamiltonian.m:44-790).  It is
written vectorised (numpy, one pass over the basis per operator) rather than as
the reference's per-descriptor loops, and it produces the sparse arrays the
GPU engine uploads.

Units follow the reference: Zeeman eigenvalues in ppm (nuclei) or as g values
(electrons), couplings in Hz, coordinates in Angstrom, relaxation rates in 1/s,
Liouvillians in rad/s.  Spin indices are 0-based.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

# CODATA values used by the reference (kernel/utilities/tolerances.m:348-360).
PLANCK_HBAR = 6.62607015e-34 / (2 * math.pi)
VACUUM_MU0 = 1.25663706127e-6
FREE_G = 2.00231930436092

# (multiplicity, gyromagnetic ratio in rad/s/T), kernel/spin.m:86-131.
NUCLEI = {
    'E': (2, -1.76085963023e11),
    '1H': (2, 2.6752218744e8),
    '2H': (3, 4.10662791e7),
    '13C': (2, 6.728284e7),
    '14N': (3, 1.9337792e7),
    '15N': (2, -2.71261804e7),
}

# Default ("safe") thresholds of kernel/utilities/tolerances.m.
DEFAULT_TOLS = dict(inter_cutoff=1e-10, liouv_zero=1e-10, prox_cutoff=100.0)


# ---------------------------------------------------------------------------
# Single-spin algebra
# ---------------------------------------------------------------------------

def _spin_ops(mult: int):
    s = (mult - 1) / 2
    mz = np.arange(mult - 1, -1, -1) - s
    up = np.zeros((mult, mult))
    for i in range(mult - 1):
        up[i, i + 1] = math.sqrt(s * (s + 1) - mz[i + 1] * (mz[i + 1] + 1))
    return up, up.T.copy(), np.diag(mz)


def _ist_matrices(mult: int) -> list:
    """Unnormalised irreducible spherical tensors T(l,m), ordered by code l*l+l-m
    (same recursion as kernel/operators/irr_sph_ten.m:61-75)."""
    up, dn, _ = _spin_ops(mult)
    out = []
    for l in range(mult):
        if l == 0:
            out.append(np.eye(mult))
            continue
        t = ((-1) ** l) * 2 ** (-l / 2) * np.linalg.matrix_power(up, l)
        out.append(t)
        for q in range(l - 1, -l - 1, -1):
            t = (dn @ t - t @ dn) / math.sqrt((l + q + 1) * (l - q))
            out.append(t)
    return out


def _product_tables(mult: int):
    """Left/right multiplication tables in the normalised IST basis:
    left[n, m, k] = <e_k|T_n e_m>, right[n, m, k] = <e_k|e_m T_n>
    (the quantity kernel/cache/ist_product_table.m tabulates)."""
    T = np.array(_ist_matrices(mult))                    # (d, mult, mult), real
    nrm = np.sqrt(np.einsum('kij,kij->k', T, T))
    E = T / nrm[:, None, None]
    left = np.einsum('kij,nil,mlj->nmk', E, T, E)
    right = np.einsum('kij,mil,nlj->nmk', E, E, T)
    left[np.abs(left) < 1e-15] = 0.0
    right[np.abs(right) < 1e-15] = 0.0
    return left, right


# ---------------------------------------------------------------------------
# Geometry helpers
# ---------------------------------------------------------------------------

def euler_dcm(a: float, b: float, g: float) -> np.ndarray:
    """ZYZ active rotation Rz(a) Ry(b) Rz(g) (kernel/conventions/transforms/euler2dcm.m)."""
    def rz(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
    cb, sb = math.cos(b), math.sin(b)
    ry = np.array([[cb, 0.0, sb], [0.0, 1.0, 0.0], [-sb, 0.0, cb]])
    return rz(a) @ ry @ rz(g)


def sph_components(M: np.ndarray):
    """Isotropic, rank-1 and rank-2 spherical components of a real 3x3 tensor in
    the order [+1,0,-1] and [+2..-2] (kernel/conventions/transforms/mat2sphten.m)."""
    M = np.asarray(M, float)
    iso = np.trace(M) / 3
    r1 = np.array([-0.5 * ((M[2, 0] - M[0, 2]) - 1j * (M[2, 1] - M[1, 2])),
                   1j / math.sqrt(2) * (M[0, 1] - M[1, 0]),
                   -0.5 * ((M[2, 0] - M[0, 2]) + 1j * (M[2, 1] - M[1, 2]))])
    sxy = M[0, 1] + M[1, 0]
    sxz = M[0, 2] + M[2, 0]
    syz = M[1, 2] + M[2, 1]
    dxy = M[0, 0] - M[1, 1]
    r2 = np.array([0.5 * (dxy - 1j * sxy), -0.5 * (sxz - 1j * syz),
                   (2 * M[2, 2] - M[0, 0] - M[1, 1]) / math.sqrt(6),
                   0.5 * (sxz + 1j * syz), 0.5 * (dxy + 1j * sxy)])
    return iso, r1, r2


# ---------------------------------------------------------------------------
# Spin system
# ---------------------------------------------------------------------------

@dataclass
class SpinSystem:
    """Interaction content of one molecule (the reference's ``spin_system``
    after ``create``): Zeeman and coupling tensors in rad/s, T1/T2 rates."""
    isotopes: list
    magnet: float
    zeeman: list                      # 3x3 rad/s (lab frame)
    couplings: dict                   # (a, b) -> 3x3 rad/s, a != b
    r1: np.ndarray
    r2: np.ndarray
    relaxation: bool
    tols: dict = field(default_factory=lambda: dict(DEFAULT_TOLS))

    @property
    def nspins(self) -> int:
        return len(self.isotopes)

    @property
    def mults(self) -> np.ndarray:
        return np.array([NUCLEI[i][0] for i in self.isotopes])

    @property
    def gammas(self) -> np.ndarray:
        return np.array([NUCLEI[i][1] for i in self.isotopes])

    @property
    def carriers(self) -> np.ndarray:
        return -self.gammas * self.magnet


def make_spin_system(isotopes, magnet, zeeman_eigs=None, zeeman_euler=None,
                     coordinates=None, coupling_scalar=None, coupling_eigs=None,
                     coupling_euler=None, r1=None, r2=None, tols=None) -> SpinSystem:
    """Build interaction tensors the way kernel/create.m:742-1046 does.

    zeeman_eigs[n]: principal values, ppm for nuclei / g for electrons.
    coupling_scalar / coupling_eigs: dicts keyed (a, b), Hz.
    coordinates: Angstrom, dipolar tensors as kernel/utilities/dipolar.m:150-177."""
    tols = dict(DEFAULT_TOLS, **(tols or {}))
    n = len(isotopes)
    gam = np.array([NUCLEI[i][1] for i in isotopes])
    mult = [NUCLEI[i][0] for i in isotopes]
    carrier = -gam * magnet
    zee = []
    for s in range(n):
        Z = np.zeros((3, 3))
        if zeeman_eigs is not None and zeeman_eigs[s] is not None and np.max(np.abs(zeeman_eigs[s])) > 0:
            eul = None if zeeman_euler is None else zeeman_euler[s]
            S = np.eye(3) if eul is None else euler_dcm(*eul)
            C = S @ np.diag(zeeman_eigs[s]) @ S.T
            Z = (C + C.T) / 2
        if isotopes[s][0] == 'E':
            zee.append(Z * carrier[s] / FREE_G)
        else:
            zee.append((np.eye(3) + 1e-6 * Z) * carrier[s])
    cpl = {}

    def add(key, M):
        cpl[key] = cpl.get(key, np.zeros((3, 3))) + M

    if coordinates is not None:
        xyz = [None if c is None else np.asarray(c, float) for c in coordinates]
        for a in range(n):
            for b in range(n):
                if a == b or xyz[a] is None or xyz[b] is None:
                    continue
                d = xyz[b] - xyz[a]
                r = float(np.linalg.norm(d))
                if not r < tols['prox_cutoff']:
                    continue
                if r < 0.5:
                    raise ValueError(f'spins {a} and {b} collide')
                u = d / r
                pre = 0.5 * gam[a] * gam[b] * PLANCK_HBAR * VACUUM_MU0 / (4 * math.pi * (r * 1e-10) ** 3)
                D = pre * (np.eye(3) - 3 * np.outer(u, u))
                add((a, b), D - np.eye(3) * np.trace(D) / 3)
    for key, eigs in (coupling_eigs or {}).items():
        if np.linalg.norm(eigs) > tols['inter_cutoff']:
            eul = (coupling_euler or {}).get(key)
            S = np.eye(3) if eul is None else euler_dcm(*eul)
            C = 2 * math.pi * S @ np.diag(eigs) @ S.T
            add(key, (C + C.T) / 2)
    for key, j in (coupling_scalar or {}).items():
        if abs(j) > tols['inter_cutoff']:
            add(key, 2 * math.pi * j * np.eye(3))
    # (a, a): quadratic coupling of spin a (quadrupolar or zero-field splitting)
    cpl = {k: M for k, M in cpl.items() if np.linalg.norm(M, 2) >= 2 * math.pi * tols['inter_cutoff']}
    for (a, b) in cpl:
        if a == b and mult[a] < 3:
            raise ValueError(f'spin {a} has multiplicity {mult[a]}: no quadratic coupling')
    relax = r1 is not None or r2 is not None
    r1 = np.zeros(n) if r1 is None else np.asarray(r1, float)
    r2 = np.zeros(n) if r2 is None else np.asarray(r2, float)
    return SpinSystem(list(isotopes), float(magnet), zee, cpl, r1, r2, relax, tols)


# ---------------------------------------------------------------------------
# Basis
# ---------------------------------------------------------------------------

@dataclass
class Basis:
    """Sorted spherical-tensor Liouville basis: ``codes[i, s]`` is the IST code of
    spin s in state i; state 0 is the unit state."""
    codes: np.ndarray
    radix: np.ndarray
    keys: np.ndarray

    @property
    def dim(self) -> int:
        return self.codes.shape[0]

    def find(self, keys: np.ndarray) -> np.ndarray:
        """Row index of each key, -1 where the state is outside the basis."""
        pos = np.searchsorted(self.keys, keys)
        pos = np.minimum(pos, self.keys.size - 1)
        return np.where(self.keys[pos] == keys, pos, -1)


def _clusters(ss: SpinSystem, approximation: str, level: int, space_level: int) -> list:
    n = ss.nspins
    if approximation == 'none':
        return [tuple(range(n))]
    if approximation == 'IK-0':
        return list(itertools.combinations(range(n), level))
    if approximation == 'IK-1':
        cut = 2 * math.pi * ss.tols['inter_cutoff']
        adj = np.eye(n, dtype=bool)
        for (a, b), M in ss.couplings.items():
            if np.linalg.norm(M, 2) > cut:
                adj[a, b] = adj[b, a] = True
        out = set()
        # connected clusters up to `level` spins grown by adjacency (kernel/utilities/dfpt.m)
        frontier = {(i,) for i in range(n)}
        out |= frontier
        for _ in range(level - 1):
            grown = set()
            for c in frontier:
                nb = np.nonzero(adj[list(c)].any(axis=0))[0]
                nb = [j for j in nb if j not in c]
                if not nb:
                    grown.add(c)
                for j in nb:
                    grown.add(tuple(sorted(c + (int(j),))))
            frontier = grown
            out |= grown
        for i in range(n):        # proximity clusters at space_level 1: single spins
            out.add((i,))
        return sorted(out)
    raise ValueError(f'unsupported basis approximation {approximation!r}')


def decoupled_basis(ss: SpinSystem, basis: Basis, spins) -> Basis:
    """The basis without the states in which a decoupled spin is active
    (kernel/decouple.m zeroes their rows and columns of L and their
    populations, so they never take part; dropping them gives the same
    dynamics on a smaller problem)."""
    if not spins:
        return basis
    if any(s not in ss.isotopes for s in spins):
        raise ValueError('the system does not contain the spins specified')
    dec = np.array([iso in spins for iso in ss.isotopes])
    keep = basis.codes[:, dec].sum(axis=1) == 0
    return Basis(basis.codes[keep], basis.radix, basis.keys[keep])


def build_basis(ss: SpinSystem, approximation: str = 'none', level: int = 0,
                space_level: int = 1, projections=None) -> Basis:
    """Union of all product states over spin clusters (kernel/basis.m:186-465)."""
    d = ss.mults ** 2
    radix = np.ones(ss.nspins, np.int64)
    for s in range(ss.nspins - 2, -1, -1):
        radix[s] = radix[s + 1] * d[s + 1]
    blocks = []
    for cl in _clusters(ss, approximation, level, space_level):
        cl = list(cl)
        grids = np.meshgrid(*[np.arange(d[s]) for s in cl], indexing='ij')
        sub = np.stack([g.ravel() for g in grids], axis=1)
        if projections is not None:
            l = np.floor(np.sqrt(sub)).astype(np.int64)
            msum = (l * l + l - sub).sum(axis=1)
            keep = np.isin(msum, np.atleast_1d(projections)) | (sub.sum(axis=1) == 0)
            sub = sub[keep]
        codes = np.zeros((sub.shape[0], ss.nspins), np.int64)
        codes[:, cl] = sub
        blocks.append(codes)
    codes = np.vstack(blocks)
    keys, first = np.unique(codes @ radix, return_index=True)     # one key per product state
    return Basis(codes[first].astype(np.int16), radix, keys)


# ---------------------------------------------------------------------------
# Superoperators
# ---------------------------------------------------------------------------

class OperatorFactory:
    """Builds product-operator superoperators on a basis (semantics of
    kernel/operators/superop.m, vectorised over basis states)."""

    def __init__(self, ss: SpinSystem, basis: Basis):
        self.ss, self.basis = ss, basis
        self.tables = {int(m): _product_tables(int(m)) for m in np.unique(ss.mults)}
        self.op_cache = {}          # operator products as summed COO matrices

    def comm_coo(self, ops) -> sp.coo_matrix:
        """Commutation superoperator of a product of single-spin operators,
        cached (it depends only on the basis and the spins' multiplicities)."""
        return self.coo(ops, 'comm')

    def coo(self, ops, kind: str) -> sp.coo_matrix:
        """The superoperator of a product of single-spin operators ('comm',
        'left' or 'right'), cached."""
        key = tuple(ops) if kind == 'comm' else (kind,) + tuple(ops)
        if key not in self.op_cache:
            self.op_cache[key] = self.operator(ops, kind).tocoo()
        return self.op_cache[key]

    def product(self, codes: dict, side: str) -> sp.csr_matrix:
        """Left or right multiplication by prod_s T(codes[s]) (normalised basis).

        For the 'leftofcomm'/'rightofcomm' halves, terms whose input or output
        is the unit state on all active spins are dropped (they cancel exactly
        in the commutator, superop.m:139-145)."""
        r, c, v = self.product_coo(codes, side)
        dim = self.basis.dim
        return sp.csr_matrix((v, (r, c)), shape=(dim, dim))

    def product_coo(self, codes: dict, side: str):
        """The same product as (rows, cols, values) triplets."""
        b = self.basis
        dim = b.dim
        if not codes:
            ar = np.arange(dim)
            return ar, ar.copy(), np.ones(dim, complex)
        comm_half = side.endswith('ofcomm')
        which = 0 if side.startswith('left') else 1
        cols = np.arange(dim)
        vals = np.ones(dim)
        out_active_zero = np.ones(dim, bool)
        in_active_zero = np.ones(dim, bool)
        keys = b.keys.copy()
        for s, c in codes.items():
            tab = self.tables[int(self.ss.mults[s])][which][c]      # [m_in, k_out]
            nz = tab != 0
            cnt_m = nz.sum(axis=1)
            kpad = np.argsort(~nz, axis=1, kind='stable')           # nonzero k first, ascending
            m_in = b.codes[cols, s].astype(np.int64)
            cnt = cnt_m[m_in]
            rep = np.repeat(np.arange(cols.size), cnt)
            start = np.cumsum(cnt) - cnt
            within = np.arange(rep.size) - np.repeat(start, cnt)
            mm = m_in[rep]
            k_out = kpad[mm, within]
            cols, vals = cols[rep], vals[rep] * tab[mm, k_out]
            keys = keys[rep] + (k_out - mm) * b.radix[s]
            out_active_zero = out_active_zero[rep] & (k_out == 0)
            in_active_zero = in_active_zero[rep] & (mm == 0)
        if comm_half:
            keep = ~(out_active_zero | in_active_zero)
            cols, vals, keys = cols[keep], vals[keep], keys[keep]
        r = b.find(keys)
        ok = r >= 0
        return r[ok], cols[ok], vals[ok].astype(complex)

    def commutator(self, codes: dict) -> sp.csr_matrix:
        r, c, v = self.commutator_coo(codes)
        dim = self.basis.dim
        return sp.csr_matrix((v, (r, c)), shape=(dim, dim))

    def commutator_coo(self, codes: dict):
        rl, cl, vl = self.product_coo(codes, 'leftofcomm')
        rr, cr, vr = self.product_coo(codes, 'rightofcomm')
        return np.concatenate([rl, rr]), np.concatenate([cl, cr]), np.concatenate([vl, -vr])

    # Human-readable product operators: lists of (op, spin) with op in
    # E, Lz, L+, L-, Lx, Ly and the rank-2 tensors T2,m (kernel/utilities/
    # human2opspec.m conventions; T(l,m) is state code l*l+l-m, coefficient 1).
    _CODE = {'E': ((0, 1.0),), 'Lz': ((2, 1.0),), 'L+': ((1, -math.sqrt(2)),),
             'L-': ((3, math.sqrt(2)),),
             'Lx': ((1, -math.sqrt(2) / 2), (3, math.sqrt(2) / 2)),
             'Ly': ((1, -math.sqrt(2) / 2j), (3, -math.sqrt(2) / 2j)),
             'T2,+2': ((4, 1.0),), 'T2,+1': ((5, 1.0),), 'T2,0': ((6, 1.0),), 'T2,-1': ((7, 1.0),),
             'T2,-2': ((8, 1.0),)}

    def operator(self, ops, kind: str = 'comm') -> sp.csr_matrix:
        r, c, v = self.operator_coo(ops, kind)
        dim = self.basis.dim
        M = sp.csr_matrix((v, (r, c)), shape=(dim, dim))
        M.sum_duplicates()
        return M

    def operator_coo(self, ops, kind: str = 'comm'):
        """Superoperator of a product of single-spin operators as (rows, cols,
        values) triplets; duplicates are summed when a matrix is formed."""
        terms = [({}, 1.0 + 0j)]
        for op, s in ops:
            new = []
            for codes, c in terms:
                for code, f in self._CODE[op]:
                    cc = dict(codes)
                    if code:
                        cc[s] = code
                    new.append((cc, c * f))
            terms = new
        rs, cs, vs = [], [], []
        for codes, c in terms:
            r, col, v = self.commutator_coo(codes) if kind == 'comm' else self.product_coo(codes, kind)
            rs.append(r)
            cs.append(col)
            vs.append(c * v)
        return np.concatenate(rs), np.concatenate(cs), np.concatenate(vs)

    def state(self, op: str, isotope: str) -> np.ndarray:
        """Liouville-space vector of sum_s op(s) over spins of an isotope
        (kernel/state.m 'exact': left-multiplication applied to the unit state)."""
        unit = np.zeros(self.basis.dim, complex)
        unit[0] = 1.0
        v = np.zeros(self.basis.dim, complex)
        spins = [s for s, i in enumerate(self.ss.isotopes) if i == isotope]
        if not spins:
            raise ValueError(f'no {isotope} spins in the system')
        for s in spins:
            v = v + self.operator([(op, s)], 'left') @ unit
        return v


# ---------------------------------------------------------------------------
# Hamiltonian in rotational-basis form
# ---------------------------------------------------------------------------

_R23 = math.sqrt(2 / 3)
_R18 = math.sqrt(1 / 8)

# Spin-operator parts of rank-1/rank-2 coupling tensors, per strength
# (kernel/hamiltonian.m:384-580): (opL, opS, rank-1 weights [+1,0,-1], rank-2 weights [+2..-2]).
_BILINEAR = {
    'zz': ('Lz', 'Lz', (0, 0, 0), (0, 0, _R23, 0, 0)),
    '+-': ('L+', 'L-', (0, -_R18, 0), (0, 0, -_R23 / 4, 0, 0)),
    '-+': ('L-', 'L+', (0, _R18, 0), (0, 0, -_R23 / 4, 0, 0)),
    'z+': ('Lz', 'L+', (0.5, 0, 0), (0, -0.5, 0, 0, 0)),
    '+z': ('L+', 'Lz', (-0.5, 0, 0), (0, -0.5, 0, 0, 0)),
    'z-': ('Lz', 'L-', (0, 0, 0.5), (0, 0, 0, 0.5, 0)),
    '-z': ('L-', 'Lz', (0, 0, -0.5), (0, 0, 0, 0.5, 0)),
    '++': ('L+', 'L+', (0, 0, 0), (0.5, 0, 0, 0, 0)),
    '--': ('L-', 'L-', (0, 0, 0), (0, 0, 0, 0, 0.5)),
}
_STRENGTH_TERMS = {
    'strong': ('zz', '+-', '-+', 'z+', '+z', 'z-', '-z', '++', '--'),
    'secular': ('zz', '+-', '-+'), 'zz': ('zz',), 'z*': ('zz', 'z+', 'z-'),
    '*z': ('zz', '+z', '-z'), 'ignore': (),
}


def interaction_strengths(ss: SpinSystem, assumptions: str):
    """Per-spin Zeeman and per-pair coupling strengths (kernel/assume.m:89-200)."""
    ele = [i[0] == 'E' for i in ss.isotopes]
    if assumptions == 'nmr':
        zs = ['secular'] * ss.nspins
        cs = {(a, b): ('secular' if ss.isotopes[a] == ss.isotopes[b] else 'zz') for (a, b) in ss.couplings}
    elif assumptions == 'esr':
        zs = ['secular' if e else 'full' for e in ele]
        cs = {}
        for (a, b) in ss.couplings:
            if ele[a] and not ele[b]:
                cs[(a, b)] = 'z*'
            elif ele[b] and not ele[a]:
                cs[(a, b)] = '*z'
            elif ele[a] and ele[b]:
                cs[(a, b)] = 'secular'
            else:
                cs[(a, b)] = 'strong'
    elif assumptions == 'labframe':
        zs = ['full'] * ss.nspins
        cs = {(a, b): 'strong' for (a, b) in ss.couplings}
    else:
        raise ValueError("assumptions must be 'nmr', 'esr' or 'labframe'")
    return zs, cs


_FACTORIES: dict = {}
_FACTORY_LIMIT = 8


def factory_for(ss: SpinSystem, basis: Basis) -> OperatorFactory:
    """An operator factory shared by systems with the same isotopes and
    basis (operator matrices and states depend on nothing else), least
    recently used first out after a few bases."""
    key = (tuple(ss.isotopes), tuple(int(m) for m in ss.mults), basis.dim, basis.keys.tobytes())
    f = _FACTORIES.pop(key, None)
    if f is None:
        f = OperatorFactory(ss, basis)
        if len(_FACTORIES) >= _FACTORY_LIMIT:
            _FACTORIES.pop(next(iter(_FACTORIES)))
    _FACTORIES[key] = f
    return f


@dataclass
class RotationalHamiltonian:
    """``H(Omega) = I + sum_{r,k,m} D^r_{km}(Omega) Q[(r,k,m)]`` before Hermitisation."""
    dim: int
    iso: sp.csr_matrix
    aniso: dict                       # (r, k, m) with 0-based k, m -> csr


def interaction_terms(ss: SpinSystem, assumptions: str):
    """The operator content of the Hamiltonian (kernel/hamiltonian.m:59-790):
    isotropic terms ``(coefficient, ops)`` and anisotropic terms ``(ist
    weights (8,), irreducible components (8,), ops)``, ``ops`` a list of
    ``(operator, spin)``."""
    tz = ss.tols['liouv_zero']
    zs, cs = interaction_strengths(ss, assumptions)
    iso_terms = []       # (coefficient, ops)
    ani_terms = []       # (ist weights (8,), irreducible components (8,), ops)
    for s in range(ss.nspins):
        i0, r1, r2 = sph_components(ss.zeeman[s])
        if zs[s] == 'secular':
            i0 = i0 - ss.carriers[s]
        if abs(i0) > tz:
            iso_terms.append((i0, [('Lz', s)]))
        if np.linalg.norm(r1) > tz or np.linalg.norm(r2) > tz:
            irr = np.concatenate([r1, r2])
            if zs[s] == 'full':
                ani_terms.append((np.array([-0.5, 0, 0, 0, -0.5, 0, 0, 0]), irr, [('L+', s)]))
                ani_terms.append((np.array([0, 0, 0, 0, 0, _R23, 0, 0]), irr, [('Lz', s)]))
                ani_terms.append((np.array([0, 0, -0.5, 0, 0, 0, 0.5, 0]), irr, [('L-', s)]))
            else:
                ani_terms.append((np.array([0, 0, 0, 0, 0, _R23, 0, 0]), irr, [('Lz', s)]))
    cut = 2 * math.pi * ss.tols['inter_cutoff']
    for (a, b), M in ss.couplings.items():
        strength = cs[(a, b)]
        j, r1, r2 = sph_components(M)
        if a == b:
            # quadratic coupling (hamiltonian.m:191-257): traceless symmetric,
            # rank-2 operators of the spin itself
            if abs(j) > 1e-6 * np.linalg.norm(r2) or np.linalg.norm(r1) > 1e-6 * np.linalg.norm(r2):
                raise ValueError('quadratic couplings must be traceless and symmetric')
            irr = np.concatenate([np.zeros(3, complex), r2])
            ops = (['T2,+2', 'T2,+1', 'T2,0', 'T2,-1', 'T2,-2'] if strength == 'strong' else ['T2,0'])
            for op in ops:
                ist = np.zeros(8)
                ist[3 + 2 - int(op[3:])] = 1.0
                ani_terms.append((ist, irr, [(op, a)]))
            continue
        if abs(j) > cut:
            if strength in ('strong', 'secular'):
                iso_terms += [(j, [('Lz', a), ('Lz', b)]), (j / 2, [('L+', a), ('L-', b)]),
                              (j / 2, [('L-', a), ('L+', b)])]
            elif strength in ('zz', 'z*', '*z'):
                iso_terms.append((j, [('Lz', a), ('Lz', b)]))
        if np.linalg.norm(r1) > tz or np.linalg.norm(r2) > tz:
            irr = np.concatenate([r1, r2])
            for name in _STRENGTH_TERMS[strength]:
                opL, opS, w1, w2 = _BILINEAR[name]
                ani_terms.append((np.array(w1 + w2, float), irr, [(opL, a), (opS, b)]))
    return iso_terms, ani_terms


def _term_groups(ss: SpinSystem, assumptions: str):
    """[(key, [(coefficient, ops), ...])]: the isotropic part (key None) and
    every rotational component (r, k, m) with at least one coefficient above
    liouv_zero."""
    tz = ss.tols['liouv_zero']
    iso_terms, ani_terms = interaction_terms(ss, assumptions)
    groups = [(None, iso_terms)]
    for r in (1, 2):
        off = r * r - 1
        for k in range(2 * r + 1):
            for m in range(2 * r + 1):
                weighted = []
                for ist, irr, ops in ani_terms:
                    c = ist[off + k] * irr[off + m]
                    if abs(c) > tz:
                        weighted.append((c, ops))
                if weighted:
                    groups.append(((r, k, m), weighted))
    return groups


@dataclass
class HamiltonianMonomials:
    """Input of the on-GPU construction: the basis as mixed-radix keys and
    the Hamiltonian as single-code monomials coef * [T(code_a) T(code_b), .]."""
    mults: np.ndarray                 # (nspins,) int32
    keys: np.ndarray                  # (dim,) int64, ascending
    radix: np.ndarray                 # (nspins,) int64
    terms: list                       # [(r, k, m)], term t+1 of the monomials
    mono_term: np.ndarray             # (n,) int32, 0 = isotropic part
    mono_spins: np.ndarray            # (n, 2) int32, -1 = none
    mono_codes: np.ndarray            # (n, 2) int32
    mono_coefs: np.ndarray            # (n,) complex128


def hamiltonian_monomials(ss: SpinSystem, basis: Basis, assumptions: str) -> HamiltonianMonomials:
    """The same Hamiltonian as ``rotational_hamiltonian`` as monomials: each
    human-readable operator product is expanded into products of single
    irreducible spherical tensor codes (``OperatorFactory._CODE``)."""
    groups = _term_groups(ss, assumptions)
    terms, mt, msp, mco, mcf = [], [], [], [], []
    for t, (key, weighted) in enumerate(groups):
        if key is not None:
            terms.append(key)
        for c, ops in weighted:
            for combo in itertools.product(*[OperatorFactory._CODE[op] for op, _ in ops]):
                f = 1.0 + 0j
                sp_, co_ = [-1, -1], [0, 0]
                for slot, ((op, spin), (code, fac)) in enumerate(zip(ops, combo)):
                    f *= fac
                    if code:
                        sp_[slot], co_[slot] = spin, code
                mt.append(t)
                msp.append(sp_)
                mco.append(co_)
                mcf.append(c * f)
    return HamiltonianMonomials(np.asarray(ss.mults, np.int32), np.ascontiguousarray(basis.keys, np.int64),
                                np.ascontiguousarray(basis.radix, np.int64), terms,
                                np.asarray(mt, np.int32), np.asarray(msp, np.int32).reshape(-1, 2),
                                np.asarray(mco, np.int32).reshape(-1, 2), np.asarray(mcf, np.complex128))


def rotational_hamiltonian(ss: SpinSystem, basis: Basis, assumptions: str,
                           factory: OperatorFactory | None = None, kind: str = 'comm') -> RotationalHamiltonian:
    """Isotropic part and rotational basis (kernel/hamiltonian.m:59-790);
    kind 'left' gives left-side product superoperators (hamiltonian.m's
    'left' argument, for thermal equilibria)."""
    f = factory or OperatorFactory(ss, basis)
    groups = _term_groups(ss, assumptions)
    op = lambda ops: f.coo(ops, kind)        # one superoperator per distinct operator product

    dim = basis.dim

    def assemble(weighted):
        # sum_i c_i M_i in one pass: concatenate the scaled triplets, then
        # sum duplicates once
        if not weighted:
            return None
        rows = np.concatenate([op(ops).row for _, ops in weighted])
        cols = np.concatenate([op(ops).col for _, ops in weighted])
        vals = np.concatenate([c * op(ops).data for c, ops in weighted])
        M = sp.csr_matrix((vals, (rows, cols)), shape=(dim, dim))
        M.sum_duplicates()
        M.eliminate_zeros()
        return M

    I = assemble(groups[0][1])
    if I is None:
        I = sp.csr_matrix((dim, dim), dtype=complex)
    aniso = {}
    for key, weighted in groups[1:]:
        acc = assemble(weighted)
        if acc is not None and acc.nnz:
            aniso[key] = acc
    return RotationalHamiltonian(dim, I, aniso)


HBAR = 6.62607015e-34 / (2 * math.pi)      # J s (kernel/utilities/tolerances.m:348)
KBOL = 1.380649e-23                        # J/K (kernel/utilities/tolerances.m:351)


def _wigner_all(terms, alphas, betas, gammas) -> np.ndarray:
    """D^r_{km}(alpha_o, beta_o, gamma_o) for every term (r, k, m) and
    orientation o, (n_terms, n_orient) complex."""
    from .singlerot import wigner_d
    out = np.zeros((len(terms), len(alphas)), complex)
    for o, (a, b, g) in enumerate(zip(alphas, betas, gammas)):
        cache = {}
        for t, (r, k, m) in enumerate(terms):
            if r not in cache:
                cache[r] = wigner_d(r, a, b, g)
            out[t, o] = cache[r][k, m]
    return out


def equilibrium_states(H: RotationalHamiltonian, temperature: float, alphas=None, betas=None, gammas=None):
    """Thermal equilibrium exp(-beta H(Omega)) unit / <unit|...> for every
    orientation (kernel/states/equilibrium.m, sphten-liouv; H made of
    left-side product superoperators of the lab-frame Hamiltonian,
    H(Omega) = I + herm(sum D Q) as orientation.m builds it; beta = hbar/kT).
    Without angles: the isotropic state exp(-beta I) unit.  Taylor series in
    substeps of at most 2 in the 1-norm, stopped below the FP64 epsilon, as
    kernel/step.m does.  Returns (n_orient, dim), or (dim,) without angles."""
    if not temperature:
        raise ValueError('temperature must be specified (and non-zero)')
    beta = HBAR / (KBOL * float(temperature))
    dim = H.dim
    keys = sorted(H.aniso) if alphas is not None else []
    Qs = [sp.csr_matrix(H.aniso[k]) for k in keys]
    QHs = [Q.conj().T.tocsr() for Q in Qs]
    I = sp.csr_matrix(H.iso)
    n_or = 1 if alphas is None else len(alphas)
    D = _wigner_all(keys, alphas, betas, gammas) if keys else np.zeros((0, n_or), complex)
    norm1 = abs(I).sum(axis=0).max() + sum(abs(Q).sum(axis=0).max() for Q in Qs)
    nsub = max(1, int(math.ceil(float(norm1) * beta / 2)))
    h = beta / nsub

    def apply(V):
        out = I @ V
        for t in range(len(keys)):
            out = out + 0.5 * ((Qs[t] @ V) * D[t][None, :] + (QHs[t] @ V) * np.conj(D[t])[None, :])
        return out

    rho = np.zeros((dim, n_or), complex)
    rho[0] = 1.0
    for _ in range(nsub):
        term = rho.copy()
        k = 1
        while True:
            term = (-h / k) * apply(term)
            rho = rho + term
            k += 1
            if np.abs(term).max() <= np.finfo(float).eps * np.abs(rho).max() or k > 200:
                break
    rho = rho / rho[0][None, :]
    return rho[:, 0] if alphas is None else rho.T.copy()


def relaxation_diagonal(ss: SpinSystem, basis: Basis, damp_rate: float = 0.0) -> np.ndarray:
    """Diagonal of the T1/T2 relaxation superoperator (kernel/utilities/rlx_t1_t2.m:145-176):
    each state decays at the sum of R1 over its longitudinal spins and R2 over its
    transverse spins; with ``damp_rate`` (kernel/relaxation.m:638-684, 'damp',
    isotropic) every state but the unit state also decays at that rate.
    Returned with the reference's sign (non-positive)."""
    c = basis.codes.astype(np.int64)
    out = np.zeros(basis.dim)
    if ss.relaxation:
        l = np.floor(np.sqrt(c)).astype(np.int64)
        m = l * l + l - c
        active = l != 0
        longi = active & (m == 0)
        trans = active & (m != 0)
        out = -(longi @ ss.r1 + trans @ ss.r2)
    if damp_rate:
        out = out - float(damp_rate) * (c != 0).any(axis=1)
    return out
