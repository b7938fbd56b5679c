"""FP64 restatement of Spinach's static powder-FID path (test infrastructure).

TEST INFRASTRUCTURE ONLY -- the oracle.  See ``oracle/__init__.py`` for who may
import it.  Every function names the reference file and lines it restates
(paths relative to the Spinach source tree).  The restatement is deliberately
literal: loops and masks follow the reference's own order of operations so
that FP64 results can be compared at 1e-10 relative.

Conventions kept from the reference:
  * spin indices inside ``SpinSystem`` are 0-based (MATLAB is 1-based);
  * the spherical-tensor Liouville basis is the sorted list of per-spin state
    codes ``l*l+l-m`` (kernel/indexing/lm2lin.m) with the unit state first;
  * a sparse superoperator has row = output state, column = input state.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

EPS = np.finfo(np.float64).eps

# Fundamental constants, kernel/utilities/tolerances.m:348-360.
HBAR = 6.62607015e-34 / (2 * np.pi)
MU0 = 1.25663706127e-6
FREEG = 2.00231930436092

# Multiplicities and gyromagnetic ratios (rad/s/T), kernel/spin.m:86-131.
ISOTOPES = {
    'E': (2, -1.76085963023e11),
    '1H': (2, 2.6752218744e8),
    '2H': (3, 4.10662791e7),
    '13C': (2, 6.728284e7),
    '14N': (3, 1.9337792e7),
    '15N': (2, -2.71261804e7),
}


def tolerances(mode: str = 'default') -> dict:
    """kernel/utilities/tolerances.m:36-290 ('safe default' and 'paranoia' branches)."""
    if mode == 'paranoia':
        return dict(inter_cutoff=EPS, liouv_zero=EPS, prop_chop=EPS, zte_tol=np.nan,
                    prox_cutoff=np.inf, krylov_tol=10000, dense_matrix=0.15, small_matrix=200)
    if mode != 'default':
        raise ValueError('tolerance mode must be default or paranoia')
    return dict(inter_cutoff=1e-10, liouv_zero=1e-10, prop_chop=1e-10, zte_tol=1e-24,
                prox_cutoff=100.0, krylov_tol=10000, dense_matrix=0.15, small_matrix=200)


# --------------------------------------------------------------------------
# Angular momentum helpers
# --------------------------------------------------------------------------

def pauli(mult: int) -> dict:
    """kernel/utilities/pauli.m: spin operators for a multiplicity (Lz descending)."""
    s = (mult - 1) / 2
    prjs = np.arange(mult - 1, -1, -1) - s
    p = np.zeros((mult, mult), complex)
    m = np.zeros((mult, mult), complex)
    for i in range(mult - 1):
        p[i, i + 1] = math.sqrt(s * (s + 1) - prjs[i + 1] * (prjs[i + 1] + 1))
        m[i + 1, i] = math.sqrt(s * (s + 1) - prjs[i] * (prjs[i] - 1))
    z = np.diag(prjs).astype(complex)
    return dict(p=p, m=m, z=z, u=np.eye(mult, dtype=complex), x=(p + m) / 2, y=(p - m) / 2j)


def irr_sph_ten(mult: int, k: int | None = None) -> list:
    """kernel/operators/irr_sph_ten.m:35-87 (unnormalised single-spin ISTs)."""
    if k is None:
        out = []
        for n in range(mult):
            out.extend(irr_sph_ten(mult, n))
        return out
    if k == 0:
        return [np.eye(mult, dtype=complex)]
    L = pauli(mult)
    T = [((-1) ** k) * (2 ** (-k / 2)) * np.linalg.matrix_power(L['p'], k)]
    for n in range(2, 2 * k + 2):
        q = k - n + 2
        prev = T[-1]
        T.append((1 / math.sqrt((k + q) * (k - q + 1))) * (L['m'] @ prev - prev @ L['m']))
    return T


def lm2lin(l, m):
    """kernel/indexing/lm2lin.m."""
    return l * l + l - m


def lin2lm(i):
    """kernel/indexing/lin2lm.m."""
    i = np.asarray(i)
    l = np.floor(np.sqrt(i)).astype(np.int64)
    return l, l * l + l - i


def hdot(a, b):
    """kernel/utilities/hdot.m: sum(conj(A).*B)."""
    return np.sum(np.conj(a) * b)


def ist_product_table(mult: int):
    """kernel/cache/ist_product_table.m:94-118, computed (never loaded).

    Returns (left, right) with left[n, m, k] = <e_k | T_n e_m> in the
    normalised IST basis e = T/|T| (right: <e_k | e_m T_n>).
    """
    T = irr_sph_ten(mult)
    d = mult * mult
    norms = np.array([math.sqrt(hdot(t, t).real) for t in T])
    left = np.zeros((d, d, d))
    right = np.zeros((d, d, d))
    for k in range(d):
        for m in range(d):
            for n in range(d):
                left[n, m, k] = (norms[n] * hdot(T[k] / norms[k], (T[n] / norms[n]) @ (T[m] / norms[m]))).real
                right[n, m, k] = (norms[n] * hdot(T[k] / norms[k], (T[m] / norms[m]) @ (T[n] / norms[n]))).real
    return left, right


def wigner(l: int, alp: float, bet: float, gam: float) -> np.ndarray:
    """kernel/utilities/wigner.m:39-87 (rows/cols in descending projection)."""
    if l == 1:
        egp1 = np.exp(-1j * gam); egm1 = np.exp(1j * gam)
        eap1 = np.exp(-1j * alp); eam1 = np.exp(1j * alp)
        sb = math.sin(bet); cb = math.cos(bet)
        return np.array([
            [eap1 * egp1 * (1 / 2 + cb / 2), -eap1 * sb / math.sqrt(2), eap1 * egm1 * (1 / 2 - cb / 2)],
            [egp1 * sb / math.sqrt(2), cb, -egm1 * sb / math.sqrt(2)],
            [eam1 * egp1 * (1 / 2 - cb / 2), eam1 * sb / math.sqrt(2), eam1 * egm1 * (1 / 2 + cb / 2)]])
    if l == 2:
        egp2 = np.exp(-2j * gam); egp1 = np.exp(-1j * gam)
        egm1 = np.exp(1j * gam); egm2 = np.exp(2j * gam)
        eap2 = np.exp(-2j * alp); eap1 = np.exp(-1j * alp)
        eam1 = np.exp(1j * alp); eam2 = np.exp(2j * alp)
        sb = math.sin(bet); cb = math.cos(bet)
        cbh4 = math.cos(bet / 2) ** 4; sbh4 = math.sin(bet / 2) ** 4
        s38 = math.sqrt(3 / 8); s32 = math.sqrt(3 / 2)
        return np.array([
            [eap2 * cbh4 * egp2, eap2 * (-sb * (1 + cb) / 2) * egp1, eap2 * s38 * sb ** 2,
             eap2 * (-sb * (1 - cb) / 2) * egm1, eap2 * sbh4 * egm2],
            [eap1 * (sb * (cb + 1) / 2) * egp2, eap1 * (2 * cb - 1) * (1 + cb) / 2 * egp1,
             eap1 * (-s32 * sb * cb), eap1 * (2 * cb + 1) * (1 - cb) / 2 * egm1, eap1 * (sb * (cb - 1) / 2) * egm2],
            [s38 * sb ** 2 * egp2, s32 * sb * cb * egp1, (3 * cb ** 2 - 1) / 2,
             -s32 * sb * cb * egm1, s38 * sb ** 2 * egm2],
            [-eam1 * (sb * (cb - 1) / 2) * egp2, eam1 * (2 * cb + 1) * (1 - cb) / 2 * egp1,
             eam1 * (s32 * sb * cb), eam1 * (2 * cb - 1) * (1 + cb) / 2 * egm1, eam1 * (-sb * (cb + 1) / 2) * egm2],
            [eam2 * sbh4 * egp2, eam2 * sb * (1 - cb) / 2 * egp1, eam2 * s38 * sb ** 2,
             eam2 * sb * (1 + cb) / 2 * egm1, eam2 * cbh4 * egm2]])
    L = pauli(2 * l + 1)
    return sla.expm(-1j * L['z'] * alp) @ sla.expm(-1j * L['y'] * bet) @ sla.expm(-1j * L['z'] * gam)


def euler2dcm(alp: float, bet: float, gam: float) -> np.ndarray:
    """kernel/conventions/transforms/euler2dcm.m (ZYZ, active)."""
    ca, sa = math.cos(alp), math.sin(alp)
    cb, sb = math.cos(bet), math.sin(bet)
    cg, sg = math.cos(gam), math.sin(gam)
    Ra = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
    Rb = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    Rg = np.array([[cg, -sg, 0], [sg, cg, 0], [0, 0, 1]])
    return Ra @ Rb @ Rg


def mat2sphten(M: np.ndarray):
    """kernel/conventions/transforms/mat2sphten.m:41-67 -> (rank0, rank1[3], rank2[5])."""
    M = np.zeros((3, 3)) if M is None else np.asarray(M, float)
    r1 = np.zeros(3, complex)
    r2 = np.zeros(5, complex)
    r0 = np.trace(M) / 3
    r1[0] = -(1 / 2) * (M[2, 0] - M[0, 2] - 1j * (M[2, 1] - M[1, 2]))
    r1[1] = +(1j / math.sqrt(2)) * (M[0, 1] - M[1, 0])
    r1[2] = -(1 / 2) * (M[2, 0] - M[0, 2] + 1j * (M[2, 1] - M[1, 2]))
    r2[0] = +(1 / 2) * (M[0, 0] - M[1, 1] - 1j * (M[0, 1] + M[1, 0]))
    r2[1] = -(1 / 2) * (M[0, 2] + M[2, 0] - 1j * (M[1, 2] + M[2, 1]))
    r2[2] = +(1 / math.sqrt(6)) * (2 * M[2, 2] - M[0, 0] - M[1, 1])
    r2[3] = +(1 / 2) * (M[0, 2] + M[2, 0] + 1j * (M[1, 2] + M[2, 1]))
    r2[4] = +(1 / 2) * (M[0, 0] - M[1, 1] + 1j * (M[0, 1] + M[1, 0]))
    return r0, r1, r2


# --------------------------------------------------------------------------
# Spin system: create / dipolar / assume / basis
# --------------------------------------------------------------------------

@dataclass
class SpinSystem:
    isotopes: list
    magnet: float
    tols: dict
    mults: np.ndarray = None
    gammas: np.ndarray = None
    basefrqs: np.ndarray = None
    zeeman: list = None            # 3x3 rad/s per spin
    coupling: dict = field(default_factory=dict)   # (n,k) -> 3x3 rad/s
    coordinates: list = None
    r1: list = None
    r2: list = None
    theories: list = field(default_factory=list)
    zeeman_strength: list = None
    coupling_strength: dict = None
    basis: np.ndarray = None
    lpst: dict = None
    rpst: dict = None
    enable: list = field(default_factory=list)

    @property
    def nspins(self):
        return len(self.isotopes)


def create(sys: dict, inter: dict, tol_mode: str = 'default') -> SpinSystem:
    """kernel/create.m:459-466 (carriers), :742-814 (Zeeman), :954-1046 (couplings),
    :1254-1373 (T1/T2 rates).  Units: Zeeman eigs in ppm (nuclei) or g (electrons),
    coupling eigs/scalars in Hz, coordinates in Angstrom, rates in 1/s."""
    iso = list(sys['isotopes'])
    ss = SpinSystem(isotopes=iso, magnet=float(sys['magnet']), tols=tolerances(tol_mode))
    ss.enable = list(sys.get('enable', []))
    n = len(iso)
    ss.mults = np.array([ISOTOPES[i][0] for i in iso])
    ss.gammas = np.array([ISOTOPES[i][1] for i in iso])
    ss.basefrqs = -ss.gammas * ss.magnet
    zin = inter.get('zeeman', None)
    zee = [np.zeros((3, 3)) for _ in range(n)]
    if zin is not None:
        if 'eigs' in zin:
            for k in range(n):
                eigs = zin['eigs'][k]
                if eigs is not None and np.max(np.abs(eigs)) > 0:
                    eul = zin.get('euler', [None] * n)[k]
                    S = np.eye(3) if eul is None else euler2dcm(*eul)
                    comp = S @ np.diag(eigs) @ S.T
                    zee[k] = zee[k] + (comp + comp.T) / 2
        if 'scalar' in zin:
            for k in range(n):
                if zin['scalar'][k] is not None and abs(zin['scalar'][k]) > 0:
                    zee[k] = zee[k] + np.eye(3) * zin['scalar'][k]
        for k in range(n):
            if iso[k][0] == 'E':
                zee[k] = zee[k] * ss.basefrqs[k] / FREEG
            else:
                zee[k] = (np.eye(3) + 1e-6 * zee[k]) * ss.basefrqs[k]
    else:
        zee = [np.eye(3) * ss.basefrqs[k] for k in range(n)]
    ss.zeeman = zee
    cpl = {(a, b): np.zeros((3, 3)) for a in range(n) for b in range(n)}
    ss.coordinates = inter.get('coordinates', None)
    if ss.coordinates is not None:
        _dipolar(ss, cpl)
    cin = inter.get('coupling', None)
    if cin is not None:
        cutoff = ss.tols['inter_cutoff']
        if 'eigs' in cin:
            for (a, b), eigs in sorted(cin['eigs'].items(), key=lambda kv: (kv[0][1], kv[0][0])):
                if np.linalg.norm(eigs) > cutoff:
                    eul = cin.get('euler', {}).get((a, b), None)
                    S = np.eye(3) if eul is None else euler2dcm(*eul)
                    comp = 2 * np.pi * S @ np.diag(eigs) @ S.T
                    cpl[(a, b)] = cpl[(a, b)] + (comp + comp.T) / 2
        if 'scalar' in cin:
            for (a, b), j in sorted(cin['scalar'].items(), key=lambda kv: (kv[0][1], kv[0][0])):
                if abs(j) > cutoff:
                    cpl[(a, b)] = cpl[(a, b)] + 2 * np.pi * np.eye(3) * j
    ss.coupling = {}
    for key, M in cpl.items():
        if np.linalg.norm(M, 2) >= 2 * np.pi * ss.tols['inter_cutoff']:
            ss.coupling[key] = M
    ss.temperature = inter.get('temperature', None)
    rl = inter.get('relaxation', [])
    ss.theories = list(rl)
    ss.r1 = list(inter.get('r1_rates', [0.0] * n))
    ss.damp_rate = inter.get('damp_rate', 0.0)
    ss.r2 = list(inter.get('r2_rates', [0.0] * n))
    return ss


def _dipolar(ss: SpinSystem, cpl: dict):
    """kernel/utilities/dipolar.m:30-185 (no PBC, one chemical species)."""
    n = ss.nspins
    for a in range(n):
        for b in range(n):
            ca, cb = ss.coordinates[a], ss.coordinates[b]
            if ca is None or cb is None or a == b:
                continue
            dv = np.asarray(cb, float) - np.asarray(ca, float)
            dist = np.linalg.norm(dv)
            if not dist < ss.tols['prox_cutoff']:
                continue
            if dist < 0.5:
                raise ValueError(f'collision detected between spin {a} and spin {b}')
            ort = dv / dist
            A = 0.5 * ss.gammas[a] * ss.gammas[b] * HBAR * MU0 / (4 * np.pi * (dist * 1e-10) ** 3)
            D = A * (np.eye(3) - 3 * np.outer(ort, ort))
            D = D - np.eye(3) * np.trace(D) / 3
            cpl[(a, b)] = cpl[(a, b)] + D


def assume(ss: SpinSystem, assumptions: str) -> SpinSystem:
    """kernel/assume.m:89-136 ('nmr') and :138-200 ('esr')."""
    n = ss.nspins
    zs, cs = [None] * n, {}
    ele = [i[0] == 'E' for i in ss.isotopes]
    if assumptions == 'nmr':
        zs = ['secular'] * n
        for a in range(n):
            for b in range(n):
                cs[(a, b)] = 'secular' if ss.isotopes[a] == ss.isotopes[b] else 'zz'
    elif assumptions == 'esr':
        zs = ['secular' if e else 'full' for e in ele]
        for a in range(n):
            for b in range(n):
                if ele[a] and not ele[b]:
                    cs[(a, b)] = 'z*'
                elif ele[b] and not ele[a]:
                    cs[(a, b)] = '*z'
                elif ele[a] and ele[b]:
                    cs[(a, b)] = 'secular'
                else:
                    cs[(a, b)] = 'strong'
    elif assumptions == 'labframe':
        # kernel/assume.m:278-300: everything in full
        zs = ['full'] * n
        for a in range(n):
            for b in range(n):
                cs[(a, b)] = 'strong'
    else:
        raise ValueError('only nmr, esr and labframe assumptions are restated')
    ss.zeeman_strength, ss.coupling_strength = zs, cs
    return ss


def _dfpt(conmatrix: np.ndarray, max_size: int) -> np.ndarray:
    """kernel/utilities/dfpt.m: connected subgraphs up to max_size spins."""
    n = conmatrix.shape[0]
    subgraphs = [(i,) for i in range(n)]
    for _ in range(2, max_size + 1):
        grown = set()
        for sg in subgraphs:
            nb = np.any(conmatrix[:, list(sg)], axis=1)
            nb[list(sg)] = False
            idx = np.nonzero(nb)[0]
            if idx.size == 0:
                grown.add(tuple(sorted(sg + (sg[-1],))))
            else:
                for j in idx:
                    grown.add(tuple(sorted(sg + (int(j),))))
        subgraphs = sorted(grown)
    out = np.zeros((len(subgraphs), n), bool)
    for r, sg in enumerate(subgraphs):
        out[r, list(sg)] = True
    return out


def basis(ss: SpinSystem, bas: dict) -> SpinSystem:
    """kernel/basis.m:155-183 (state lists), :186-269 (subgraphs for none/IK-0/IK-1),
    :314-430 (per-subgraph descriptors, projections filter), :436-465 (dedupe,
    sortrows) and :553-563 (product tables)."""
    if bas.get('formalism', 'sphten-liouv') != 'sphten-liouv':
        raise ValueError('only sphten-liouv is restated')
    n = ss.nspins
    approx = bas.get('approximation', 'none')
    if approx == 'none':
        subgraphs = np.ones((1, n), bool)
    elif approx == 'IK-0':
        combos = list(itertools.combinations(range(n), bas['level']))
        subgraphs = np.zeros((len(combos), n), bool)
        for r, c in enumerate(combos):
            subgraphs[r, list(c)] = True
    elif approx == 'IK-1':
        cutoff = 2 * np.pi * ss.tols['inter_cutoff']
        con = np.zeros((n, n), bool)
        for (a, b), M in ss.coupling.items():
            if np.linalg.norm(M, 2) > cutoff:
                con[a, b] = True
        con = con | np.eye(n, dtype=bool)
        con = con | con.T
        prox = np.eye(n, dtype=bool)
        if ss.coordinates is not None:
            for a in range(n):
                for b in range(n):
                    if a != b and ss.coordinates[a] is not None and ss.coordinates[b] is not None:
                        d = np.linalg.norm(np.subtract(ss.coordinates[b], ss.coordinates[a]))
                        prox[a, b] = d < ss.tols['prox_cutoff']
        prox = prox | prox.T
        subgraphs = np.vstack([_dfpt(con, bas['level']), _dfpt(prox, bas.get('space_level', 1))])
    else:
        raise ValueError('unsupported approximation')
    subgraphs = np.unique(subgraphs, axis=0)
    rows = []
    for sg in subgraphs:
        spins = np.nonzero(sg)[0]
        lists = [range(ss.mults[s] ** 2) for s in spins]
        local = np.zeros((int(np.prod([ss.mults[s] ** 2 for s in spins])), n), np.int64)
        for r, combo in enumerate(itertools.product(*lists)):
            local[r, spins] = combo
        if 'projections' in bas:
            _, M = lin2lm(local)
            mask = np.zeros(local.shape[0], bool)
            mask[0] = True
            pn = M.sum(axis=1)
            for k in np.atleast_1d(bas['projections']):
                mask |= pn == k
            local = local[mask]
        rows.append(local)
    allrows = np.unique(np.vstack(rows), axis=0)   # unique(...,'rows') + sortrows
    ss.basis = allrows
    ss.lpst, ss.rpst = {}, {}
    for m in np.unique(ss.mults):
        ss.lpst[int(m)], ss.rpst[int(m)] = ist_product_table(int(m))
    return ss


# --------------------------------------------------------------------------
# Operators and states
# --------------------------------------------------------------------------

def superop(ss: SpinSystem, opspec: np.ndarray, side: str) -> np.ndarray:
    """kernel/operators/superop.m:36-185 -> rows [row(out), col(in), coeff]."""
    if side == 'comm':
        A = superop(ss, opspec, 'leftofcomm')
        B = superop(ss, opspec, 'rightofcomm')
        B = B.copy(); B[:, 2] = -B[:, 2]
        return np.vstack([A, B])
    if side == 'acomm':
        return np.vstack([superop(ss, opspec, 'left'), superop(ss, opspec, 'right')])
    active = np.nonzero(opspec)[0]
    dim = ss.basis.shape[0]
    if active.size == 0:
        idx = np.arange(dim, dtype=float)
        return np.stack([idx, idx, np.ones(dim)], axis=1)
    srcs, dsts, coefs = [], [], []
    for s in active:
        tbl = ss.lpst if side in ('left', 'leftofcomm') else ss.rpst
        pt = tbl[int(ss.mults[s])][int(opspec[s])]      # pt[m_in, k_out]
        d_idx, s_idx = np.nonzero(pt)
        # MATLAB find() walks column-major: sort by column then row
        order = np.lexsort((d_idx, s_idx))
        d_idx, s_idx = d_idx[order], s_idx[order]
        dsts.append(d_idx); srcs.append(s_idx); coefs.append(pt[d_idx, s_idx])
    frm = srcs[0][:, None]; to = dsts[0][:, None]; coeff = coefs[0]
    for k in range(1, len(active)):
        ns = srcs[k].size; nf = frm.shape[0]
        frm = np.hstack([np.repeat(frm, ns, axis=0), np.tile(srcs[k][:, None], (nf, 1))])
        to = np.hstack([np.repeat(to, ns, axis=0), np.tile(dsts[k][:, None], (nf, 1))])
        coeff = np.kron(coeff, coefs[k])
    if side in ('leftofcomm', 'rightofcomm'):
        kill = (frm.sum(axis=1) == 0) | (to.sum(axis=1) == 0)
        frm, to, coeff = frm[~kill], to[~kill], coeff[~kill]
    bcols = ss.basis[:, active]
    inactive = np.setdiff1d(np.arange(ss.nspins), active)
    out = []
    for n in range(frm.shape[0]):
        smask = np.all(bcols == frm[n], axis=1)
        sidx = np.nonzero(smask)[0]
        if sidx.size == 0:
            continue
        dmask = np.all(bcols == to[n], axis=1)
        didx = np.nonzero(dmask)[0]
        ssub = ss.basis[np.ix_(sidx, inactive)]
        dsub = ss.basis[np.ix_(didx, inactive)]
        if ssub.shape == dsub.shape and np.array_equal(ssub, dsub):
            out.append(np.stack([sidx, didx, np.full(sidx.size, coeff[n])], axis=1))
        else:
            lookup = {tuple(r): i for i, r in zip(didx, dsub)}
            pairs = [(si, lookup[tuple(r)]) for si, r in zip(sidx, ssub) if tuple(r) in lookup]
            if pairs:
                pr = np.array(pairs, float)
                out.append(np.hstack([pr, np.full((len(pairs), 1), coeff[n])]))
    if not out:
        return np.array([[0.0, 0.0, 0.0]])
    return np.vstack(out).astype(float)


def human2opspec(ss: SpinSystem, operators, spins):
    """kernel/utilities/human2opspec.m (spin-only subset: E, L+, L-, Lx, Ly, Lz, Tl,m)."""
    if isinstance(operators, str) and isinstance(spins, (int, np.integer)):
        return human2opspec(ss, [operators], [int(spins)])
    if isinstance(operators, str) and isinstance(spins, str):
        nums = [i for i, s in enumerate(ss.isotopes) if s == spins] if spins not in ('all',) \
            else list(range(ss.nspins))
        if not nums:
            raise ValueError('no such spins in the system.')
        specs, cfs = [], []
        for k in nums:
            a, b = human2opspec(ss, [operators], [k])
            specs.extend(a); cfs.extend(b)
        return specs, cfs
    specs = [np.zeros(ss.nspins, np.int64)]
    cfs = [1.0 + 0j]
    for op, s in zip(operators, spins):
        if op == 'E':
            for x in specs:
                x[s] = 0
        elif op == 'L+':
            for x in specs:
                x[s] = 1
            cfs = [-math.sqrt(2) * c for c in cfs]
        elif op == 'L-':
            for x in specs:
                x[s] = 3
            cfs = [math.sqrt(2) * c for c in cfs]
        elif op in ('Lx', 'Ly'):
            a = [x.copy() for x in specs]; b = [x.copy() for x in specs]
            for x in a:
                x[s] = 1
            for x in b:
                x[s] = 3
            if op == 'Lx':
                ca, cb = -math.sqrt(2) / 2, math.sqrt(2) / 2
            else:
                ca, cb = -math.sqrt(2) / 2j, -math.sqrt(2) / 2j
            specs = a + b
            cfs = [ca * c for c in cfs] + [cb * c for c in cfs]
        elif op == 'Lz':
            for x in specs:
                x[s] = 2
        elif op.startswith('T'):
            l, m = (int(v) for v in op[1:].split(','))
            for x in specs:
                x[s] = lm2lin(l, m)
        else:
            raise ValueError('unrecognized operator specification.')
    return specs, cfs


def operator(ss: SpinSystem, operators, spins, operator_type: str = 'comm') -> sp.csc_matrix:
    """kernel/operator.m:71-215 (sphten-liouv branch), returned in CSC form."""
    specs, cfs = human2opspec(ss, operators, spins)
    parts = []
    for spec, c in zip(specs, cfs):
        A = superop(ss, spec, operator_type).astype(complex)
        A[:, 2] *= c
        parts.append(A)
    A = np.vstack(parts)
    dim = ss.basis.shape[0]
    return sp.csc_matrix((A[:, 2], (A[:, 0].real.astype(np.int64), A[:, 1].real.astype(np.int64))),
                         shape=(dim, dim))


def state(ss: SpinSystem, states, spins) -> np.ndarray:
    """kernel/state.m:75-153, 'exact' method: operator(...,'left')*unit."""
    dim = ss.basis.shape[0]
    unit = np.zeros(dim, complex); unit[0] = 1.0
    return operator(ss, states, spins, 'left') @ unit


# --------------------------------------------------------------------------
# Hamiltonian, orientation, relaxation
# --------------------------------------------------------------------------

_S23 = math.sqrt(2 / 3)
_S18 = math.sqrt(1 / 8)


def _coupling_terms(strength: str):
    """Anisotropic coupling descriptor rows, kernel/hamiltonian.m:384-580.

    Returns [(opL, opS, ist1 (3,), ist2 (5,))]."""
    zz = ('Lz', 'Lz', [0, 0, 0], [0, 0, _S23, 0, 0])
    pm = ('L+', 'L-', [0, -_S18, 0], [0, 0, -_S23 / 4, 0, 0])
    mp = ('L-', 'L+', [0, +_S18, 0], [0, 0, -_S23 / 4, 0, 0])
    zp = ('Lz', 'L+', [0.5, 0, 0], [0, -0.5, 0, 0, 0])
    pz = ('L+', 'Lz', [-0.5, 0, 0], [0, -0.5, 0, 0, 0])
    zm = ('Lz', 'L-', [0, 0, 0.5], [0, 0, 0, 0.5, 0])
    mz = ('L-', 'Lz', [0, 0, -0.5], [0, 0, 0, 0.5, 0])
    pp = ('L+', 'L+', [0, 0, 0], [0.5, 0, 0, 0, 0])
    mm = ('L-', 'L-', [0, 0, 0], [0, 0, 0, 0, 0.5])
    table = {
        'strong': [zz, pm, mp, zp, pz, zm, mz, pp, mm],
        'z*': [zz, zp, zm],
        '*z': [zz, pz, mz],
        'secular': [zz, pm, mp],
        'zz': [zz],
        'z+': [zp], '+z': [pz], 'T(L,+1)': [zp, pz],
        'z-': [zm], '-z': [mz], 'T(L,-1)': [zm, mz],
        'ignore': [],
    }
    return table[strength]


def hamiltonian(ss: SpinSystem, operator_type: str = 'comm'):
    """kernel/hamiltonian.m:44-790 -> (I, Q) with Q[r][k][m] (0-based k, m);
    operator_type 'left' gives left-side product superoperators (the 'left'
    argument of hamiltonian.m, used for thermal equilibria).

    Descriptor rows are (isotropic, ist[8], irr[8], operator spec); I and Q are
    assembled as in :705-790 and cleaned to liouv_zero."""
    tz = ss.tols['liouv_zero']
    rows = []   # (iso, ist(8), irr(8), ops(list), spins(list))
    n = ss.nspins
    for s in range(n):
        Z = ss.zeeman[s]
        st = ss.zeeman_strength[s]
        _, lam, phi = mat2sphten(Z)
        irr = np.concatenate([lam, phi])
        aniso = (np.linalg.norm(lam) > tz) or (np.linalg.norm(phi) > tz)
        iso = 0.0
        if st == 'full':
            iso = np.trace(Z) / 3
        elif st == 'secular':
            iso = np.trace(Z) / 3 - ss.basefrqs[s]
        iso = iso if abs(iso) > tz else 0.0
        ist = {op: np.zeros(8, complex) for op in ('L+', 'Lz', 'L-')}
        if aniso and st == 'full':
            ist['L+'][0] = -0.5; ist['L+'][4] = -0.5
            ist['Lz'][5] = _S23
            ist['L-'][2] = -0.5; ist['L-'][6] = +0.5
        elif aniso and st == 'secular':
            ist['Lz'][5] = _S23
        for op in ('L+', 'Lz', 'L-'):
            isov = iso if op == 'Lz' else 0.0
            irrv = irr if aniso else np.zeros(8, complex)
            rows.append((isov, ist[op], irrv, [op], [s]))
        # quadratic couplings (hamiltonian.m:191-257): rank-2 operators of the
        # spin itself, all five ('strong') or T(2,0) alone ('secular')
        Mq = ss.coupling.get((s, s))
        if Mq is not None and np.linalg.norm(Mq, 2) > 2 * np.pi * ss.tols['inter_cutoff']:
            iq, lq, pq = mat2sphten(Mq)
            if np.linalg.norm(iq) > 1e-6 * np.linalg.norm(pq) or np.linalg.norm(lq) > 1e-6 * np.linalg.norm(pq):
                raise ValueError('quadratic couplings must be traceless and symmetric.')
            irrq = np.concatenate([np.zeros(3, complex), pq])
            stq = ss.coupling_strength[(s, s)]
            if stq == 'strong':
                qops = [('T2,+2', 3), ('T2,+1', 4), ('T2,0', 5), ('T2,-1', 6), ('T2,-2', 7)]
            elif stq == 'secular':
                qops = [('T2,0', 5)]
            else:
                raise ValueError('unknown strength specification for the quadratic coupling.')
            for op, idx in qops:
                istq = np.zeros(8, complex)
                istq[idx] = 1.0
                rows.append((0.0, istq, irrq, [op], [s]))
    cutoff = 2 * np.pi * ss.tols['inter_cutoff']
    pairs = sorted([k for k, M in ss.coupling.items() if k[0] != k[1] and np.linalg.norm(M, 2) > cutoff],
                   key=lambda ab: (ab[1], ab[0]))
    for (a, b) in pairs:
        M = ss.coupling[(a, b)]
        st = ss.coupling_strength[(a, b)]
        ciso = np.trace(M) / 3
        iso_rows = []
        if abs(ciso) > cutoff:
            if st in ('strong', 'secular'):
                iso_rows = [('Lz', 'Lz', ciso), ('L+', 'L-', ciso / 2), ('L-', 'L+', ciso / 2)]
            elif st in ('z*', '*z', 'zz'):
                iso_rows = [('Lz', 'Lz', ciso)]
        _, lam, phi = mat2sphten(M)
        aniso = (np.linalg.norm(lam) > tz) or (np.linalg.norm(phi) > tz)
        irr = np.concatenate([lam, phi]) if aniso else np.zeros(8, complex)
        entries = {}
        for opL, opS, v in iso_rows:
            entries.setdefault((opL, opS), [0.0, np.zeros(8, complex)])[0] = v
        if aniso:
            for opL, opS, i1, i2 in _coupling_terms(st):
                entries.setdefault((opL, opS), [0.0, np.zeros(8, complex)])[1] = np.array(i1 + i2, complex)
        for (opL, opS), (isov, ist) in entries.items():
            rows.append((isov, ist, irr, [opL, opS], [a, b]))
    # kill insignificant rows (hamiltonian.m:268-273, 583-588)
    kept = []
    for isov, ist, irr, ops, spins in rows:
        ma = abs(isov) < tz
        mb = np.sum(np.abs(irr)) < tz
        mc = np.sum(np.abs(ist)) < tz
        if not (ma and (mb or mc)):
            kept.append((isov, ist, irr, ops, spins))
    opers = [operator(ss, ops, spins, operator_type) for _, _, _, ops, spins in kept]
    dim = ss.basis.shape[0]
    I = sp.csc_matrix((dim, dim), dtype=complex)
    for (isov, _, _, _, _), O in zip(kept, opers):
        if abs(isov) > tz:
            I = I + isov * O
    I = clean_up(ss, I, tz)
    Q = {1: [[None] * 3 for _ in range(3)], 2: [[None] * 5 for _ in range(5)]}
    for r in (1, 2):
        for m in range(2 * r + 1):
            for k in range(2 * r + 1):
                acc = sp.csc_matrix((dim, dim), dtype=complex)
                for (_, ist, irr, _, _), O in zip(kept, opers):
                    coeff = ist[r * r + k - 1] * irr[r * r + m - 1]
                    if abs(coeff) > tz:
                        acc = acc + coeff * O
                Q[r][k][m] = clean_up(ss, acc, tz)
    return I, Q


def orientation(Q: dict, angles) -> sp.csc_matrix:
    """kernel/orientation.m:29-57: sum_r sum_km D^r(k,m) Q{r}{k,m}, then (H+H')/2."""
    H = None
    for r in sorted(Q):
        D = wigner(r, *angles)
        for k in range(2 * r + 1):
            for m in range(2 * r + 1):
                if Q[r][k][m] is not None and Q[r][k][m].nnz > 0:
                    term = D[k, m] * Q[r][k][m]
                    H = term if H is None else H + term
    if H is None:
        return None
    return (H + H.conj().T) / 2


def relaxation(ss: SpinSystem) -> sp.csc_matrix:
    """kernel/relaxation.m:72-93 with kernel/utilities/rlx_t1_t2.m:32-178
    (scalar rates), plus :638-684 ('damp', isotropic: RD = -rate*1, then
    R + RD - (U'*RD*U)*(U*U') so that the unit state U is not damped)."""
    dim = ss.basis.shape[0]
    R = sp.csc_matrix((dim, dim), dtype=complex)
    if 't1_t2' in ss.theories:
        R = R + _rlx_t1_t2(ss)
    if 'damp' in ss.theories:
        dr = np.asarray(getattr(ss, 'damp_rate', 0.0), float)
        rate = float(np.mean(np.diag(dr))) if dr.ndim == 2 else float(dr)
        RD = -rate * sp.identity(dim, dtype=complex, format='csc')
        u = np.zeros(dim, complex)
        u[np.where((ss.basis == 0).all(axis=1))[0][0]] = 1.0
        U = sp.csc_matrix(u.reshape(-1, 1))
        R = R + RD - (U.conj().T @ RD @ U).toarray()[0, 0] * (U @ U.conj().T)
    return sp.csc_matrix(R)


def _rlx_t1_t2(ss: SpinSystem) -> sp.csc_matrix:
    """kernel/utilities/rlx_t1_t2.m:32-178 with scalar R1/R2 per spin."""
    L, M = lin2lm(ss.basis)
    mask = L != 0
    r1 = np.asarray(ss.r1, float); r2 = np.asarray(ss.r2, float)
    long_ = (M == 0) & mask
    tran = (M != 0) & mask
    r1d = (long_ * r1[None, :]).sum(axis=1)
    r2d = (tran * r2[None, :]).sum(axis=1)
    return sp.diags(-r1d, 0, format='csc').astype(complex) + sp.diags(-r2d, 0, format='csc').astype(complex)


# --------------------------------------------------------------------------
# Numerics: clean_up, cheap_norm, propagator, step, krylov, evolution
# --------------------------------------------------------------------------

def _mround(x):
    """MATLAB round(): half away from zero, real and imaginary parts separately."""
    def r(v):
        return np.sign(v) * np.floor(np.abs(v) + 0.5)
    if np.iscomplexobj(x):
        return r(x.real) + 1j * r(x.imag)
    return r(x)


def clean_up(ss: SpinSystem, A, tol):
    """kernel/utilities/clean_up.m:22-89 (non-MEX branch): tol*round(A/tol).

    Dense/sparse storage switching is a storage decision only and is not
    restated; the arithmetic is."""
    if tol == 0 or (isinstance(tol, float) and math.isnan(tol)):
        return A
    if sp.issparse(A):
        A = A.tocsc(copy=True)
        A.data = tol * _mround((1 / tol) * A.data)
        A.eliminate_zeros()
        return A
    return tol * _mround((1 / tol) * A)


def cheap_norm(A) -> float:
    """kernel/utilities/cheap_norm.m:44-51: 1-norm on the CPU path."""
    if sp.issparse(A):
        return float(abs(A).sum(axis=0).max()) if A.nnz else 0.0
    return float(np.abs(A).sum(axis=0).max()) if A.size else 0.0


def propagator(ss: SpinSystem, L, dt: float) -> np.ndarray:
    """kernel/propagator.m:34-211: expm below small_matrix, else chopped Taylor
    with scaling and squaring.  Returns a dense array."""
    dim = L.shape[0]
    if dim < ss.tols['small_matrix']:
        Ld = L.toarray() if sp.issparse(L) else L
        return sla.expm((-1j * dt) * Ld)
    chop = ss.tols['prop_chop']
    A = (-1j * dt) * (L.toarray() if sp.issparse(L) else L)
    A = clean_up(ss, A, chop)
    nrm = cheap_norm(A)
    if nrm > 1e9:
        raise ValueError('norm of -i*L*dt exceeds 1e9, check your L and your dt.')
    elif nrm > 1024:
        chop = EPS
    n_sq = max(0, int(math.ceil(math.log2(nrm)))) if nrm > 0 else 0
    if n_sq > 0:
        A = (1 / 2 ** n_sq) * A
    P = np.eye(dim, dtype=complex)
    nxt = P.copy()
    n = 1
    while np.count_nonzero(nxt) > 0:
        nxt = (1 / n) * (nxt @ A)
        nxt = clean_up(ss, nxt, chop)
        P = P + nxt
        n += 1
    P = clean_up(ss, P, chop)
    for _ in range(n_sq):
        P = clean_up(ss, P @ P, chop)
    return P


def _reordered_taylor(L, rho, t, nsteps):
    """kernel/step.m:328-375 (single generator)."""
    for _ in range(nsteps):
        nxt = rho
        k = 1
        while np.count_nonzero(np.abs(nxt) > EPS) > 0:
            nxt = -(1j / k) * (t / nsteps) * (L @ nxt)
            rho = rho + nxt
            k += 1
    return rho


def step(ss: SpinSystem, L, rho, dt: float):
    """kernel/step.m:204-267 (Liouville branch, CPU 1-norm)."""
    if dt == 0:
        return rho
    rho = np.asarray(rho, complex)
    scaling = np.max(np.abs(rho))
    if scaling == 0:
        return rho
    rho = rho / scaling
    nsteps = int(math.ceil(cheap_norm(L) * abs(dt) / 2))
    if nsteps > 1e4:
        raise ValueError('either dt is too long, or L is too big: |L*dt|>1e4, check both.')
    rho = _reordered_taylor(L, rho, dt, nsteps)
    return scaling * rho


def krylov_observable(ss: SpinSystem, L, coil, rho, dt: float, nsteps: int) -> np.ndarray:
    """kernel/krylov.m:139-163 ('observable')."""
    L = sp.csr_matrix(L)
    ans = np.zeros(nsteps + 1, complex)
    ans[0] = np.vdot(coil, rho)
    for n in range(1, nsteps + 1):
        rho = step(ss, L, rho, dt)
        ans[n] = np.vdot(coil, rho)
    return ans


def evolution_observable(ss: SpinSystem, L, coil, rho, dt: float, nsteps: int) -> np.ndarray:
    """kernel/evolution.m:503-587 ('observable', trajectory-level reduction off)."""
    L = clean_up(ss, sp.csc_matrix(L), ss.tols['liouv_zero'])
    rho = clean_up(ss, np.asarray(rho, complex), ss.tols['zte_tol'])
    coil = clean_up(ss, np.asarray(coil, complex), ss.tols['zte_tol'])
    dim = L.shape[0]
    if dim < ss.tols['krylov_tol'] and 'krylov' not in ss.enable:
        P = propagator(ss, L, dt)
        ans = np.zeros(nsteps + 1, complex)
        for n in range(nsteps + 1):
            ans[n] = np.vdot(coil, rho)
            rho = P @ rho
        return ans
    return krylov_observable(ss, L, coil, rho, dt, nsteps)


def decouple(ss: SpinSystem, L, rho, spins):
    """kernel/decouple.m:46-95 (sphten-liouv, one spatial point): rows and
    columns of L and entries of rho of every state in which a decoupled spin
    is not in its unit state are zeroed."""
    if not spins:
        return L, rho
    if any(s not in ss.isotopes for s in spins):
        raise ValueError('the system does not contain the spins specified.')
    dec = np.array([iso in spins for iso in ss.isotopes])
    zero = ss.basis[:, dec].sum(axis=1) != 0
    keep = sp.diags((~zero).astype(float))
    L = clean_up(ss, sp.csc_matrix(keep @ L @ keep), ss.tols['liouv_zero'])
    rho = np.where(zero, 0.0, np.asarray(rho, complex))
    return L, rho


def acquire(ss: SpinSystem, parameters: dict, H, R) -> np.ndarray:
    """experiments/acquire.m:42-73: L=H+iR, the decoupling (:51), the
    homodecoupling L + 2*pi*pwr*oper (:54-62), the dead time (:65-67), then
    evolution(...,1/sweep,npoints-1,'observable')."""
    L = H + 1j * R
    rho0 = parameters['rho0']
    L, rho0 = decouple(ss, L, rho0, parameters.get('decouple', []))
    if 'homodec_oper' in parameters:
        L = L + 2 * np.pi * parameters['homodec_pwr'] * parameters['homodec_oper']
    if 'dead_time' in parameters:
        rho0 = step(ss, sp.csr_matrix(L), rho0, parameters['dead_time'])
    return evolution_observable(ss, L, parameters['coil'], rho0,
                                1.0 / parameters['sweep'], parameters['npoints'] - 1)


def evolution_trajectory(ss: SpinSystem, L, rho, dt: float, nsteps: int) -> np.ndarray:
    """kernel/evolution.m:310-381 ('trajectory', one subspace): the states at
    steps 0..nsteps as columns; propagator below krylov_tol, else repeated
    step() (kernel/krylov.m 'trajectory')."""
    L = clean_up(ss, sp.csc_matrix(L), ss.tols['liouv_zero'])
    rho = clean_up(ss, np.asarray(rho, complex), ss.tols['zte_tol'])
    dim = L.shape[0]
    ans = np.zeros((dim, nsteps + 1), complex)
    if dim < ss.tols['krylov_tol'] and 'krylov' not in ss.enable:
        P = propagator(ss, L, dt)
        for n in range(nsteps + 1):
            ans[:, n] = rho
            rho = P @ rho
    else:
        L = sp.csr_matrix(L)
        ans[:, 0] = rho
        for n in range(1, nsteps + 1):
            rho = step(ss, L, rho, dt)
            ans[:, n] = rho
    return clean_up(ss, ans, ss.tols['zte_tol'])


def _spatial(parameters: dict, op):
    """kron(speye(spc_dim), op): an operator of the spin space projected into
    a context's spatial (rotor or Fourier) space; spc_dim = 1 by default."""
    n = int(parameters.get('spc_dim', 1))
    return op if n == 1 else sp.kron(sp.identity(n), sp.csr_matrix(op), format='csr')


def cpmg(ss: SpinSystem, parameters: dict, H, R) -> np.ndarray:
    """experiments/cpmg.m:29-63 (K = 0, one spatial point): a 90-degree pulse
    step(pulse_op, rho0, pi/2), a half-echo of npoints-1 steps, then nloops
    times a 180-degree pulse on the last state and an echo of 2*npoints-1
    steps; the detected trajectories concatenated.  The pulse operator is
    projected into the spatial space first, kron(speye(spc_dim), pulse_op)
    (:33; spc_dim = 1 in the powder context)."""
    L = H + 1j * R
    coil = np.asarray(parameters['coil'], complex)
    P = _spatial(parameters, parameters['pulse_op'])
    dt = parameters['timestep']
    rho = step(ss, P, parameters['rho0'], np.pi / 2)
    traj = evolution_trajectory(ss, L, rho, dt, parameters['npoints'] - 1)
    fid = [coil.conj() @ traj]
    for _ in range(parameters['nloops']):
        last = step(ss, P, traj[:, -1], np.pi)
        traj = evolution_trajectory(ss, L, last, dt, 2 * parameters['npoints'] - 1)
        fid.append(coil.conj() @ traj)
    return np.concatenate(fid)


def hp_acquire(ss: SpinSystem, parameters: dict, H, R) -> np.ndarray:
    """experiments/hp_acquire.m (K = 0, no decoupling): pulse_op by
    pulse_angle; if echo_time is given, echo_time of evolution ('final', one
    step), echo_oper by echo_angle, echo_time again; then the observable of
    npoints-1 steps of 1/sweep.  Both operators are projected into the
    spatial space, kron(speye(spc_dim), op) (:57,69)."""
    L = H + 1j * R
    rho = step(ss, _spatial(parameters, parameters['pulse_op']), parameters['rho0'], parameters['pulse_angle'])
    if 'echo_time' in parameters:
        rho = evolution_trajectory(ss, L, rho, parameters['echo_time'], 1)[:, -1]
        rho = step(ss, _spatial(parameters, parameters['echo_oper']), rho, parameters['echo_angle'])
        rho = evolution_trajectory(ss, L, rho, parameters['echo_time'], 1)[:, -1]
    return evolution_observable(ss, L, parameters['coil'], rho, 1.0 / parameters['sweep'],
                                parameters['npoints'] - 1)


def evolution_refocus(ss: SpinSystem, stack, L, dt: float) -> np.ndarray:
    """kernel/evolution.m:402-470 ('refocus', one subspace): column n of the
    stack is propagated n steps; propagator below krylov_tol, else the stack
    stepping of kernel/krylov.m:116-137."""
    L = clean_up(ss, sp.csc_matrix(L), ss.tols['liouv_zero'])
    stack = clean_up(ss, np.array(stack, complex), ss.tols['zte_tol'])
    dim, ncol = stack.shape
    if dim < ss.tols['krylov_tol'] and 'krylov' not in ss.enable:
        P = propagator(ss, L, dt)
        for n in range(1, ncol):
            stack[:, n:] = P @ stack[:, n:]
    else:
        L = sp.csr_matrix(L)
        for n in range(1, ncol):
            stack[:, n:] = step(ss, L, stack[:, n:], dt)
    return clean_up(ss, stack, ss.tols['zte_tol'])


def eseem(ss: SpinSystem, parameters: dict, H, R, first_angle: float = np.pi / 2) -> np.ndarray:
    """experiments/esr_dipolar/eseem.m:40-64 (K = 0, no screening): 90-degree
    pulse, trajectory of npoints-1 steps of timestep/2, 180-degree pulse on
    every column, refocusing, detection."""
    L = H + 1j * R
    P = parameters['pulse_op']
    tau = parameters['timestep'] / 2
    rho = step(ss, P, parameters['rho0'], first_angle)
    stack = evolution_trajectory(ss, L, rho, tau, parameters['npoints'] - 1)
    stack = step(ss, P, stack, np.pi)
    stack = evolution_refocus(ss, stack, L, tau)
    return np.asarray(parameters['coil'], complex).conj() @ stack


def oopeseem(ss: SpinSystem, parameters: dict, H, R) -> np.ndarray:
    """experiments/esr_dipolar/oopeseem.m (K = 0, no screening): eseem.m with
    a 45-degree first pulse."""
    return eseem(ss, parameters, H, R, first_angle=np.pi / 4)


def evolution_final(ss: SpinSystem, L, rho, dt: float, nsteps: int) -> np.ndarray:
    """kernel/evolution.m:168-246 ('final', one subspace): below krylov_tol the
    user timing is replaced by nsteps_opt = max(1, ceil(log2(dim/(ncols*log 2))))
    steps of total_time/nsteps_opt with one propagator (:196-234); otherwise
    kernel/krylov.m:84-90, one step() of the whole time.  rho may be a stack."""
    L = clean_up(ss, sp.csc_matrix(L), ss.tols['liouv_zero'])
    rho = clean_up(ss, np.array(rho, complex), ss.tols['zte_tol'])
    dim = L.shape[0]
    total = dt * nsteps
    if dim < ss.tols['krylov_tol'] and 'krylov' not in ss.enable:
        ncols = 1 if rho.ndim == 1 else rho.shape[1]
        n_opt = max(1, math.ceil(math.log2(dim / (ncols * math.log(2)))))
        P = propagator(ss, L, total / n_opt)
        for _ in range(n_opt):
            rho = P @ rho
    else:
        rho = step(ss, sp.csr_matrix(L), rho, total)
    return clean_up(ss, rho, ss.tols['zte_tol'])


def deer_3p_hard(ss: SpinSystem, parameters: dict, H, R) -> np.ndarray:
    """experiments/esr_dipolar/deer_3p_hard_deer.m ('brief' output, K = 0):
    probe 90-degree pulse, trajectory of nsteps steps of stepsize, pump
    180-degree pulse on every column, the reversed stack refocused, probe
    180-degree pulse, nsteps more steps ('final'), detection on coil_prob
    divided by its 2-norm."""
    L = H + 1j * R
    dt, n = parameters['stepsize'], parameters['nsteps']
    rho = step(ss, parameters['ex_prob'], parameters['rho0'], np.pi / 2)
    stack = evolution_trajectory(ss, L, rho, dt, n)
    stack = step(ss, parameters['ex_pump'], stack, np.pi)
    stack[:, ::-1] = evolution_refocus(ss, stack[:, ::-1], L, dt)
    stack = step(ss, parameters['ex_prob'], stack, np.pi)
    stack = evolution_final(ss, L, stack, dt, n)
    coil = np.asarray(parameters['coil_prob'], complex)
    return coil.conj() @ stack / np.linalg.norm(coil)


def inv_rec(ss: SpinSystem, parameters: dict, H, R) -> np.ndarray:
    """experiments/inv_rec.m (K = 0): rho0 = equilibrium(spin_system), the
    isotropic lab-frame equilibrium (equilibrium.m:63-67, hamiltonian.m with
    one output builds no anisotropic part); Ly of spins{1} from L+; a
    180-degree pulse, n_delays steps of max_delay/n_delays ('trajectory'), a
    90-degree pulse on every column, then the observable of npoints-1 steps of
    1/sweep on L+; the answer is npoints x (n_delays+1)."""
    import copy
    L = H + 1j * R
    ssL = assume(copy.deepcopy(ss), 'labframe')
    IL, _ = hamiltonian(ssL, 'left')
    rho0 = equilibrium(ssL, IL, {}, (0.0, 0.0, 0.0))
    spin = parameters['spins'][0]
    coil = state(ss, 'L+', spin)
    Lp = operator(ss, 'L+', spin)
    Ly = (Lp - Lp.conj().T) / 2j
    rho = step(ss, Ly, rho0, np.pi)
    nd = parameters['n_delays']
    stack = evolution_trajectory(ss, L, rho, parameters['max_delay'] / nd, nd)
    stack = step(ss, Ly, stack, np.pi / 2)
    return np.stack([evolution_observable(ss, L, coil, stack[:, k], 1.0 / parameters['sweep'],
                                          parameters['npoints'] - 1) for k in range(nd + 1)], axis=1)


def deer_3p_hard_echo(ss: SpinSystem, parameters: dict, H, R) -> np.ndarray:
    """experiments/esr_dipolar/deer_3p_hard_echo.m (K = 0): probe 90 degrees,
    tb, pump 180 degrees, ta-tb, probe 180 degrees, ta-tc/2 (each 'final', one
    step), then the echo observed over tc in nsteps steps."""
    L = H + 1j * R
    ta, tb, tc, n = parameters['ta'], parameters['tb'], parameters['tc'], parameters['nsteps']
    rho = step(ss, parameters['ex_prob'], parameters['rho0'], np.pi / 2)
    rho = evolution_final(ss, L, rho, tb, 1)
    rho = step(ss, parameters['ex_pump'], rho, np.pi)
    rho = evolution_final(ss, L, rho, ta - tb, 1)
    rho = step(ss, parameters['ex_prob'], rho, np.pi)
    rho = evolution_final(ss, L, rho, ta - 0.5 * tc, 1)
    return evolution_observable(ss, L, parameters['coil'], rho, tc / n, n)


# --------------------------------------------------------------------------
# Grids and the powder context
# --------------------------------------------------------------------------

def grid_zcwn(n: int):
    """kernel/grids/grid_fibon.m:70-78 ('zcwn'); uniform weights 1/n."""
    phi = (1 + math.sqrt(5)) / 2
    k = np.arange(n)
    bets = np.arccos(2 * (k / n) - 1)
    gams = 2 * np.pi * k / phi ** 2
    return np.zeros(n), bets, gams, np.full(n, 1.0 / n)


def grid_fib(parm: int):
    """kernel/grids/grid_fibon.m:43-54 ('fib', 2*parm+1 points); uniform weights."""
    phi = (1 + math.sqrt(5)) / 2
    k = np.arange(-parm, parm + 1)
    bets = np.arccos(2 * k / (2 * parm + 1))
    gams = 2 * np.pi * k / phi
    n = 2 * parm + 1
    return np.zeros(n), bets, gams, np.full(n, 1.0 / n)


def frqoffset(ss: SpinSystem, H, spins, offsets):
    """kernel/frqoffset.m:27-55: H + 2*pi*offset*Lz(isotope) per channel;
    channels naming the same isotope must carry the same offset."""
    if not spins:
        raise ValueError('parameters.spins variable cannot be empty.')
    if len(offsets) != len(spins):
        raise ValueError('parameters.offset must have the same number of elements as parameters.spins')
    if any(s not in ss.isotopes for s in spins):
        raise ValueError('parameters.spins refers to a spin that is not present in the system.')
    seen = {}
    for s, off in zip(spins, offsets):
        if s in seen and seen[s] != off:
            raise ValueError('offsets on channels referring to the same spin must be the same.')
        seen[s] = off
    for s in sorted(seen, key=spins.index):
        if seen[s] != 0:
            H = H + 2 * np.pi * seen[s] * operator(ss, 'Lz', s)
    return H


def equilibrium(ss: SpinSystem, I, Q, angles) -> np.ndarray:
    """kernel/states/equilibrium.m:53-100 (sphten-liouv, four arguments):
    H = I + orientation(Q, angles), rho = step(H, unit, -1i*beta) =
    exp(-beta*H) unit with beta = hbar/(k*T), normalised to <unit|rho> = 1.
    I and Q are left-side product superoperators of the lab-frame Hamiltonian."""
    if ss.temperature is None or ss.temperature == 0:
        raise ValueError('temperature must be specified (and non-zero)')
    beta = HBAR / (1.380649e-23 * ss.temperature)
    A = orientation(Q, angles)
    H = I if A is None else I + A
    dim = H.shape[0]
    unit = np.zeros(dim, complex)
    unit[0] = 1.0
    if np.abs(H @ unit).sum() < 1e-10:
        raise ValueError('H and Q must be left side product superops, not commutation superops.')
    rho = step(ss, sp.csr_matrix(H), unit, -1j * beta)
    return rho / np.vdot(unit, rho)


def powder_setup(ss: SpinSystem, assumptions: str):
    """kernel/contexts/powder.m:148-161: assume, then [I,Q]=hamiltonian once."""
    ss = assume(ss, assumptions)
    I, Q = hamiltonian(ss)
    return ss, I, Q


def powder_orientation_fid(ss, I, Q, parameters, angles) -> np.ndarray:
    """One iteration of kernel/contexts/powder.m:226-274 with @acquire."""
    A = orientation(Q, angles)
    H = I if A is None else I + A
    H = (H + H.conj().T) / 2
    R = relaxation(ss)
    return acquire(ss, parameters, H, R)


def powder_orientation_cpmg(ss, I, Q, parameters, angles) -> np.ndarray:
    """One iteration of kernel/contexts/powder.m:226-274 with @cpmg."""
    A = orientation(Q, angles)
    H = I if A is None else I + A
    H = (H + H.conj().T) / 2
    return cpmg(ss, parameters, H, relaxation(ss))


def fourdif1(N: int):
    """kernel/derivatives/fourdif.m:44-77 with m = 1: rotor grid points and the
    first-derivative Fourier collocation matrix (first column, then Toeplitz)."""
    x = 2 * np.pi * np.arange(N) / N
    h = 2 * np.pi / N
    kk = np.arange(1, N)
    n1 = (N - 1) // 2
    n2 = -(-(N - 1) // 2)
    if N % 2 == 0:
        topc = 1 / np.tan(np.arange(1, n2 + 1) * h / 2)
        col1 = np.concatenate([[0.0], 0.5 * ((-1.0) ** kk) * np.concatenate([topc, -topc[:n1][::-1]])])
    else:
        topc = 1 / np.sin(np.arange(1, n2 + 1) * h / 2)
        col1 = np.concatenate([[0.0], 0.5 * ((-1.0) ** kk) * np.concatenate([topc, topc[:n1][::-1]])])
    row1 = -col1
    return x, sla.toeplitz(col1, row1)


_MAS_SEQUENCES = {'acquire': 'acquire', 'hp_acquire': 'hp_acquire', 'cpmg': 'cpmg'}


def _mas_sequence(name):
    if name not in _MAS_SEQUENCES:
        raise ValueError(f'sequence {name!r} is not restated for the MAS contexts')
    return globals()[_MAS_SEQUENCES[name]]


def singlerot_orientation_fid(ss, I, Q, parameters, angles, sequence: str = 'acquire') -> np.ndarray:
    """One orientation of kernel/contexts/singlerot.m:134-307 with @acquire
    (or @hp_acquire / @cpmg, which project their pulses with spc_dim),
    sphten-liouv, no rotating frames: H_n = I + sum D_comp(k,m) Q{r}{k,m} with
    D_comp = D_lab2rot*D_rotor(phi_n)*D_mol2rot (:269-283, not Hermitised
    without rframes), G = clean_up(blkdiag(H)+1i*M, liouv_zero) (:298),
    M = 2*pi*rate*kron(d/dphi, I) (:190), R and states projected into rotor
    space (:191-215)."""
    N = 2 * parameters['max_rank'] + 1
    dim = I.shape[0]
    phases, Dfd = fourdif1(N)
    x, y, z = parameters['axis']
    rotor_phi = math.atan2(y, x)
    rotor_theta = math.pi / 2 - math.atan2(z, math.hypot(x, y))
    M = 2 * np.pi * parameters['rate'] * sp.kron(sp.csr_matrix(Dfd), sp.identity(dim))
    H = []
    for n in range(N):
        Hn = sp.csc_matrix(I, dtype=complex)
        for r in sorted(Q):
            Dc = wigner(r, rotor_phi, rotor_theta, 0) @ wigner(r, 0, 0, phases[n]) @ wigner(r, *angles)
            for k in range(2 * r + 1):
                for m in range(2 * r + 1):
                    if Q[r][k][m] is not None:
                        Hn = Hn + Dc[k, m] * Q[r][k][m]
        H.append(Hn)
    G = clean_up(ss, sp.csc_matrix(sp.block_diag(H) + 1j * M), ss.tols['liouv_zero'])
    R = sp.kron(sp.identity(N), relaxation(ss))
    if parameters.get('single_crystal'):
        space = np.zeros(N); space[0] = 1.0
    else:
        space = np.full(N, 1.0 / N)
    par = dict(parameters, rho0=np.kron(space, parameters['rho0']),
               coil=np.kron(np.ones(N), parameters['coil']), spc_dim=N)
    return _mas_sequence(sequence)(ss, par, G, R)


def powder_orientation_hp_acquire(ss, I, Q, parameters, angles) -> np.ndarray:
    """One iteration of kernel/contexts/powder.m:226-274 with @hp_acquire."""
    A = orientation(Q, angles)
    H = I if A is None else I + A
    H = (H + H.conj().T) / 2
    return hp_acquire(ss, parameters, H, relaxation(ss))


def powder_orientation_eseem(ss, I, Q, parameters, angles) -> np.ndarray:
    """One iteration of kernel/contexts/powder.m:226-274 with @eseem."""
    A = orientation(Q, angles)
    H = I if A is None else I + A
    H = (H + H.conj().T) / 2
    return eseem(ss, parameters, H, relaxation(ss))


def powder_orientation_sequence(ss, I, Q, parameters, angles, sequence) -> np.ndarray:
    """One iteration of kernel/contexts/powder.m:226-274 with any restated
    sequence function(ss, parameters, H, R)."""
    A = orientation(Q, angles)
    H = I if A is None else I + A
    H = (H + H.conj().T) / 2
    return sequence(ss, parameters, H, relaxation(ss))


def powder_orientation_deer(ss, I, Q, parameters, angles) -> np.ndarray:
    """One iteration of kernel/contexts/powder.m:226-274 with @deer_3p_hard_deer."""
    A = orientation(Q, angles)
    H = I if A is None else I + A
    H = (H + H.conj().T) / 2
    return deer_3p_hard(ss, parameters, H, relaxation(ss))


def floquet_orientation_fid(ss, I, Q, parameters, angles, sequence: str = 'acquire') -> np.ndarray:
    """One orientation of kernel/contexts/floquet.m:94-186 with @acquire (or
    @hp_acquire / @cpmg, which project their pulses with spc_dim):
    Fourier components of the rotor-frame Hamiltonian up to the highest
    interaction rank, F = sum_h kron(spdiags(1, h), T_h) + M, states in the
    zeroth Fourier component."""
    int_ranks = [r for r in sorted(Q) if any(q is not None and q.nnz for row in Q[r] for q in row)]
    max_int = max(int_ranks + [2])
    mr = parameters['max_rank']
    N = 2 * mr + 1
    dim = I.shape[0]
    x, y, z = parameters['axis']
    phi = math.atan2(y, x)
    theta = math.pi / 2 - math.atan2(z, math.hypot(x, y))
    M = 2 * np.pi * parameters['rate'] * sp.kron(sp.diags(np.arange(-mr, mr + 1, dtype=float)), sp.identity(dim))
    T = [sp.csc_matrix((dim, dim), dtype=complex) for _ in range(2 * max_int + 1)]
    for r in int_ranks:
        L2R = wigner(r, phi, theta, 0)
        R2L = L2R.conj().T
        Dm = L2R @ wigner(r, *angles) @ R2L
        for n in range(2 * r + 1):
            Dr = np.zeros((2 * r + 1, 2 * r + 1))
            Dr[n, n] = 1.0
            D = L2R @ Dr @ R2L @ Dm
            for m in range(2 * r + 1):
                for k in range(2 * r + 1):
                    if Q[r][k][m] is not None:
                        T[n - r + max_int] = T[n - r + max_int] + Q[r][k][m] * D[k, m]
    T[max_int] = T[max_int] + I
    F = sp.csc_matrix((N * dim, N * dim), dtype=complex)
    for h in range(2 * max_int + 1):
        d = h - max_int
        F = F + sp.kron(sp.diags(np.ones(N - abs(d)), d, shape=(N, N)), T[h])
    F = clean_up(ss, sp.csc_matrix(F + M), ss.tols['liouv_zero'])
    Rf = sp.kron(sp.identity(N), relaxation(ss))
    e = np.zeros(N)
    e[(N - 1) // 2] = 1.0
    par = dict(parameters, rho0=np.kron(e, parameters['rho0']), coil=np.kron(e, parameters['coil']), spc_dim=N)
    return _mas_sequence(sequence)(ss, par, F, Rf)


def powder(ss: SpinSystem, parameters: dict, assumptions: str, grid, setup=None,
           sum_up: bool = True):
    """kernel/contexts/powder.m:99-309 with pulse_sequence=@acquire, serial order.

    ``grid`` is (alphas, betas, gammas, weights).  Returns the weighted FID
    (powder.m:280-287) or the list of per-orientation FIDs (sum_up=false)."""
    if setup is None:
        ss, I, Q = powder_setup(ss, assumptions)
    else:
        I, Q = setup
    al, be, ga, w = grid
    fids = [powder_orientation_fid(ss, I, Q, parameters, (al[n], be[n], ga[n])) for n in range(len(w))]
    if not sum_up:
        return fids
    ans = w[0] * fids[0]
    for n in range(1, len(fids)):
        ans = ans + w[n] * fids[n]
    return ans
