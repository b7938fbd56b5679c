"""Host side of the Spinach-style calls (spinach_gb300.contexts): the
checks that powder.m, acquire.m, frqoffset.m and equilibrium.m make before
any orientation runs, and the thermal-equilibrium states against the oracle."""
import copy

import numpy as np
import pytest

from oracle import spinach_ref as R
from spinach_gb300 import contexts as X, spin_system as S


def _system(temperature=None):
    sys_ = dict(isotopes=['13C', '1H'], magnet=14.1)
    inter = dict(zeeman=dict(eigs=[[10.0, 70.0, 180.0], [1.0, 3.0, 8.0]], euler=[[0.1, 0.7, 1.9], [0, 0, 0]]),
                 coupling=dict(scalar={(0, 1): 140.0}))
    if temperature:
        inter['temperature'] = temperature
    return sys_, inter, X.basis(X.create(sys_, inter), dict(approximation='none'))


def test_argument_checks_before_any_run():
    _, _, spin_system = _system()
    base = dict(grid=(np.zeros(2), np.ones(2), np.ones(2), np.full(2, 0.5)), rho0=('Lx', '13C'),
                coil=('L+', '13C'), sweep=1e4, npoints=16)
    with pytest.raises(ValueError):                      # decoupling outside acquire
        X.powder(spin_system, 'cpmg', dict(base, decouple=['1H'], pulse_op=('Ly', '13C'), nloops=1,
                                           timestep=1e-4), 'nmr')
    with pytest.raises(ValueError):                      # equilibrium request and an explicit rho0
        X.powder(spin_system, 'acquire', dict(base, needs=['aniso_eq']), 'nmr')
    with pytest.raises(ValueError):                      # unknown need
        X.powder(spin_system, 'acquire', dict(base, needs=['zeeman_op']), 'nmr')
    with pytest.raises(ValueError):                      # offsets and spins of different lengths
        X.powder(spin_system, 'acquire', dict(base, spins=['13C', '1H'], offset=[1.0]), 'nmr')
    with pytest.raises(ValueError):                      # two offsets for one isotope
        X.powder(spin_system, 'acquire', dict(base, spins=['13C', '13C'], offset=[1.0, 2.0]), 'nmr')
    with pytest.raises(ValueError):                      # no temperature for the equilibrium
        X.powder(spin_system, 'acquire', dict({k: v for k, v in base.items() if k != 'rho0'}, needs=['iso_eq']),
                 'nmr')
    with pytest.raises(ValueError):
        X.create(dict(isotopes=['1H'], magnet=1.0), dict(relaxation=['redfield']))


def test_equilibrium_states_match_oracle():
    sys_, inter, spin_system = _system(temperature=300.0)
    HL = S.rotational_hamiltonian(spin_system.ss, spin_system.basis, 'labframe', spin_system.factory(), kind='left')
    angs = np.array([[0.1, 0.5, 0.9], [0.0, 2.0, -1.0], [1.2, 0.3, 0.4]])
    st = S.equilibrium_states(HL, 300.0, angs[:, 0], angs[:, 1], angs[:, 2])
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(approximation='none', level=0, space_level=1))
    ssL = R.assume(copy.deepcopy(ss), 'labframe')
    IL, QL = R.hamiltonian(ssL, 'left')
    for i, a in enumerate(angs):
        ref = R.equilibrium(ssL, IL, QL, tuple(a))
        dev = ref - np.eye(1, ref.size)[0]
        assert np.abs(st[i] - ref).max() <= 1e-12 * np.abs(dev).max()
    iso = S.equilibrium_states(S.RotationalHamiltonian(HL.dim, HL.iso, {}), 300.0)
    assert iso.shape == (HL.dim,) and iso[0] == 1.0


class _DenseEngine:
    """Exact dense stand-in for the engine's run semantics, used to check the
    host side of the contexts on CPU: L(Omega) = Herm(I + sum D(Omega)(j,m)
    Q{r}{j,m}) + iR propagated with expm, pulses exp(-1i*angle*P), a segment
    of n steps records n+1 points unless record is False."""

    class _Res:
        def __init__(self, fids, w):
            self.fids = np.array(fids)
            self.fid = (np.asarray(w)[:, None] * self.fids).sum(axis=0)

    def upload(self, I, terms, Rx, rho0, coil):
        self.sys = (I, terms, Rx, np.asarray(rho0, complex), np.asarray(coil, complex))

    def _L(self, a, b, g):
        from spinach_gb300 import singlerot as SR
        I, terms, Rx, _, _ = self.sys
        H = I.toarray().astype(complex)
        D = {r: SR.wigner_d(r, a, b, g) for r in {k[0] for k in terms}}
        for (r, j, m), T in terms.items():
            H = H + D[r][j, m] * T.toarray()
        L = (H + H.conj().T) / 2
        return L if Rx is None else L + 1j * Rx.toarray()

    def _program(self, al, be, ga, w, ops, prog):
        from scipy.linalg import expm
        _, _, _, rho0, coil = self.sys
        fids = []
        for a, b, g in zip(al, be, ga):
            L, rho, out = self._L(a, b, g), rho0.copy(), []
            for item in prog:
                if item[0] == 'pulse':
                    rho = expm(-1j * item[2] * ops[item[1]].toarray()) @ rho
                    continue
                n, dt, record = item[1], item[2], (item[3] if len(item) > 3 else True)
                P = expm(-1j * L * dt)
                if record:
                    out.append(np.vdot(coil, rho))
                for _ in range(n):
                    rho = P @ rho
                    if record:
                        out.append(np.vdot(coil, rho))
            fids.append(out)
        return self._Res(fids, w)

    def run(self, al, be, ga, w, dt, nsteps, precision=None, per_orientation=False):
        return self._program(al, be, ga, w, [], [('evolve', nsteps, dt)])

    def run_sequence(self, al, be, ga, w, ops, prog, precision=None, per_orientation=False):
        return self._program(al, be, ga, w, ops, prog)

    def run_cpmg(self, al, be, ga, w, dt, npoints, nloops, P, precision=None, per_orientation=False):
        prog = [('pulse', 0, np.pi / 2), ('evolve', npoints - 1, dt)]
        for _ in range(nloops):
            prog += [('pulse', 0, np.pi), ('evolve', 2 * npoints - 1, dt)]
        return self._program(al, be, ga, w, [P], prog)

    def run_deer(self, al, be, ga, w, stepsize, nsteps, ex_prob, ex_pump, precision=None, per_orientation=False):
        from scipy.linalg import expm
        _, _, _, rho0, coil = self.sys
        fids = []
        for a, b, g in zip(al, be, ga):
            U = expm(-1j * self._L(a, b, g) * stepsize)
            Pp, Pu = expm(-1j * np.pi * ex_prob.toarray()), expm(-1j * np.pi * ex_pump.toarray())
            r = expm(-1j * np.pi / 2 * ex_prob.toarray()) @ rho0
            out = []
            for j in range(nsteps + 1):
                x = np.linalg.matrix_power(U, nsteps) @ Pp @ np.linalg.matrix_power(U, nsteps - j) @ Pu @ r
                out.append(np.vdot(coil, x) / np.linalg.norm(coil))
                r = U @ r
            fids.append(out)
        return self._Res(fids, w)

    def set_initial_states(self, states):
        if states is not None:
            raise NotImplementedError('per-orientation states are not modelled here')

    def close(self):
        pass


@pytest.mark.parametrize('context,sequence', [('singlerot', 'hp_acquire'), ('floquet', 'cpmg'),
                                              ('singlerot', 'cpmg'), ('floquet', 'hp_acquire')])
def test_mas_contexts_project_pulses_into_rotor_space(context, sequence):
    """singlerot.m / floquet.m with @hp_acquire and @cpmg: the pulses act on
    every rotor point or Fourier component, kron(speye(spc_dim), op)
    (hp_acquire.m:57,69, cpmg.m:33); the context's uploaded system and
    programs, run exactly, against the oracle."""
    sys_, inter, spin_system = _system()
    al, be, ga = np.array([0.0, 0.0, 0.0]), np.array([0.4, 1.3, 2.5]), np.array([0.3, 2.0, 4.1])
    w = np.array([0.2, 0.5, 0.3])
    base = dict(rate=8e3, axis=(1, 1, 1), max_rank=2, grid=(al, be, ga, w))
    if sequence == 'hp_acquire':
        seq = dict(pulse_op=('Ly', '13C'), pulse_angle=np.pi / 2, echo_time=3e-5, echo_oper=('Lx', '13C'),
                   echo_angle=np.pi, sweep=2e4, npoints=12)
    else:
        seq = dict(pulse_op=('Ly', '13C'), timestep=5e-5, npoints=6, nloops=2)
    parameters = dict(base, rho0=('Lz', '13C'), coil=('L+', '13C'), **seq)
    fid, _ = getattr(X, context)(spin_system, sequence, parameters, 'nmr', engine=_DenseEngine())
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(approximation='none', level=0, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(base, rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, 'L+', '13C'))
    for k in ('pulse_op', 'echo_oper'):
        if k in seq:
            par[k] = R.operator(ss, seq[k][0], seq[k][1])
    par.update({k: v for k, v in seq.items() if k not in ('pulse_op', 'echo_oper')})
    one = R.singlerot_orientation_fid if context == 'singlerot' else R.floquet_orientation_fid
    ref = sum(w[i] * one(ss, I, Q, par, (al[i], be[i], ga[i]), sequence=sequence) for i in range(3))
    assert np.abs(ref).max() > 0.05
    assert np.abs(fid - ref).max() <= 1e-9 * np.abs(ref).max()


def test_powder_deer_context_matches_oracle():
    """powder(..., @deer_3p_hard_deer, ...): the probe coil is the detection
    state and the answer is the 'brief' DEER trace."""
    sys_, inter, spin_system = _system()
    g = (np.zeros(3), np.array([0.4, 1.3, 2.5]), np.array([0.3, 2.0, 4.1]), np.array([0.2, 0.5, 0.3]))
    parameters = dict(grid=g, rho0=('Lz', '13C'), coil_prob=('L+', '13C'), ex_prob=('Ly', '13C'),
                      ex_pump=('Ly', '1H'), stepsize=2e-4, nsteps=10, output='brief')
    trace, _ = X.powder(spin_system, 'deer_3p_hard_deer', parameters, 'nmr', engine=_DenseEngine())
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(approximation='none', level=0, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil_prob=R.state(ss, 'L+', '13C'),
               ex_prob=R.operator(ss, 'Ly', '13C'), ex_pump=R.operator(ss, 'Ly', '1H'), stepsize=2e-4, nsteps=10)
    ref = sum(g[3][i] * R.powder_orientation_deer(ss, I, Q, par, (g[0][i], g[1][i], g[2][i])) for i in range(3))
    assert np.abs(ref).max() > 0.05
    assert np.abs(trace - ref).max() <= 1e-9 * np.abs(ref).max()
    with pytest.raises(ValueError):
        X.powder(spin_system, 'deer_3p_hard_deer', dict(parameters, output='detailed'), 'nmr',
                 engine=_DenseEngine())


def test_powder_deer_echo_context_matches_oracle():
    """powder(..., @deer_3p_hard_echo, ...) as a pulse program (three hard
    pulses, three silent delays, the echo over tc) against the oracle."""
    sys_, inter, spin_system = _system()
    g = (np.zeros(3), np.array([0.4, 1.3, 2.5]), np.array([0.3, 2.0, 4.1]), np.array([0.2, 0.5, 0.3]))
    times = dict(ta=6e-4, tb=2e-4, tc=4e-4, nsteps=16)
    parameters = dict(grid=g, rho0=('Lz', '13C'), coil=('L+', '13C'), ex_prob=('Ly', '13C'), ex_pump=('Ly', '1H'),
                      **times)
    echo, _ = X.powder(spin_system, 'deer_3p_hard_echo', parameters, 'nmr', engine=_DenseEngine())
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(approximation='none', level=0, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, 'L+', '13C'), ex_prob=R.operator(ss, 'Ly', '13C'),
               ex_pump=R.operator(ss, 'Ly', '1H'), **times)
    ref = sum(g[3][i] * R.powder_orientation_sequence(ss, I, Q, par, (g[0][i], g[1][i], g[2][i]),
                                                      R.deer_3p_hard_echo) for i in range(3))
    assert echo.shape == (17,) and np.abs(ref).max() > 0.05
    assert np.abs(echo - ref).max() <= 1e-9 * np.abs(ref).max()


def test_powder_single_crystal_matches_crystal():
    """tests/kernel/test_ctx_powder_crystal.m: powder() on the single_crystal
    grid equals crystal() at zero Euler angles (1e-12), and the oracle."""
    sys_ = dict(isotopes=['1H'], magnet=14.1)
    inter = dict(zeeman=dict(eigs=[[-2.0, -2.0, 4.0]], euler=[[0.0, 0.0, 0.0]]))
    bas = dict(approximation='none', projections=[1])
    spin_system = X.basis(X.create(sys_, inter), bas)
    rho = X.state(spin_system, 'L+', '1H')
    parameters = dict(spins=['1H'], rho0=rho, coil=rho, decouple=[], offset=[0.0], sweep=2000.0, npoints=4,
                      grid='single_crystal', orientation=[0.0, 0.0, 0.0])
    fid_powder, g = X.powder(spin_system, 'acquire', parameters, 'nmr', engine=_DenseEngine())
    fid_crystal = X.crystal(spin_system, 'acquire', parameters, 'nmr', engine=_DenseEngine())
    assert g[3].tolist() == [1.0] and np.abs(fid_powder - fid_crystal).max() <= 1e-12
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(bas, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(rho0=R.state(ss, 'L+', '1H'), coil=R.state(ss, 'L+', '1H'), sweep=2000.0, npoints=4)
    assert np.abs(fid_crystal - R.powder_orientation_fid(ss, I, Q, par, (0.0, 0.0, 0.0))).max() <= 1e-12
    # another orientation through crystal() against the oracle
    ang = [0.3, 1.1, -0.4]
    f = X.crystal(spin_system, 'acquire', dict(parameters, orientation=ang), 'nmr', engine=_DenseEngine())
    assert np.abs(f - R.powder_orientation_fid(ss, I, Q, par, tuple(ang))).max() <= 1e-12
    with pytest.raises(ValueError):                      # crystal.m: a row vector with three numbers
        X.crystal(spin_system, 'acquire', dict(parameters, orientation=[0.0, 0.0]), 'nmr', engine=_DenseEngine())


def test_powder_inv_rec_context_matches_oracle():
    """powder(..., @inv_rec, ...): the isotropic equilibrium, a 180-degree
    pulse, n_delays+1 recovery times, a 90-degree pulse and one FID each
    (npoints x (n_delays+1)), as one pulse program per delay."""
    sys_, inter, _ = _system(temperature=300.0)
    inter = dict(inter, relaxation=['damp'], damp_rate=3.0)       # damping: a recovery to see
    spin_system = X.basis(X.create(sys_, inter), dict(approximation='none'))
    g = (np.zeros(2), np.array([0.4, 1.3]), np.array([0.3, 2.0]), np.array([0.4, 0.6]))
    parameters = dict(grid=g, spins=['13C'], n_delays=3, max_delay=0.3, sweep=2e3, npoints=8)
    fids, _ = X.powder(spin_system, 'inv_rec', parameters, 'nmr', engine=_DenseEngine())
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(approximation='none', level=0, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    ref = sum(g[3][i] * R.powder_orientation_sequence(ss, I, Q, parameters, (g[0][i], g[1][i], g[2][i]), R.inv_rec)
              for i in range(2))
    # 13C thermal polarisation at 14.1 T and 300 K is of order 1e-5; the
    # first point changes with the recovery delay
    assert fids.shape == (8, 4) and np.abs(ref).max() > 1e-6
    assert abs(ref[0, 0] - ref[0, -1]) > 0.1 * np.abs(ref).max()
    assert np.abs(fids - ref).max() <= 1e-9 * np.abs(ref).max()
    # sum_up = 0: one npoints x (n_delays+1) answer per orientation
    cells, _ = X.powder(spin_system, 'inv_rec', dict(parameters, sum_up=0), 'nmr', engine=_DenseEngine())
    assert len(cells) == 2 and all(c.shape == (8, 4) for c in cells)
    assert np.abs(g[3][0] * cells[0] + g[3][1] * cells[1] - fids).max() <= 1e-12 * np.abs(fids).max()
    with pytest.raises(ValueError):
        X.powder(spin_system, 'inv_rec', dict(parameters, rho0=('Lz', '13C')), 'nmr', engine=_DenseEngine())
