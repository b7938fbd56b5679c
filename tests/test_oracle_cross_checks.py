"""Oracle vs an independent Zeeman-basis model, and the product-side
spin-system builder vs the oracle's literal restatement."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import spinach_ref as R
from oracle.kron_model import KronModel
from oracle_cases import oracle_system, rel_err
from spinach_gb300 import spin_system as S, workloads as W


def _c0_like(relax):
    w = W.c0()
    if relax:
        rng = np.random.default_rng(11)
        w.r1 = list(rng.uniform(1, 50, 3))
        w.r2 = list(rng.uniform(100, 900, 3))
    return w


@pytest.mark.parametrize('relax', [False, True])
def test_full_basis_fid_matches_kron_model(relax):
    """Basis-invariance: full spherical-tensor basis vs Zeeman Liouville space."""
    w = _c0_like(relax)
    ss, I, Q = oracle_system(w)
    km = KronModel(ss)
    rho_st, coil_st = R.state(ss, *w.rho0), R.state(ss, *w.coil)
    # state(...,'exact') is the Hilbert operator applied to the unit state E/sqrt(d)
    rho_h = km.spin_op(*w.rho0) / np.sqrt(km.dim)
    coil_h = km.spin_op(*w.coil) / np.sqrt(km.dim)
    assert abs(np.vdot(coil_st, rho_st) - np.vdot(coil_h.ravel(), rho_h.ravel())) < 1e-14
    par = dict(rho0=rho_st, coil=coil_st, sweep=1 / w.dt, npoints=129)
    for ang in [(0.0, 0.7, 1.3), (0.0, 2.1, 5.0), (0.4, 1.0, -0.3)]:
        f_st = R.powder_orientation_fid(ss, I, Q, par, ang)
        f_kr = km.fid(ang, rho_h, coil_h, w.dt, 128)
        # both models form rotating-frame offsets as differences of ~4e9 rad/s
        # lab-frame numbers: 1e-16 * 4e9 rad/s * 1.3 ms is ~5e-10 of phase
        assert rel_err(f_st, f_kr) < 1e-8, ang


@pytest.mark.parametrize('wl', ['c0', 'c4', 'deuterium'])
def test_builder_matches_oracle_operators(wl):
    w = getattr(W, wl)()
    if wl == 'c4':            # keep the CPU suite fast: electron, 14N, three protons
        w.isotopes = w.isotopes[:5]
        w.zeeman_eigs, w.zeeman_euler = w.zeeman_eigs[:5], w.zeeman_euler[:5]
        w.coupling_eigs = {k: v for k, v in w.coupling_eigs.items() if max(k) < 5}
        w.r1, w.r2 = w.r1[:5], w.r2[:5]
    ss, I, Q = oracle_system(w)
    L = W.build(w)
    assert L.dim == ss.basis.shape[0]
    scale = max(abs(I).max(), max(abs(q).max() for r in Q for row in Q[r] for q in row if q.nnz))
    assert abs(L.I - I).max() <= 1e-14 * scale
    for r in Q:
        for k in range(2 * r + 1):
            for m in range(2 * r + 1):
                ref = Q[r][k][m]
                got = L.terms.get((r, k, m))
                if got is None:
                    assert ref.nnz == 0 or abs(ref).max() <= 1e-14 * scale
                else:
                    assert abs(got - ref).max() <= 1e-14 * scale
    assert np.abs(L.rho0 - R.state(ss, *w.rho0)).max() < 1e-15
    assert np.abs(L.coil - R.state(ss, *w.coil)).max() < 1e-15
    assert np.abs(L.R.diagonal() - R.relaxation(ss).diagonal()).max() < 1e-12


def test_builder_matches_oracle_c1_basis():
    w = W.c1()
    ss, I, Q = oracle_system(w)
    L = W.build(w)
    assert L.dim == 1156 == ss.basis.shape[0]
    assert abs(L.I - I).max() <= 1e-14 * abs(I).max()
    for (r, k, m), q in L.terms.items():
        assert abs(q - Q[r][k][m]).max() <= 1e-14 * abs(Q[r][k][m]).max()


def test_ik1_basis_dimension_of_epr_radical():
    """IK-1 level 3 on the electron-centred coupling graph of e + 14N + 10 1H."""
    w = W.c4()
    ss = W.spin_system_of(w)
    b = S.build_basis(ss, 'IK-1', 3)
    assert b.dim == 2736
    ss_o = R.create(dict(isotopes=w.isotopes, magnet=w.magnet),
                    dict(zeeman=dict(eigs=w.zeeman_eigs, euler=w.zeeman_euler),
                         coupling=dict(eigs=w.coupling_eigs, euler=w.coupling_euler)))
    ss_o = R.basis(ss_o, dict(approximation='IK-1', level=3, space_level=1))
    assert np.array_equal(ss_o.basis, b.codes)


@pytest.mark.parametrize('relax', [False, True])
def test_cpmg_matches_kron_model(relax):
    """experiments/cpmg.m restated on the spherical-tensor basis vs the same
    pulse sequence with Hilbert-space pulses U rho U^dagger."""
    w = _c0_like(relax)
    ss, I, Q = oracle_system(w)
    km = KronModel(ss)
    rho_h = km.spin_op('Lz', '13C') / np.sqrt(km.dim)
    coil_h = km.spin_op(*w.coil) / np.sqrt(km.dim)
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, *w.coil), pulse_op=R.operator(ss, 'Ly', '13C'),
               timestep=w.dt, npoints=20, nloops=3)
    for ang in [(0.0, 0.7, 1.3), (0.4, 1.0, -0.3)]:
        f_st = R.powder_orientation_cpmg(ss, I, Q, par, ang)
        f_kr = km.cpmg(ang, rho_h, coil_h, km.spin_op('Ly', '13C'), w.dt, 20, 3)
        assert f_st.shape == (20 * 7,)
        assert np.abs(f_kr).max() > 0.1
        assert rel_err(f_st, f_kr) < 1e-8, ang


def test_cpmg_with_a_zero_pulse_is_one_continuous_acquisition():
    """Each echo starts from the last state of the previous segment: with no
    pulse the segments tile one acquisition, the joints counted twice."""
    w = W.c0()
    ss, I, Q = oracle_system(w)
    zero = 0 * R.operator(ss, 'Ly', '13C')
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), pulse_op=zero, timestep=w.dt,
               npoints=10, nloops=2)
    ang = (0.0, 1.1, 0.5)
    f = R.powder_orientation_cpmg(ss, I, Q, par, ang)
    acq = R.powder_orientation_fid(ss, I, Q, dict(rho0=par['rho0'], coil=par['coil'], sweep=1 / w.dt,
                                                  npoints=10 + 2 * 19), ang)
    idx = list(range(10)) + list(range(9, 29)) + list(range(28, 48))
    assert rel_err(f, acq[idx]) < 1e-12


@pytest.mark.parametrize('relax', [False, True])
def test_eseem_matches_kron_model(relax):
    """experiments/esr_dipolar/eseem.m restated on the spherical-tensor basis
    (trajectory, stacked pulse, refocusing) vs Hilbert-space pulses."""
    w = _c0_like(relax)
    ss, I, Q = oracle_system(w)
    km = KronModel(ss)
    rho_h = km.spin_op('Lz', '13C') / np.sqrt(km.dim)
    coil_h = km.spin_op(*w.coil) / np.sqrt(km.dim)
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, *w.coil), pulse_op=R.operator(ss, 'Ly', '13C'),
               timestep=2 * w.dt, npoints=24)
    for ang in [(0.0, 0.7, 1.3), (0.4, 1.0, -0.3)]:
        f_st = R.powder_orientation_eseem(ss, I, Q, par, ang)
        f_kr = km.eseem(ang, rho_h, coil_h, km.spin_op('Ly', '13C'), 2 * w.dt, 24)
        assert f_st.shape == (24,)
        assert np.abs(f_kr).max() > 0.1
        assert rel_err(f_st, f_kr) < 1e-8, ang


@pytest.mark.parametrize('relax', [False, True])
def test_deer_matches_kron_model(relax):
    """experiments/esr_dipolar/deer_3p_hard_deer.m restated on the
    spherical-tensor basis (trajectory, stacked pump pulse, reversed
    refocusing, probe pulse, 'final' evolution) vs Hilbert-space pulses, the
    probe on 13C and the pump on the protons."""
    w = _c0_like(relax)
    ss, I, Q = oracle_system(w)
    km = KronModel(ss)
    rho_h = km.spin_op('Lz', '13C') / np.sqrt(km.dim)
    coil_h = km.spin_op('L+', '13C') / np.sqrt(km.dim)
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil_prob=R.state(ss, 'L+', '13C'),
               ex_prob=R.operator(ss, 'Ly', '13C'), ex_pump=R.operator(ss, 'Ly', '1H'), stepsize=w.dt, nsteps=20)
    for ang in [(0.0, 0.7, 1.3), (0.4, 1.0, -0.3)]:
        f_st = R.powder_orientation_deer(ss, I, Q, par, ang) * np.linalg.norm(par['coil_prob'])
        f_kr = km.deer_3p(ang, rho_h, coil_h, km.spin_op('Ly', '13C'), km.spin_op('Ly', '1H'), w.dt, 20)
        assert f_st.shape == (21,)
        assert np.abs(f_kr).max() > 0.05
        assert rel_err(f_st, f_kr) < 1e-8, ang


def test_oopeseem_matches_kron_model():
    """experiments/esr_dipolar/oopeseem.m (the 45-degree first pulse)
    restated on the spherical-tensor basis vs Hilbert-space pulses."""
    w = _c0_like(True)
    ss, I, Q = oracle_system(w)
    km = KronModel(ss)
    rho_h = km.spin_op('Lz', '13C') / np.sqrt(km.dim)
    coil_h = km.spin_op(*w.coil) / np.sqrt(km.dim)
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, *w.coil), pulse_op=R.operator(ss, 'Ly', '13C'),
               timestep=2 * w.dt, npoints=24)
    ang = (0.4, 1.0, -0.3)
    f_st = R.powder_orientation_sequence(ss, I, Q, par, ang, R.oopeseem)
    f_kr = km.eseem(ang, rho_h, coil_h, km.spin_op('Ly', '13C'), 2 * w.dt, 24, first_angle=np.pi / 4)
    assert np.abs(f_kr).max() > 0.05
    assert rel_err(f_st, f_kr) < 1e-8
    # not the in-phase echo
    assert rel_err(f_st, R.powder_orientation_eseem(ss, I, Q, par, ang)) > 0.1


def test_quadratic_coupling_matches_kron_model():
    """The 2H quadratic coupling (hamiltonian.m:191-257, T(2,0) under 'nmr')
    against L.A.L's secular part (A_zz/2)(3Lz^2 - L^2) in Hilbert space."""
    w = W.deuterium()
    ss, I, Q = oracle_system(w)
    km = KronModel(ss)
    rho_h = km.spin_op('Lx', '2H') / np.sqrt(km.dim)
    coil_h = km.spin_op('L+', '2H') / np.sqrt(km.dim)
    par = dict(rho0=R.state(ss, 'Lx', '2H'), coil=R.state(ss, 'L+', '2H'), sweep=1 / w.dt, npoints=129)
    for ang in [(0.0, 0.7, 1.3), (0.4, 1.0, -0.3), (0.0, 2.5, 4.0)]:
        f_st = R.powder_orientation_fid(ss, I, Q, par, ang)
        f_kr = km.fid(ang, rho_h, coil_h, w.dt, 128)
        assert rel_err(f_st, f_kr) < 1e-9, ang


def test_quadratic_coupling_rules():
    from spinach_gb300 import spin_system as S
    with pytest.raises(ValueError):                      # spin-1/2 has no rank-2 operators
        S.make_spin_system(['1H', '13C'], 14.1, coupling_eigs={(0, 0): [-1e3, -1e3, 2e3]})
    ss = S.make_spin_system(['2H'], 14.1, coupling_eigs={(0, 0): [-1e4, -1e4, 3e4]})   # not traceless
    with pytest.raises(ValueError):
        S.interaction_terms(ss, 'nmr')


def test_strong_quadratic_coupling_matches_hilbert_space():
    """'esr' assumptions keep the whole quadratic coupling of a nucleus
    (hamiltonian.m:216-229, five T(2,m)) and its full Zeeman interaction: one
    14N against H = L.Z.e_z + L.A.L built from spin matrices."""
    import scipy.linalg as sla
    from oracle.kron_model import KronModel
    sys_ = dict(isotopes=['14N'], magnet=0.34, enable=[])
    A = 2 * np.pi * np.array([[-0.4e6, 0.1e6, 0.05e6], [0.1e6, -0.6e6, 0.2e6], [0.05e6, 0.2e6, 1.0e6]])
    evals, evecs = np.linalg.eigh(A / (2 * np.pi))
    inter = dict(zeeman=dict(eigs=[[10.0, 20.0, 40.0]], euler=[[0.1, 0.2, 0.3]]),
                 coupling=dict(eigs={(0, 0): list(evals)}))
    ss = R.create(sys_, inter)
    # put the coupling in as the full matrix (create.m adds 2*pi*S*diag(eigs)*S')
    ss.coupling[(0, 0)] = A
    ss = R.basis(ss, dict(approximation='none', level=0, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'esr')
    km = KronModel(ss)
    Lx, Ly, Lz = (km.ops[0][k] for k in ('x', 'y', 'z'))
    Lv = [Lx, Ly, Lz]
    rho = R.state(ss, 'Lx', '14N')
    coil = R.state(ss, 'L+', '14N')
    rho_h = km.spin_op('Lx', '14N') / np.sqrt(km.dim)
    coil_h = km.spin_op('L+', '14N') / np.sqrt(km.dim)
    dt, n = 2e-8, 96
    par = dict(rho0=rho, coil=coil, sweep=1 / dt, npoints=n + 1)
    for ang in [(0.0, 0.0, 0.0), (0.3, 1.1, -0.7)]:
        Rm = R.euler2dcm(*ang)
        Z = Rm @ ss.zeeman[0] @ Rm.T
        Ar = Rm @ A @ Rm.T
        H = sum(Z[i, 2] * Lv[i] for i in range(3)) + sum(Ar[i, j] * Lv[i] @ Lv[j] for i in range(3) for j in range(3))
        Lh = np.kron(H, np.eye(3)) - np.kron(np.eye(3), H.T)
        P = sla.expm(-1j * dt * Lh)
        r = rho_h.reshape(-1).astype(complex)
        f_h = []
        for _ in range(n + 1):
            f_h.append(np.vdot(coil_h.reshape(-1), r))
            r = P @ r
        f_st = R.powder_orientation_fid(ss, I, Q, par, ang)
        assert rel_err(f_st, np.array(f_h)) < 1e-9, ang


def test_frequency_offsets_match_oracle():
    """powder.m:157 frqoffset (kernel/frqoffset.m): 2*pi*offset*Lz per isotope."""
    import copy
    w = copy.deepcopy(W.c0())
    w.extra['offset'] = {'13C': 1500.0, '1H': -300.0}
    ss, I, Q = oracle_system(w)
    L = W.build(w)
    assert abs(L.I - I).max() <= 1e-14 * abs(I).max()
    w0 = W.c0()
    assert abs(W.build(w0).I - L.I).max() > 1e3             # the offsets are there
    with pytest.raises(ValueError):
        R.frqoffset(ss, I, ['13C', '13C'], [1.0, 2.0])
    with pytest.raises(ValueError):
        R.frqoffset(ss, I, ['15N'], [1.0])


def test_isotropic_damping_matches_oracle():
    """relaxation.m 'damp' (isotropic): every state but the unit state decays
    at damp_rate, on top of T1/T2."""
    import copy
    w = copy.deepcopy(W.c0())
    rng = np.random.default_rng(4)
    w.r1, w.r2 = list(rng.uniform(1, 5, 3)), list(rng.uniform(5, 20, 3))
    w.extra['damp_rate'] = 37.0
    ss, I, Q = oracle_system(w)
    L = W.build(w)
    Ro = R.relaxation(ss)
    assert abs(Ro - sp.diags(Ro.diagonal())).max() == 0
    assert np.abs(L.R.diagonal() - Ro.diagonal()).max() <= 1e-12
    assert L.R.diagonal()[0] == 0 and abs(Ro.diagonal()[0]) == 0


def _dense_fid(L, g, dt, nsteps):
    """FID of the product-built system at one orientation by dense expm."""
    import scipy.linalg as sla
    from spinach_gb300 import singlerot as SRt
    H = L.I.toarray().astype(complex)
    for (r, k, m), Qm in L.terms.items():
        H = H + SRt.wigner_d(r, *g)[k, m] * Qm.toarray()
    H = (H + H.conj().T) / 2
    P = sla.expm(-1j * dt * (H + 1j * L.R.toarray()))
    rho, out = L.rho0.copy(), []
    for _ in range(nsteps + 1):
        out.append(np.vdot(L.coil, rho))
        rho = P @ rho
    return np.array(out)


def test_decoupling_as_a_smaller_basis_matches_the_masked_liouvillian():
    """acquire.m:51 / decouple.m zero the rows and columns of the states in
    which a decoupled spin is active; the builder drops those states."""
    import copy
    w = copy.deepcopy(W.c0())
    w.extra['decouple'] = ['1H']
    ss, I, Q = oracle_system(w)
    L = W.build(w)
    assert L.dim == 4 and ss.basis.shape[0] == 64            # 13C alone survives
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=65,
               decouple=['1H'])
    for ang in [(0.0, 0.7, 1.3), (0.2, 2.0, -1.0)]:
        assert rel_err(_dense_fid(L, ang, w.dt, 64), R.powder_orientation_fid(ss, I, Q, par, ang)) < 1e-12


def test_homodecoupling_matches_oracle():
    import copy
    w = copy.deepcopy(W.c0())
    w.extra['homodec'] = ('Lx', '1H', 2500.0)
    ss, I, Q = oracle_system(w)
    L = W.build(w)
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=65,
               homodec_oper=R.operator(ss, 'Lx', '1H'), homodec_pwr=2500.0)
    ang = (0.0, 1.1, 0.4)
    assert rel_err(_dense_fid(L, ang, w.dt, 64), R.powder_orientation_fid(ss, I, Q, par, ang)) < 1e-10


@pytest.mark.parametrize('approx', ['IK-0', 'IK-1'])
def test_restricted_basis_at_full_level_is_the_full_basis(approx):
    """basis.m:186-269: an IK-0 or IK-1 basis whose correlation level equals
    the spin count keeps every product state, so the restricted-basis
    machinery (oracle and product builder alike) must return the full basis,
    and the FIDs computed in it must match the independent Zeeman-basis model
    (oracle/kron_model.py) -- the check that pins the IK code paths of c1, c2
    and c4 on a system small enough for the model."""
    w = _c0_like(True)
    w.approximation, w.level = approx, len(w.isotopes)
    ss, I, Q = oracle_system(w)
    assert ss.basis.shape[0] == 4 ** len(w.isotopes)
    full = _c0_like(True)
    ssf, _, _ = oracle_system(full)
    assert sorted(map(tuple, ss.basis.tolist())) == sorted(map(tuple, ssf.basis.tolist()))
    L = W.build(w)
    pss = W.spin_system_of(w)
    pb = S.build_basis(pss, w.approximation, w.level)
    assert pb.dim == 4 ** len(w.isotopes)
    assert sorted(map(tuple, pb.codes.tolist())) == sorted(map(tuple, ss.basis.tolist()))
    km = KronModel(ss)
    rho_h = km.spin_op(*w.rho0) / np.sqrt(km.dim)
    coil_h = km.spin_op(*w.coil) / np.sqrt(km.dim)
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=129)
    for ang in [(0.0, 0.7, 1.3), (0.4, 1.9, -0.3)]:
        f_st = R.powder_orientation_fid(ss, I, Q, par, ang)
        f_kr = km.fid(ang, rho_h, coil_h, w.dt, 128)
        assert rel_err(f_st, f_kr) < 1e-8, ang
    assert L.dim == ss.basis.shape[0]
