"""Pin the oracle against the closed-form expectations of the reference's own tests.

Each test names the reference test (tests/kernel/*.m in the Spinach tree) whose
expectation it restates; tolerances are the reference's.
"""
import math

import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp

from oracle import spinach_ref as R


def close(obs, ref, abs_tol, rel_tol):
    """tests/lib/test_close.m:27-71: ||obs-ref||_2 <= abs_tol + rel_tol*max(1,||ref||_2)."""
    obs = np.asarray(obs.toarray() if sp.issparse(obs) else obs).ravel()
    ref = np.asarray(ref.toarray() if sp.issparse(ref) else ref).ravel()
    assert np.all(np.isfinite(obs)) and np.all(np.isfinite(ref))
    err = np.linalg.norm(obs - ref)
    assert err <= abs_tol + rel_tol * max(1.0, np.linalg.norm(ref)), err


def one_spin(tol='default', **inter):
    ss = R.create(dict(isotopes=['1H'], magnet=14.1), inter, tol)
    return R.basis(ss, dict(approximation='none'))


# test_wigner_angular_suite.m:44-53
def test_wigner_rank1_beta_half_pi():
    ref = np.array([[0.5, -1 / math.sqrt(2), 0.5], [1 / math.sqrt(2), 0, -1 / math.sqrt(2)],
                    [0.5, 1 / math.sqrt(2), 0.5]])
    close(R.wigner(1, 0, math.pi / 2, 0), ref, 1e-14, 1e-14)


def test_wigner_identity_and_unitarity():
    close(R.wigner(2, 0, 0, 0), np.eye(5), 1e-14, 1e-14)
    D = R.wigner(2, 0.2, 0.4, 0.7)
    close(D.conj().T @ D, np.eye(5), 1e-13, 1e-13)


def test_wigner_closed_forms_match_generic_route():
    """wigner.m:79-86: expm route for general ranks must agree with the closed forms."""
    for l in (1, 2):
        Lp = R.pauli(2 * l + 1)
        a, b, g = 0.3, 1.1, -0.7
        gen = sla.expm(-1j * Lp['z'] * a) @ sla.expm(-1j * Lp['y'] * b) @ sla.expm(-1j * Lp['z'] * g)
        close(R.wigner(l, a, b, g), gen, 1e-13, 1e-13)


# cache/ist_product_table.m:40-81 (hard-coded spin-1/2 tables)
SPIN_HALF_LEFT = {
    0: [[1, 0, 0, 0], [0, 0, 0, -0.5], [0, 0, 0.5, 0], [0, -0.5, 0, 0]],
    1: [[0, 1, 0, 0], [0.5, 0, -0.5, 0], [0, 0.5, 0, 0], [0, 0, 0, 0]],
    2: [[0, 0, 1, 0], [0, 0, 0, -0.5], [0.5, 0, 0, 0], [0, 0.5, 0, 0]],
    3: [[0, 0, 0, 1], [0, 0, 0, 0], [0, 0, 0, -0.5], [0.5, 0, 0.5, 0]],
}
SPIN_HALF_RIGHT = {
    0: [[1, 0, 0, 0], [0, 0, 0, -0.5], [0, 0, 0.5, 0], [0, -0.5, 0, 0]],
    1: [[0, 1, 0, 0], [0.5, 0, 0.5, 0], [0, -0.5, 0, 0], [0, 0, 0, 0]],
    2: [[0, 0, 1, 0], [0, 0, 0, 0.5], [0.5, 0, 0, 0], [0, -0.5, 0, 0]],
    3: [[0, 0, 0, 1], [0, 0, 0, 0], [0, 0, 0, 0.5], [0.5, 0, -0.5, 0]],
}


def test_computed_product_table_matches_hard_coded_spin_half():
    left, right = R.ist_product_table(2)
    for k in range(4):
        close(left[:, :, k], np.array(SPIN_HALF_LEFT[k]), 1e-15, 1e-15)
        close(right[:, :, k], np.array(SPIN_HALF_RIGHT[k]), 1e-15, 1e-15)


def test_product_table_reproduces_matrix_products_spin_one():
    """Table entries for mult=3 reproduce T_n T_m in the normalised IST basis."""
    T = R.irr_sph_ten(3)
    E = [t / math.sqrt(R.hdot(t, t).real) for t in T]
    left, _ = R.ist_product_table(3)
    for n in (1, 2, 5):
        for m in (0, 3, 7):
            recon = sum(left[n, m, k] * E[k] for k in range(9))
            close(recon, T[n] @ E[m], 1e-13, 1e-13)


# test_liouville_commutator.m:33-38 (restated in the spherical-tensor basis)
def test_commutator_is_left_minus_right():
    ss = one_spin(zeeman=dict(scalar=[0.0]))
    comm = R.operator(ss, 'Lz', 0, 'comm')
    left = R.operator(ss, 'Lz', 0, 'left')
    right = R.operator(ss, 'Lz', 0, 'right')
    close(comm, left - right, 1e-15, 1e-15)


# test_zeeman_hamiltonian.m:33-38 (Liouville-space form)
def test_zeeman_offset_sign_and_units():
    ss = one_spin(zeeman=dict(scalar=[1.0]))
    ss = R.assume(ss, 'nmr')
    I, _ = R.hamiltonian(ss)
    nu = 1e-6 * R.ISOTOPES['1H'][1] * 14.1 / (2 * math.pi)     # ppm2hz(1, 14.1, '1H')
    close(I, -2 * math.pi * nu * R.operator(ss, 'Lz', 0, 'comm'), 1e-6, 1e-12)


# test_scalar_coupling_hamiltonian.m:35-42 (Liouville-space form)
def test_scalar_coupling_is_2piJ_I_dot_S():
    ss = R.create(dict(isotopes=['1H', '1H'], magnet=0.0),
                  dict(zeeman=dict(scalar=[0.0, 0.0]), coupling=dict(scalar={(0, 1): 10.0})))
    ss = R.assume(R.basis(ss, dict(approximation='none')), 'nmr')
    I, _ = R.hamiltonian(ss)
    ref = sum(R.operator(ss, [o, o], [0, 1], 'comm') for o in ('Lx', 'Ly', 'Lz'))
    close(I, 2 * math.pi * 10 * ref, 1e-9, 1e-12)


# test_relaxation_t2_rate.m
def test_t2_eigenvalue_on_Lplus():
    ss = one_spin(zeeman=dict(scalar=[0.0]), relaxation=['t1_t2'], r1_rates=[2.0], r2_rates=[7.0])
    Rm = R.relaxation(ss)
    rho = R.state(ss, 'L+', '1H')
    close(Rm @ rho, -7.0 * rho, 1e-12, 1e-12)
    close(Rm @ R.state(ss, 'Lz', '1H'), -2.0 * R.state(ss, 'Lz', '1H'), 1e-12, 1e-12)


# test_liquid_single_spin_fid.m
def test_zero_offset_fid_is_constant():
    ss = one_spin(zeeman=dict(scalar=[0.0]))
    ss = R.assume(ss, 'nmr')
    I, _ = R.hamiltonian(ss)
    rho = R.state(ss, 'L+', '1H')
    fid = R.acquire(ss, dict(rho0=rho, coil=rho, sweep=1000, npoints=8), I, sp.csc_matrix(I.shape))
    close(fid, fid[0] * np.ones(8), 1e-12, 1e-12)


# test_dynamic_propagation_frontends.m:39-143
def test_propagator_step_evolution_krylov_frontends():
    ss = one_spin(zeeman=dict(scalar=[0.0]))
    ss.tols['small_matrix'] = 2               # force the Taylor branch
    L = R.operator(ss, 'Lz', 0, 'comm')
    rho = R.state(ss, 'Lx', '1H') + 0.25 * R.state(ss, 'Ly', '1H')
    dt = 2.5e-4
    P = R.propagator(ss, L, dt)
    Pref = sla.expm(-1j * L.toarray() * dt)
    close(P, Pref, 1e-10, 1e-10)
    close(R.step(ss, L, rho, dt), Pref @ rho, 1e-12, 1e-12)
    close(R.step(ss, L, rho, 0.0), rho, 1e-14, 1e-14)
    coil = R.state(ss, 'Lx', '1H')
    ss.tols['small_matrix'] = 200             # evolution/krylov checks use the default system
    P = R.propagator(ss, L, dt)
    traj = [rho, P @ rho, P @ P @ rho, P @ P @ P @ rho]
    ref = np.array([np.vdot(coil, t) for t in traj])
    close(R.evolution_observable(ss, L, coil, rho, dt, 3), ref, 1e-12, 1e-12)
    close(R.krylov_observable(ss, L, coil, rho, dt, 3), ref, 1e-12, 1e-12)


# test_dynamic_frame_frontends.m:147-178
def test_orientation_contracts_populated_components():
    Q = {1: [[sp.csc_matrix((2, 2), dtype=complex) for _ in range(3)] for _ in range(3)],
         2: [[sp.csc_matrix((2, 2), dtype=complex) for _ in range(5)] for _ in range(5)]}
    Q[1][0][2] = sp.csc_matrix(np.array([[0, 1], [0, 0]], complex))
    Q[1][2][0] = sp.csc_matrix(np.array([[0, 0], [1, 0]], complex))
    Q[2][2][2] = sp.csc_matrix(np.array([[1, 0], [0, -1]], complex))
    ang = (0.2, 0.3, -0.4)
    D1, D2 = R.wigner(1, *ang), R.wigner(2, *ang)
    ref = D1[0, 2] * Q[1][0][2] + D1[2, 0] * Q[1][2][0] + D2[2, 2] * Q[2][2][2]
    ref = (ref + ref.conj().T) / 2
    close(R.orientation(Q, ang), ref, 1e-14, 1e-14)


# test_grid_geometry_suite.m:77-85
def test_fibonacci_grid_geometry():
    al, be, ga, w = R.grid_fib(3)
    assert al.size == 7 and np.all(al == 0)
    xyz = np.stack([np.sin(be) * np.cos(ga), np.sin(be) * np.sin(ga), np.cos(be)], 1)
    close(np.linalg.norm(xyz, axis=1), np.ones(7), 1e-14, 1e-14)
    al, be, ga, w = R.grid_zcwn(200)
    assert al.size == 200 and abs(w.sum() - 1) < 1e-14


# test_ctx_powder_average.m:34-61 (single-spin CSA, projections=+1 basis)
def test_powder_sum_equals_explicit_weighted_sum():
    ss = R.create(dict(isotopes=['1H'], magnet=14.1),
                  dict(zeeman=dict(eigs=[[-2, -2, 4]], euler=[[0, 0, 0]])))
    ss = R.basis(ss, dict(approximation='none', projections=[1]))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    rho = R.state(ss, 'L+', '1H')
    par = dict(rho0=rho, coil=rho, sweep=2000, npoints=3)
    grid = R.grid_fib(4)
    avg = R.powder(ss, par, 'nmr', grid, setup=(I, Q))
    cells = R.powder(ss, par, 'nmr', grid, setup=(I, Q), sum_up=False)
    ref = grid[3][0] * cells[0]
    for n in range(1, len(cells)):
        ref = ref + grid[3][n] * cells[n]
    close(avg, ref, 1e-12, 1e-12)
    # closed form: one spin, axial CSA -> fid(t) = <rho|rho> exp(-i w(beta) t)
    gam = R.ISOTOPES['1H'][1]
    for n, b in enumerate(grid[1]):
        w = -gam * 14.1 * 1e-6 * (0.0 + 4.0 * (3 * math.cos(b) ** 2 - 1) / 2)
        t = np.arange(3) / 2000
        close(cells[n], np.vdot(rho, rho) * np.exp(-1j * w * t), 1e-9, 1e-9)


# test_orientation_average_suite.m (the orientation() part; average() is
# average Hamiltonian theory, not on this path)
def test_orientation_at_zero_euler_angles():
    Q = {1: [[None] * 3 for _ in range(3)]}
    Q[1][0][0] = sp.csc_matrix(np.array([[1.0, 0.0], [0.0, 0.0]]))
    Q[1][1][1] = sp.csc_matrix(np.array([[0.0, 1.0], [1.0, 0.0]]))
    Q[1][2][2] = sp.csc_matrix(np.array([[0.0, 0.0], [0.0, 2.0]]))
    H = R.orientation(Q, (0.0, 0.0, 0.0))
    close(H, Q[1][0][0] + Q[1][1][1] + Q[1][2][2], 1e-14, 1e-14)


# test_step_matches_expm.m, restated in Liouville space: the sign convention
# rho(t) = exp(-iHt) rho(0) exp(+iHt) of density-matrix evolution
def test_step_sign_convention_in_liouville_space():
    ss = R.basis(R.create(dict(isotopes=['1H'], magnet=0.0), dict()), dict(approximation='none'))
    w, dt = 2 * math.pi * 123, 2.5e-3
    L = w * R.operator(ss, 'Lz', '1H')
    x, y = R.state(ss, 'Lx', '1H'), R.state(ss, 'Ly', '1H')
    rho = x + 0.25 * y
    c, s = math.cos(w * dt), math.sin(w * dt)
    ref = (c * x + s * y) + 0.25 * (c * y - s * x)           # Lx -> Lx cos + Ly sin under exp(-iwt Lz)
    close(R.step(ss, L, rho, dt), ref, 1e-13, 1e-13)
    close(sla.expm(-1j * dt * L.toarray()) @ rho, ref, 1e-13, 1e-13)


def test_point_dipole_xyz2dd():
    """tests/kernel/test_dynamic_physics_formulae_suite.m:38-44 (xyz2dd): a
    1H-13C pair one Angstrom apart along z has the point-dipole constant
    d = gamma1*gamma2*hbar*mu0/(4*pi*r^3) and the traceless tensor
    d*diag(1, 1, -2).  The oracle (kernel/utilities/dipolar.m, half of the
    tensor on each ordered pair) and the product's host builder must give it,
    at the reference test's 1e-6 relative tolerance (its hbar and mu0 are
    the older CODATA values)."""
    from spinach_gb300 import spin_system as S
    hbar, mu0 = 1.054571628e-34, 4 * np.pi * 1e-7
    d_ref = R.ISOTOPES['1H'][1] * R.ISOTOPES['13C'][1] * hbar * mu0 / (4 * np.pi * (1e-10) ** 3)
    M_ref = d_ref * np.diag([1.0, 1.0, -2.0])
    ss = R.create(dict(isotopes=['1H', '13C'], magnet=14.1), dict(coordinates=[[0, 0, 0], [0, 0, 1]]))
    M = ss.coupling[(0, 1)] + ss.coupling[(1, 0)]
    assert np.abs(M - M_ref).max() <= 1e-6 * abs(d_ref)
    pss = S.make_spin_system(['1H', '13C'], 14.1, coordinates=[[0, 0, 0], [0, 0, 1]])
    P = pss.couplings[(0, 1)] + pss.couplings[(1, 0)]
    assert np.abs(P - M_ref).max() <= 1e-6 * abs(d_ref)
    assert np.abs(P - M).max() <= 1e-14 * abs(d_ref)
