"""Host side of the single-rotor (MAS) Fokker-Planck workload
(kernel/contexts/singlerot.m) against the oracle's literal restatement, and
the reference's own single-rotor known answers restated on the oracle."""
import numpy as np
import pytest
import scipy.linalg as sla

from oracle import spinach_ref as R
from oracle_cases import oracle_system, rel_err
from spinach_gb300 import singlerot as SR, workloads as W


def test_wigner_matches_oracle():
    rng = np.random.default_rng(3)
    for l in (1, 2):
        for _ in range(5):
            a, b, g = rng.uniform(-np.pi, np.pi, 3)
            assert np.abs(SR.wigner_d(l, a, b, g) - R.wigner(l, a, b, g)).max() < 1e-14


@pytest.mark.parametrize('N', [1, 3, 5, 8, 9, 17])
def test_fourier_derivative_matches_fourdif(N):
    x, D = SR.fourier_derivative(N)
    xo, Do = R.fourdif1(N)
    assert np.allclose(x, xo, atol=0) and np.abs(D - Do).max() < 1e-13 * max(1.0, np.abs(Do).max())
    assert np.abs(D + D.T).max() == 0.0                     # antisymmetric: 1i*M is Hermitian


def test_rotor_space_liouvillian_matches_oracle():
    """I' + sum D(Omega) Q' assembled from the upload form equals the
    oracle's blkdiag(H_n) + 1i*M at an orientation."""
    w = W.c0()
    L = W.build(w)
    par = dict(max_rank=3, rate=12.5e3, axis=(1.0, 1.0, 1.0))
    I_fp, terms, R_fp, rho0, coil = SR.fokker_planck(L.I, L.terms, L.R, L.rho0, L.coil, **par)
    ss, I, Q = oracle_system(w)
    ang = (0.3, 1.1, -0.7)
    A = I_fp.toarray().astype(complex)
    for (r, j, m), Qp in terms.items():
        A += SR.wigner_d(r, *ang)[j, m] * Qp.toarray()
    N, dim = 7, L.dim
    phases, Dfd = R.fourdif1(N)
    rphi, rth = SR.rotor_axis_angles(par['axis'])
    blocks = []
    for n in range(N):
        Hn = I.toarray().astype(complex)
        for r in sorted(Q):
            Dc = R.wigner(r, rphi, rth, 0) @ R.wigner(r, 0, 0, phases[n]) @ R.wigner(r, *ang)
            for k in range(2 * r + 1):
                for m in range(2 * r + 1):
                    if Q[r][k][m] is not None:
                        Hn += Dc[k, m] * Q[r][k][m].toarray()
        blocks.append(Hn)
    G = sla.block_diag(*blocks) + 1j * 2 * np.pi * par['rate'] * np.kron(Dfd, np.eye(dim))
    assert np.abs(A - G).max() <= 1e-12 * np.abs(G).max()
    assert np.abs(G - G.conj().T).max() <= 1e-12 * np.abs(G).max()
    assert len(terms) == 25                                  # every D^2(j, m) is populated off the rotor axis
    assert rho0.shape == (N * dim,) and np.isclose(np.vdot(coil, rho0), np.vdot(L.coil, L.rho0))


def _one_proton():
    """tests/kernel/test_ctx_singlerot_acquire.m: one 1H with an axial shift
    tensor, projections +1 basis, max_rank 1, 1 kHz, axis [1 1 1]."""
    sys_ = dict(isotopes=['1H'], magnet=14.1, enable=[])
    inter = dict(zeeman=dict(eigs=[[-2.0, -2.0, 4.0]], euler=[[0.0, 0.0, 0.0]]))
    ss = R.create(sys_, inter)
    ss = R.basis(ss, dict(approximation='none', projections=[1]))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    return ss, I, Q


def test_reference_single_crystal_known_answers():
    ss, I, Q = _one_proton()
    rho0 = R.state(ss, 'L+', '1H')
    par = dict(rho0=rho0, coil=rho0, sweep=2000.0, npoints=3, rate=1000.0, axis=(1, 1, 1), max_rank=1,
               single_crystal=True)
    fid = R.singlerot_orientation_fid(ss, I, Q, par, (0.0, 0.0, 0.0))
    assert fid.shape == (3,)                                  # one point per requested sample
    assert abs(fid[0] - np.vdot(rho0, rho0)) <= 1e-12          # zero-time coil overlap preserved
    assert np.all(np.isfinite(fid))


def test_powder_rotor_averaging_preserves_the_zero_time_signal():
    w = W.c0()
    ss, I, Q = oracle_system(w)
    par = dict(rho0=R.state(ss, *w.rho0), coil=R.state(ss, *w.coil), sweep=1 / w.dt, npoints=4, rate=10e3,
               axis=(1, 1, 1), max_rank=2)
    fid = R.singlerot_orientation_fid(ss, I, Q, par, (0.0, 0.9, 2.0))
    assert abs(fid[0] - np.vdot(par['coil'], par['rho0'])) <= 1e-12 * abs(fid[0])


def test_grid_file_round_trip(tmp_path):
    """contexts.load_grid reads the reference's grid-file layout (MATLAB v5
    with alphas, betas, gammas, weights columns)."""
    import scipy.io as sio
    from spinach_gb300 import contexts as X
    rng = np.random.default_rng(1)
    cols = {k: rng.uniform(0, 1, (7, 1)) for k in ('alphas', 'betas', 'gammas', 'weights')}
    path = str(tmp_path / 'g.mat')
    sio.savemat(path, cols)
    g = X.load_grid(path)
    assert all(np.array_equal(a, cols[k].ravel()) for a, k in zip(g, ('alphas', 'betas', 'gammas', 'weights')))
    sio.savemat(path, {'alphas': cols['alphas']})
    with pytest.raises(ValueError):
        X.load_grid(path)


def test_floquet_liouvillian_matches_oracle():
    """floquet.m's F = sum_h kron(S_h, T_h) + M assembled from the upload form
    equals the oracle's literal construction at an orientation, and F is
    Hermitian (the engine's Hermitisation leaves it unchanged)."""
    w = W.c0()
    L = W.build(w)
    par = dict(max_rank=3, rate=12.5e3, axis=(1.0, 1.0, 1.0))
    I_f, terms, R_f, rho0, coil = SR.floquet_system(L.I, L.terms, L.R, L.rho0, L.coil, **par)
    ss, I, Q = oracle_system(w)
    ang = (0.3, 1.1, -0.7)
    A = I_f.toarray().astype(complex)
    for (r, j, m), Qp in terms.items():
        A += SR.wigner_d(r, *ang)[j, m] * Qp.toarray()
    # the oracle's Floquet matrix, rebuilt the same way floquet_orientation_fid does
    N, dim = 7, L.dim
    phi, th = SR.rotor_axis_angles(par['axis'])
    T = [np.zeros((dim, dim), complex) for _ in range(5)]
    for r in sorted(Q):
        L2R = R.wigner(r, phi, th, 0)
        Dm = L2R @ R.wigner(r, *ang) @ L2R.conj().T
        for n in range(2 * r + 1):
            Dr = np.zeros((2 * r + 1, 2 * r + 1)); Dr[n, n] = 1
            D = L2R @ Dr @ L2R.conj().T @ Dm
            for k in range(2 * r + 1):
                for mm in range(2 * r + 1):
                    if Q[r][k][mm] is not None:
                        T[n - r + 2] += D[k, mm] * Q[r][k][mm].toarray()
    T[2] += I.toarray()
    F = sum(np.kron(np.eye(N, k=h - 2), T[h]) for h in range(5))
    F = F + 2 * np.pi * par['rate'] * np.kron(np.diag(np.arange(-3, 4, dtype=float)), np.eye(dim))
    assert np.abs(A - F).max() <= 1e-12 * np.abs(F).max()
    assert np.abs(F - F.conj().T).max() <= 1e-10 * np.abs(F).max()
    assert rho0.shape == (N * dim,) and np.isclose(np.vdot(coil, rho0), np.vdot(L.coil, L.rho0))


def test_reference_floquet_acquire_known_answers():
    """tests/kernel/test_ctx_floquet_acquire.m:25-66: one 1H with an axial
    shift tensor (projections +1 basis), max_rank 1, 1 kHz about (1,1,1),
    three points at 2 kHz on the reference's 14-point Lebedev grid
    (leb_2ang_rank_5): three points, the zero-time signal equals coil'*rho0
    to 1e-12 (the Floquet projection preserves the initial overlap), all
    finite."""
    import os
    ss, I, Q = _one_proton()
    d = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'grid_leb_2ang_rank_5.npz'))
    rho0 = R.state(ss, 'L+', '1H')
    par = dict(rho0=rho0, coil=rho0, sweep=2000.0, npoints=3, rate=1000.0, axis=(1, 1, 1), max_rank=1)
    fid = sum(d['weights'][i] * R.floquet_orientation_fid(ss, I, Q, par, (d['alphas'][i], d['betas'][i],
                                                                          d['gammas'][i]))
              for i in range(d['weights'].size))
    assert fid.shape == (3,)
    assert abs(fid[0] - np.vdot(rho0, rho0)) <= 1e-12
    assert np.all(np.isfinite(fid))
