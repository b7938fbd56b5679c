"""Spinach's calling convention (spinach_gb300.contexts): the same sys / inter /
bas / parameters structures go to the oracle and to the GPU engine."""
import numpy as np
import pytest

from spinach_gb300 import contexts as X, engine as E, workloads as W
from oracle_cases import rel_err
from oracle import spinach_ref as R

pytestmark = pytest.mark.gpu


def _structures():
    sys_ = dict(isotopes=['13C', '1H', '1H'], magnet=14.1)
    inter = dict(zeeman=dict(eigs=[[10.0, 70.0, 180.0], [1.0, 3.0, 8.0], [2.0, 2.5, 6.0]],
                             euler=[[0.1, 0.7, 1.9], [0.4, 1.2, 0.3], [2.0, 0.5, 1.0]]),
                 coordinates=[[0.0, 0.0, 0.0], [1.09, 0.0, 0.0], [-0.36, 1.03, 0.0]],
                 coupling=dict(scalar={(0, 1): 140.0, (0, 2): 135.0}),
                 relaxation=['t1_t2'], r1_rates=[2.0, 5.0, 5.0], r2_rates=[20.0, 40.0, 45.0])
    bas = dict(approximation='none', level=0)
    return sys_, inter, bas


def _oracle(sys_, inter, bas, krylov=False):
    ss = R.create(dict(sys_, enable=['krylov'] if krylov else []), inter)
    ss = R.basis(ss, dict(bas, space_level=1))
    return R.powder_setup(ss, 'nmr')


def test_powder_acquire(gpu_engine):
    sys_, inter, bas = _structures()
    spin_system = X.basis(X.create(sys_, inter), bas)
    grid = W.zcwn_grid(40)
    parameters = dict(grid=grid, rho0=('Lx', '13C'), coil=('L+', '13C'), sweep=2e4, npoints=257,
                      spins=['13C', '1H'], offset=[800.0, -150.0])
    fid, _ = X.powder(spin_system, 'acquire', parameters, 'nmr', engine=gpu_engine)
    ss, I, Q = _oracle(sys_, inter, bas)
    I = R.frqoffset(ss, I, ['13C', '1H'], [800.0, -150.0])
    par = dict(rho0=R.state(ss, 'Lx', '13C'), coil=R.state(ss, 'L+', '13C'), sweep=2e4, npoints=257)
    ref = R.powder(ss, par, 'nmr', grid, setup=(I, Q))
    assert rel_err(fid, ref) <= 1e-10
    # sum_up = 0: one FID per orientation (powder.m:291-297)
    fids, _ = X.powder(spin_system, 'acquire', dict(parameters, sum_up=0), 'nmr', engine=gpu_engine)
    assert len(fids) == 40 and rel_err(sum(w * f for w, f in zip(grid[3], fids)), ref) <= 1e-10


def test_powder_hp_acquire_with_echo_and_decoupled_acquire(gpu_engine):
    sys_, inter, bas = _structures()
    spin_system = X.basis(X.create(sys_, inter), bas)
    grid = W.zcwn_grid(24)
    ss, I, Q = _oracle(sys_, inter, bas)
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, 'L+', '13C'), pulse_op=R.operator(ss, 'Ly', '13C'),
               pulse_angle=np.pi / 2, echo_time=3e-4, echo_oper=R.operator(ss, 'Lx', '13C'), echo_angle=np.pi,
               sweep=2e4, npoints=200)
    ref = sum(grid[3][i] * R.powder_orientation_hp_acquire(ss, I, Q, par, (grid[0][i], grid[1][i], grid[2][i]))
              for i in range(24))
    parameters = dict(grid=grid, rho0=('Lz', '13C'), coil=('L+', '13C'), pulse_op=('Ly', '13C'),
                      pulse_angle=np.pi / 2, echo_time=3e-4, echo_oper=('Lx', '13C'), echo_angle=np.pi,
                      sweep=2e4, npoints=200)
    fid, _ = X.powder(spin_system, 'hp_acquire', parameters, 'nmr', engine=gpu_engine)
    assert rel_err(fid, ref) <= 1e-10
    # proton-decoupled 13C acquisition (acquire.m:51)
    par2 = dict(rho0=R.state(ss, 'Lx', '13C'), coil=R.state(ss, 'L+', '13C'), sweep=2e4, npoints=200,
                decouple=['1H'])
    ref2 = R.powder(ss, par2, 'nmr', grid, setup=(I, Q))
    fid2, _ = X.powder(spin_system, 'acquire', dict(grid=grid, rho0=('Lx', '13C'), coil=('L+', '13C'), sweep=2e4,
                                                     npoints=200, decouple=['1H']), 'nmr', engine=gpu_engine)
    assert rel_err(fid2, ref2) <= 1e-10
    with pytest.raises(ValueError):
        X.powder(spin_system, 'cpmg', dict(parameters, decouple=['1H'], nloops=2, timestep=1e-4), 'nmr',
                 engine=gpu_engine)


def test_singlerot_reference_single_crystal_case(gpu_engine):
    """tests/kernel/test_ctx_singlerot_acquire.m through the context API."""
    spin_system = X.basis(X.create(dict(isotopes=['1H'], magnet=14.1),
                                   dict(zeeman=dict(eigs=[[-2.0, -2.0, 4.0]], euler=[[0.0, 0.0, 0.0]]))),
                          dict(approximation='none', projections=[1]))
    rho = X.state(spin_system, 'L+', '1H')
    parameters = dict(rho0=rho, coil=rho, sweep=2000.0, npoints=3, rate=1000.0, axis=(1, 1, 1), max_rank=1,
                      grid='single_crystal')
    fid, _ = X.singlerot(spin_system, 'acquire', parameters, 'nmr', engine=gpu_engine)
    assert fid.shape == (3,) and abs(fid[0] - np.vdot(rho, rho)) <= 1e-12 and np.all(np.isfinite(fid))


def test_reference_powder_crystal_case(gpu_engine):
    """tests/kernel/test_ctx_powder_crystal.m through the context API: powder()
    on the single_crystal grid equals crystal() at zero Euler angles."""
    sys_ = dict(isotopes=['1H'], magnet=14.1)
    inter = dict(zeeman=dict(eigs=[[-2.0, -2.0, 4.0]], euler=[[0.0, 0.0, 0.0]]))
    bas = dict(approximation='none', projections=[1])
    spin_system = X.basis(X.create(sys_, inter), bas)
    rho = X.state(spin_system, 'L+', '1H')
    parameters = dict(spins=['1H'], rho0=rho, coil=rho, decouple=[], offset=[0.0], sweep=2000.0, npoints=4,
                      grid='single_crystal', orientation=[0.0, 0.0, 0.0])
    fid_powder, _ = X.powder(spin_system, 'acquire', parameters, 'nmr', engine=gpu_engine)
    fid_crystal = X.crystal(spin_system, 'acquire', parameters, 'nmr', engine=gpu_engine)
    assert np.abs(fid_powder - fid_crystal).max() <= 1e-12
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(bas, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(rho0=R.state(ss, 'L+', '1H'), coil=R.state(ss, 'L+', '1H'), sweep=2000.0, npoints=4)
    assert rel_err(fid_crystal, R.powder_orientation_fid(ss, I, Q, par, (0.0, 0.0, 0.0))) <= 1e-10


def test_floquet_context_matches_oracle(gpu_engine):
    """kernel/contexts/floquet.m through the context API on the reference's
    14-point Lebedev grid, against the oracle's per-orientation Floquet
    restatement."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'grid_leb_2ang_rank_5.npz'))
    grid = (d['alphas'], d['betas'], d['gammas'], d['weights'])
    sys_ = dict(isotopes=['1H', '13C'], magnet=14.1)
    inter = dict(zeeman=dict(eigs=[[-20.0, -10.0, 30.0], [40.0, -60.0, 20.0]],
                             euler=[[0.0, 0.0, 0.0], [0.3, 0.9, 1.7]]),
                 coordinates=[[0.0, 0.0, 0.0], [1.1, 0.0, 0.2]])
    bas = dict(approximation='none')
    spin_system = X.basis(X.create(sys_, inter), bas)
    parameters = dict(rho0=X.state(spin_system, 'Lx', '13C'), coil=X.state(spin_system, 'L+', '13C'),
                      sweep=50e3, npoints=64, rate=10e3, axis=(1, 1, 1), max_rank=3, grid=grid)
    fid, g = X.floquet(spin_system, 'acquire', parameters, 'nmr', engine=gpu_engine)
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), bas)
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(rho0=R.state(ss, 'Lx', '13C'), coil=R.state(ss, 'L+', '13C'), sweep=50e3, npoints=64,
               rate=10e3, axis=(1, 1, 1), max_rank=3)
    ref = sum(g[3][i] * R.floquet_orientation_fid(ss, I, Q, par, (g[0][i], g[1][i], g[2][i]))
              for i in range(g[3].size))
    assert np.abs(ref).max() > 0.05
    assert rel_err(fid, ref) <= 1e-10
    one, _ = X.floquet(spin_system, 'acquire', dict(parameters, grid='single_crystal'), 'nmr', engine=gpu_engine)
    assert rel_err(one, R.floquet_orientation_fid(ss, I, Q, par, (0.0, 0.0, 0.0))) <= 1e-10


def test_reference_powder_average_case(gpu_engine):
    """tests/kernel/test_ctx_powder_average.m: on the reference's 14-point
    Lebedev grid (kernel/grids/leb_2ang_rank_5.mat, copied into a fixture)
    the powder answer equals the explicit weighted sum of the per-orientation
    answers to 1e-12, and matches the oracle."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'grid_leb_2ang_rank_5.npz'))
    grid = (d['alphas'], d['betas'], d['gammas'], d['weights'])
    sys_ = dict(isotopes=['1H'], magnet=14.1)
    inter = dict(zeeman=dict(eigs=[[-2.0, -2.0, 4.0]], euler=[[0.0, 0.0, 0.0]]))
    bas = dict(approximation='none', projections=[1])
    spin_system = X.basis(X.create(sys_, inter), bas)
    rho = X.state(spin_system, 'L+', '1H')
    parameters = dict(spins=['1H'], rho0=rho, coil=rho, decouple=[], offset=[0.0], sweep=2000.0, npoints=3,
                      grid=grid)
    fid_avg, g = X.powder(spin_system, 'acquire', parameters, 'nmr', engine=gpu_engine)
    fid_cells, _ = X.powder(spin_system, 'acquire', dict(parameters, sum_up=False), 'nmr', engine=gpu_engine)
    fid_ref = g[3][0] * fid_cells[0]
    for n in range(1, len(fid_cells)):
        fid_ref = fid_ref + g[3][n] * fid_cells[n]
    assert np.abs(fid_avg - fid_ref).max() <= 1e-12
    ss = R.basis(R.create(dict(sys_, enable=[]), inter), dict(bas, space_level=1))
    ss, I, Q = R.powder_setup(ss, 'nmr')
    par = dict(rho0=R.state(ss, 'L+', '1H'), coil=R.state(ss, 'L+', '1H'), sweep=2000.0, npoints=3)
    assert rel_err(fid_avg, R.powder(ss, par, 'nmr', grid, setup=(I, Q))) <= 1e-10


def test_anisotropic_thermal_equilibrium_hp_acquire(gpu_engine):
    """powder.m 'aniso_eq' (powder.m:244-248, states/equilibrium.m): a
    radical at 4 K with an anisotropic g tensor starts every orientation from
    its own Boltzmann state; a 90-degree pulse (hp_acquire.m) reads it out."""
    import copy
    sys_ = dict(isotopes=['E', '14N'], magnet=0.34)
    inter = dict(zeeman=dict(eigs=[[2.0020, 2.0060, 2.0100], [0.0, 0.0, 0.0]], euler=[[0.3, 0.8, 1.1], [0, 0, 0]]),
                 coupling=dict(eigs={(0, 1): [15e6, 15e6, 90e6]}, euler={(0, 1): [0.0, 0.4, 0.0]}),
                 relaxation=['t1_t2'], r1_rates=[1e5, 0.0], r2_rates=[5e6, 0.0], temperature=4.0)
    bas = dict(approximation='none', level=0)
    spin_system = X.basis(X.create(sys_, inter), bas)
    grid = W.zcwn_grid(16)
    parameters = dict(grid=grid, coil=('L+', 'E'), pulse_op=('Ly', 'E'), pulse_angle=np.pi / 2, sweep=2e8,
                      npoints=128, needs=['aniso_eq'])
    fid, _ = X.powder(spin_system, 'hp_acquire', parameters, 'esr', engine=gpu_engine)
    fid_iso, _ = X.powder(spin_system, 'hp_acquire', dict(parameters, needs=['iso_eq']), 'esr', engine=gpu_engine)
    # the oracle: labframe left-product Hamiltonian, equilibrium per orientation
    ss = R.basis(R.create(dict(sys_, enable=['krylov']), inter), dict(bas, space_level=1))
    ssL = R.assume(copy.deepcopy(ss), 'labframe')
    IL, QL = R.hamiltonian(ssL, 'left')
    ss, I, Q = R.powder_setup(ss, 'esr')
    ref = 0
    for n in range(16):
        ang = (grid[0][n], grid[1][n], grid[2][n])
        par = dict(rho0=R.equilibrium(ssL, IL, QL, ang), coil=R.state(ss, 'L+', 'E'),
                   pulse_op=R.operator(ss, 'Ly', 'E'), pulse_angle=np.pi / 2, sweep=2e8, npoints=128)
        ref = ref + grid[3][n] * R.powder_orientation_hp_acquire(ss, I, Q, par, ang)
    assert rel_err(fid, ref) <= 1e-10
    assert rel_err(fid_iso, ref) > 1e-4          # the anisotropy of the equilibrium is visible


def test_function_handle_rho0(gpu_engine):
    """powder.m:250-252: rho0 given as a function of the orientation."""
    sys_, inter, bas = _structures()
    spin_system = X.basis(X.create(sys_, inter), bas)
    grid = W.zcwn_grid(20)
    lx, lz = X.state(spin_system, 'Lx', '13C'), X.state(spin_system, 'Lz', '1H')
    rho_f = lambda a, b, g: np.cos(b) * lx + np.sin(g) * lz
    parameters = dict(grid=grid, rho0=rho_f, coil=('L+', '13C'), sweep=2e4, npoints=150)
    fid, _ = X.powder(spin_system, 'acquire', parameters, 'nmr', engine=gpu_engine)
    ref = 0
    for n in range(20):
        one = dict(parameters, rho0=rho_f(grid[0][n], grid[1][n], grid[2][n]),
                   grid=(grid[0][n:n + 1], grid[1][n:n + 1], grid[2][n:n + 1], np.ones(1)))
        ref = ref + grid[3][n] * X.powder(spin_system, 'acquire', one, 'nmr', engine=gpu_engine)[0]
    assert rel_err(fid, ref) <= 1e-12


def test_per_orientation_outputs_of_a_program(gpu_engine):
    """powder.m sum_up = false for hp_acquire (a pulse program)."""
    sys_, inter, bas = _structures()
    spin_system = X.basis(X.create(sys_, inter), bas)
    grid = W.zcwn_grid(12)
    parameters = dict(grid=grid, rho0=('Lz', '13C'), coil=('L+', '13C'), pulse_op=('Ly', '13C'),
                      pulse_angle=np.pi / 2, echo_time=2e-4, echo_oper=('Lx', '13C'), echo_angle=np.pi,
                      sweep=2e4, npoints=90)
    fid, _ = X.powder(spin_system, 'hp_acquire', parameters, 'nmr', engine=gpu_engine)
    cells, _ = X.powder(spin_system, 'hp_acquire', dict(parameters, sum_up=0), 'nmr', engine=gpu_engine)
    assert len(cells) == 12 and cells[0].shape == (90,)
    assert np.abs(sum(w * c for w, c in zip(grid[3], cells)) - fid).max() <= 1e-12 * np.abs(fid).max()
    ss, I, Q = _oracle(sys_, inter, bas)
    par = dict(rho0=R.state(ss, 'Lz', '13C'), coil=R.state(ss, 'L+', '13C'), pulse_op=R.operator(ss, 'Ly', '13C'),
               pulse_angle=np.pi / 2, echo_time=2e-4, echo_oper=R.operator(ss, 'Lx', '13C'), echo_angle=np.pi,
               sweep=2e4, npoints=90)
    for n in (0, 7):
        ref = R.powder_orientation_hp_acquire(ss, I, Q, par, (grid[0][n], grid[1][n], grid[2][n]))
        assert rel_err(cells[n], ref) <= 1e-10


def test_powder_inv_rec(gpu_engine):
    """powder(..., @inv_rec, ...) on the GPU (experiments/inv_rec.m:50-66: the
    isotropic equilibrium, a 180-degree pulse, n_delays+1 recovery times, a
    90-degree pulse and one FID each) against the oracle's restatement, FP64
    <= 1e-10 and FP32 <= 1e-5 per recovery column, and the per-orientation
    cells (sum_up = 0)."""
    sys_, inter, bas = _structures()
    # fast longitudinal relaxation, so that the recovery shows within delays
    # whose |L|*dt stays in range (2.5 ms steps)
    inter = dict(inter, temperature=300.0, r1_rates=[200.0, 300.0, 300.0], r2_rates=[400.0, 500.0, 500.0])
    spin_system = X.basis(X.create(sys_, inter), bas)
    grid = W.zcwn_grid(16)
    parameters = dict(grid=grid, spins=['13C'], n_delays=4, max_delay=0.01, sweep=2e4, npoints=96)
    ss, I, Q = _oracle(sys_, inter, bas)
    ref = sum(grid[3][i] * R.powder_orientation_sequence(ss, I, Q, parameters, (grid[0][i], grid[1][i], grid[2][i]),
                                                         R.inv_rec) for i in range(16))
    assert ref.shape == (96, 5) and abs(ref[0, 0] - ref[0, -1]) > 0.1 * np.abs(ref).max()
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        fids, _ = X.powder(spin_system, 'inv_rec', parameters, 'nmr', engine=gpu_engine, precision=prec)
        assert fids.shape == (96, 5)
        for k in range(5):
            assert rel_err(fids[:, k], ref[:, k]) <= tol, (prec, k)
    cells, _ = X.powder(spin_system, 'inv_rec', dict(parameters, sum_up=0), 'nmr', engine=gpu_engine)
    assert len(cells) == 16 and cells[3].shape == (96, 5)
    one = R.powder_orientation_sequence(ss, I, Q, parameters, (grid[0][3], grid[1][3], grid[2][3]), R.inv_rec)
    assert rel_err(cells[3], one) <= 1e-10
