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
