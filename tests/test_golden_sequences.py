"""The oracle's pulse sequences and MAS contexts against their committed FP64
fixtures (tests/golden/c0_sequences_fp64.npz, made by
``python tests/golden/make_golden.py sequences``): a change to any
restatement shows up here before it reaches a parity test."""
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.dirname(__file__)


def _maker():
    spec = importlib.util.spec_from_file_location('make_golden', os.path.join(HERE, 'golden', 'make_golden.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope='module')
def cases():
    mg = _maker()
    w, fns = mg.sequence_cases()
    gold = np.load(os.path.join(HERE, 'golden', 'c0_sequences_fp64.npz'))
    return mg, w, fns, gold


@pytest.mark.parametrize('name', ['hp_acquire', 'cpmg', 'eseem', 'oopeseem', 'deer_3p_hard_deer',
                                  'deer_3p_hard_echo', 'singlerot', 'floquet'])
def test_sequence_matches_fixture(cases, name):
    mg, w, fns, gold = cases
    from spinach_gb300 import workloads as W
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    assert gold['sel'].tolist() == mg.SEQ_SEL.tolist() and int(gold['seed']) == w.seed
    got = sum(mg.SEQ_W[i] * fns[name]((al[j], be[j], ga[j])) for i, j in enumerate(mg.SEQ_SEL))
    ref = gold[name]
    assert got.shape == ref.shape and np.abs(ref).max() > 0.01
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
