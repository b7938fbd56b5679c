"""On-GPU construction of I and Q{r}{k,m} (spx_build_system) against the host
builder of the same operators (kernel/hamiltonian.m + superop.m semantics)
and, for the small system, against the oracle."""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_powder, rel_err

pytestmark = pytest.mark.gpu

STRUCT = ('dim', 'nnz', 'ell_entries', 'value_streams', 'real_offdiag')


def _pair(gpu_engine, w, grid, nsteps):
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    ref = {p: gpu_engine.run(*grid, w.dt, nsteps, precision=p) for p in (E.FP64, E.FP32)}
    bs = W.build_spec(w)
    ms = gpu_engine.build_system(bs.monomials, bs.r_diag, bs.rho0, bs.coil)
    got = {p: gpu_engine.run(*grid, w.dt, nsteps, precision=p) for p in (E.FP64, E.FP32)}
    return ref, got, ms


@pytest.mark.parametrize('name', ['c0', 'c1', 'c4_small', 'c4', 'deuterium'])
def test_built_system_matches_host_builder(gpu_engine, name):
    w = getattr(W, name)()
    grid = W.zcwn_grid(24)
    ref, got, ms = _pair(gpu_engine, w, grid, 300)
    assert ms > 0.0
    for k in STRUCT:
        assert got[E.FP64].stats[k] == ref[E.FP64].stats[k], k
    assert rel_err(got[E.FP64].fid, ref[E.FP64].fid) <= 1e-12
    assert rel_err(got[E.FP32].fid, ref[E.FP64].fid) <= 1e-5


def test_built_c2_systems_match_host_builder(gpu_engine):
    ws = W.c2()
    dims_seen = set()
    for w in ws:
        bs = W.build_spec(w)
        if bs.dim in dims_seen:
            continue
        dims_seen.add(bs.dim)
        ref, got, _ = _pair(gpu_engine, w, W.zcwn_grid(8), 128)
        for k in STRUCT:
            assert got[E.FP64].stats[k] == ref[E.FP64].stats[k], (w.name, k)
        assert rel_err(got[E.FP64].fid, ref[E.FP64].fid) <= 1e-12, w.name
    assert len(dims_seen) >= 5


def test_built_c0_matches_oracle(gpu_engine):
    w = W.c0()
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([5, 77, 160])
    g = (al[sel], be[sel], ga[sel], np.array([0.5, 0.3, 0.2]))
    bs = W.build_spec(w)
    gpu_engine.build_system(bs.monomials, bs.r_diag, bs.rho0, bs.coil)
    ref = oracle_powder(w, g, nsteps=200)
    assert rel_err(gpu_engine.run(*g, w.dt, 200, precision=E.FP64).fid, ref) <= 1e-10


def test_build_argument_checks(gpu_engine):
    bs = W.build_spec(W.c0())
    hm = bs.monomials
    bad = lambda **kw: type(hm)(**{**hm.__dict__, **kw})
    with pytest.raises(E.SpxError):                       # keys out of order
        gpu_engine.build_system(bad(keys=hm.keys[::-1].copy()), bs.r_diag, bs.rho0, bs.coil)
    with pytest.raises(E.SpxError):                       # code beyond the spin's states
        codes = hm.mono_codes.copy()
        codes[0, 0] = 4
        gpu_engine.build_system(bad(mono_codes=codes), bs.r_diag, bs.rho0, bs.coil)
    with pytest.raises(E.SpxError):                       # radix inconsistent with the multiplicities
        gpu_engine.build_system(bad(radix=hm.radix * 2), bs.r_diag, bs.rho0, bs.coil)
    with pytest.raises(E.SpxError):                       # term index out of range
        mt = hm.mono_term.copy()
        mt[0] = len(hm.terms) + 1
        gpu_engine.build_system(bad(mono_term=mt), bs.r_diag, bs.rho0, bs.coil)
