"""Three-angle grids, uneven weights, single orientations and option checks."""
import numpy as np
import pytest

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import oracle_powder, rel_err

pytestmark = pytest.mark.gpu


def _three_angle_grid(n, seed):
    """Random Euler triples with uneven positive weights (a three-angle grid,
    kernel/contexts/powder.m:226-235 uses alpha when the grid has it)."""
    rng = np.random.default_rng(seed)
    al = rng.uniform(0, 2 * np.pi, n)
    be = np.arccos(rng.uniform(-1, 1, n))
    ga = rng.uniform(0, 2 * np.pi, n)
    wt = rng.uniform(0.5, 1.5, n)
    return al, be, ga, wt / wt.sum()


@pytest.mark.parametrize('cluster', [0, 2])
def test_radical_three_angle_grid(gpu_engine, cluster):
    """Three Euler angles and uneven weights on the EPR radical ('esr':
    complex values, terms in several rows k of Q{r}); one and two CTAs per
    orientation."""
    w = W.c4_small()
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    g = _three_angle_grid(6, 11)
    ref = oracle_powder(w, g, krylov=True, sum_up=False)
    for prec, tol in ((E.FP64, 1e-10), (E.FP32, 1e-5)):
        res = gpu_engine.run(*g, w.dt, w.nsteps, precision=prec, per_orientation=True, cluster=cluster)
        if cluster:
            assert res.stats['cluster'] == cluster
        for i in range(6):
            assert rel_err(res.fids[i], ref[i]) <= tol, (prec, i)
        assert rel_err(res.fid, sum(wi * f for wi, f in zip(g[3], ref))) <= tol
    # a rotation about the field (alpha) leaves this signal unchanged: the
    # electron is observed along z and every term is secular in it
    g2 = (g[0] + 0.7, g[1], g[2], g[3])
    res2 = gpu_engine.run(*g2, w.dt, w.nsteps, precision=E.FP64, per_orientation=True, cluster=cluster)
    assert rel_err(res2.fids[0], ref[0]) <= 1e-10


def test_single_orientation_and_device_entry_point(gpu_engine):
    import torch
    w = W.c1()
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    g = [np.array([0.3]), np.array([1.1]), np.array([2.5]), np.array([1.0])]
    host = gpu_engine.run(*g, w.dt, 300, precision=E.FP64)
    dev = torch.device('cuda', 0)
    dg = [torch.tensor(a, dtype=torch.float64, device=dev) for a in g]
    out = torch.zeros(2 * 301, dtype=torch.float64, device=dev)
    gpu_engine.run_device(dg[0].data_ptr(), dg[1].data_ptr(), dg[2].data_ptr(), dg[3].data_ptr(), 1, w.dt, 300,
                          out.data_ptr(), precision=E.FP64)
    gpu_engine.synchronize()
    fid = out.cpu().numpy().view(np.complex128)
    assert np.array_equal(fid, host.fid)
    ref = oracle_powder(w, g, nsteps=300, krylov=True)
    assert rel_err(host.fid, ref) <= 1e-10


def test_option_checks(gpu_engine):
    w = W.c0()
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    g = W.zcwn_grid(4)
    with pytest.raises(E.SpxError):
        gpu_engine.run(*g, w.dt, 16, cluster=3)
    with pytest.raises(E.SpxError):
        gpu_engine.run(*g, w.dt, 16, precision=7)
    with pytest.raises(E.SpxError):
        gpu_engine.run(*g, w.dt, 16, cluster=16)


@pytest.mark.parametrize('its', [2, 48])
def test_loose_spectral_bounds_are_caught_and_retried(gpu_engine, its):
    """Few Lanczos steps give loose Ritz bounds; a chunk whose state norm grows
    is reported by the kernel and spx_run_powder reruns with Gershgorin bounds,
    so the FID still matches the oracle (failure detection without a GPU fault)."""
    import os
    w = W.c1()
    L = W.build(w)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    gold = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_orient_krylov_fp64.npz'))
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = gold['sel']
    res = gpu_engine.run(al[sel], be[sel], ga[sel], np.full(sel.size, 1 / sel.size), w.dt, w.nsteps,
                         precision=E.FP64, per_orientation=True, lanczos_its=its)
    assert res.stats['retries'] in (0, 1)
    for i in range(sel.size):
        assert rel_err(res.fids[i], gold['fids'][i]) <= 1e-10
    with pytest.raises(E.SpxError):
        gpu_engine.run(al[:2], be[:2], ga[:2], [0.5, 0.5], w.dt, 8, lanczos_its=1)
