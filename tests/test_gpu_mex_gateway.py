"""The MEX gateway (spinach_gb300/mex/spinach_powder_gpu.cpp) linked against the
real engine library on the GPU, with the host-only mx stand-in in place of
MATLAB: the c0 system's I, Q{r}{k,m} cells, R, states and grid struct go in
as MATLAB would pass them (interleaved-complex CSC, 1-based cell positions,
etc/mex/prune_cpu.cpp conventions), and the outputs must equal the Python
binding's runs of the same engine on the same inputs (powder.m:280-297
layouts: fid (nsteps+1) x 1, fids (nsteps+1) x n_orient, two channels as
rows)."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from spinach_gb300 import engine as E, workloads as W
from oracle_cases import rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, 'tests', 'mex_stub')


def _csc(path, A):
    A = sp.csc_matrix(A, dtype=complex)
    A.sort_indices()
    n = A.shape[0]
    with open(path, 'wb') as f:
        np.array([n, A.nnz], np.int64).tofile(f)
        A.indptr.astype(np.int64).tofile(f)
        A.indices.astype(np.int64).tofile(f)
        np.ascontiguousarray(A.data).view(np.float64).tofile(f)


def _dense(path, v):
    v = np.ascontiguousarray(np.asarray(v).ravel())
    if np.iscomplexobj(v):
        v = v.view(np.float64)
    with open(path, 'wb') as f:
        np.array([v.size], np.int64).tofile(f)
        v.astype(np.float64).tofile(f)


def _read(path):
    raw = np.fromfile(path, np.float64)
    m, n = raw[:2].view(np.int64)
    return raw[2:].view(np.complex128).reshape((m, n), order='F')


@pytest.mark.skipif(shutil.which('g++') is None, reason='needs g++')
def test_gateway_on_the_real_engine(engine_lib, gpu_engine, tmp_path):
    from spinach_gb300 import spin_system as S
    lib = E.LIB_PATH
    exe = tmp_path / 'gateway_real'
    srcs = [os.path.join(ROOT, 'spinach_gb300', 'mex', 'spinach_powder_gpu.cpp'),
            os.path.join(STUB, 'mex_stub.cpp'), os.path.join(STUB, 'gateway_real.cpp')]
    cmd = ['g++', '-std=c++17', '-O1', '-I', STUB, '-I', os.path.join(ROOT, 'include'), *srcs,
           '-L', os.path.dirname(lib), '-lspinach_gpu', '-Wl,-rpath,' + os.path.dirname(lib), '-o', str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)

    w = W.c0()
    L = W.build(w)
    ss = W.spin_system_of(w)
    fac = S.factory_for(ss, S.build_basis(ss, w.approximation, w.level))
    coil2 = fac.state('Lx', '13C')
    al, be, ga, _ = W.zcwn_grid(w.n_orient)
    sel = np.array([2, 45, 90, 133, 170, 199])
    wt = np.array([0.1, 0.2, 0.15, 0.25, 0.2, 0.1])
    nsteps = 400
    keys = sorted(L.terms)
    d = str(tmp_path)
    _dense(os.path.join(d, 'meta.bin'), np.array([L.dim, sel.size, w.dt, nsteps, len(keys)], float))
    _dense(os.path.join(d, 'rkm.bin'), np.array([[r, k + 1, m + 1] for r, k, m in keys], float))
    _csc(os.path.join(d, 'I.bin'), L.I)
    _csc(os.path.join(d, 'R.bin'), L.R)
    for t, key in enumerate(keys):
        _csc(os.path.join(d, f'Q{t}.bin'), L.terms[key])
    _dense(os.path.join(d, 'rho0.bin'), np.asarray(L.rho0, complex))
    _dense(os.path.join(d, 'coils.bin'), np.concatenate([np.asarray(L.coil, complex), np.asarray(coil2, complex)]))
    _dense(os.path.join(d, 'grid.bin'), np.concatenate([al[sel], be[sel], ga[sel], wt]))
    res = subprocess.run([str(exe), d], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and 'PASS' in res.stdout, res.stdout + res.stderr

    g = (al[sel], be[sel], ga[sel], wt)
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
    r64 = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP64, per_orientation=True)
    fid_a, fids_a = _read(os.path.join(d, 'out_a_fid.bin')), _read(os.path.join(d, 'out_a_fids.bin'))
    assert fid_a.shape == (nsteps + 1, 1) and fids_a.shape == (nsteps + 1, sel.size)
    assert rel_err(fid_a[:, 0], r64.fid) <= 1e-13
    for i in range(sel.size):
        assert rel_err(fids_a[:, i], r64.fids[i]) <= 1e-13, i
    r32 = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP32)
    fid_c = _read(os.path.join(d, 'out_c_fid.bin'))
    assert rel_err(fid_c[:, 0], r32.fid) <= 1e-13
    assert rel_err(fid_c[:, 0], r64.fid) <= 1e-5
    gpu_engine.upload_coils([L.coil, coil2])
    rb = gpu_engine.run(*g, w.dt, nsteps, precision=E.FP64)
    fid_b = _read(os.path.join(d, 'out_b_fid.bin'))
    assert fid_b.shape == (2, nsteps + 1)
    for c in range(2):
        assert rel_err(fid_b[c], rb.fid[c]) <= 1e-13, c
    gpu_engine.upload(L.I, L.terms, L.R, L.rho0, L.coil)
