"""ctypes binding of the C ABI in include/spinach_gpu.h.

The shared library is built in-tree (``spinach_gb300/lib/libspinach_gpu.so``)
by ``spinach_gb300.build``.  There is no CPU fallback: constructing an
``Engine`` without the library, or without a CUDA device, raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

LIB_PATH = os.path.join(os.path.dirname(__file__), 'lib', 'libspinach_gpu.so')

FP32, FP64 = 0, 1


class SpxCsc(C.Structure):
    _fields_ = [('n', C.c_int64), ('colptr', C.POINTER(C.c_int64)),
                ('rowidx', C.POINTER(C.c_int64)), ('values', C.POINTER(C.c_double))]


class SpxOptions(C.Structure):
    _fields_ = [('precision', C.c_int32), ('chunk_steps', C.c_int32), ('threads', C.c_int32),
                ('cluster', C.c_int32), ('series_tol', C.c_double), ('chunk_target', C.c_double),
                ('lanczos_its', C.c_int32), ('flags', C.c_int32)]


FLAG_NO_FP32_CHECK, FLAG_NO_PROMOTE = 1, 2
FP32_ERROR_BAR = 1e-5


SEQ_PULSE, SEQ_EVOLVE = 0, 1


class SpxSeqOp(C.Structure):
    _fields_ = [('kind', C.c_int32), ('pulse', C.c_int32), ('angle', C.c_double), ('nsteps', C.c_int64),
                ('dt', C.c_double), ('record', C.c_int32), ('reserved', C.c_int32)]


class SpxStats(C.Structure):
    _fields_ = [('n_orientations', C.c_int64), ('nsteps', C.c_int64), ('matvecs', C.c_int64),
                ('orientations_failed', C.c_int64), ('chunk_steps', C.c_int32),
                ('max_terms', C.c_int32), ('threads', C.c_int32), ('precision', C.c_int32),
                ('kernel_ms', C.c_double), ('reduce_ms', C.c_double),
                ('min_half_width', C.c_double), ('max_half_width', C.c_double),
                ('dim', C.c_int64), ('nnz', C.c_int64), ('ell_entries', C.c_int64),
                ('value_streams', C.c_int32), ('real_offdiag', C.c_int32),
                ('cluster', C.c_int32), ('smem_bytes', C.c_int32), ('channels', C.c_int32),
                ('retries', C.c_int32), ('fp32_checked', C.c_int32), ('kernel_launches', C.c_int64),
                ('fp32_rel_error', C.c_double), ('promoted_fp64', C.c_int32), ('reserved', C.c_int32),
                ('fp32_powder_error', C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# Every entry point of include/spinach_gpu.h with its ctypes signature.
_P = C.c_void_p
_D = C.POINTER(C.c_double)
SIGNATURES = {
    'spx_create': (C.c_int, [C.POINTER(_P), C.c_int]),
    'spx_destroy': (C.c_int, [_P]),
    'spx_upload_system': (C.c_int, [_P, C.POINTER(SpxCsc), C.c_int32, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(SpxCsc),
                                    C.POINTER(SpxCsc), _D, _D]),
    'spx_run_powder': (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, C.c_double, C.c_int64,
                                 C.POINTER(SpxOptions), _D, _D]),
    'spx_run_powder_device': (C.c_int, [_P, C.c_int64, _P, _P, _P, _P, C.c_double, C.c_int64,
                                        C.POINTER(SpxOptions), _P]),
    'spx_run_powder_noalloc': (C.c_int, [_P, C.c_int64, _P, _P, _P, _P, C.c_double, C.c_int64,
                                         C.c_int32, _P]),
    'spx_run_cpmg': (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, C.c_double, C.c_int64, C.c_int32,
                               C.POINTER(SpxCsc), C.POINTER(SpxOptions), _D, _D]),
    'spx_build_system': (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int32), C.c_int64, C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32), C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32), _D, _D, _D, _D, _D]),
    'spx_run_sequence': (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, C.c_int32, C.POINTER(SpxCsc), C.c_int32,
                                   C.POINTER(SpxSeqOp), C.POINTER(SpxOptions), _D, _D]),
    'spx_run_eseem': (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, C.c_double, C.c_int64, C.POINTER(SpxCsc),
                                C.POINTER(SpxOptions), _D, _D]),
    'spx_run_oopeseem': (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, C.c_double, C.c_int64, C.POINTER(SpxCsc),
                                   C.POINTER(SpxOptions), _D, _D]),
    'spx_run_deer': (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, C.c_double, C.c_int64, C.POINTER(SpxCsc),
                               C.POINTER(SpxCsc), C.POINTER(SpxOptions), _D, _D]),
    'spx_upload_coils': (C.c_int, [_P, C.c_int32, _D]),
    'spx_set_initial_states': (C.c_int, [_P, C.c_int64, _D]),
    'spx_autotune': (C.c_int, [_P, C.c_int64, _P, _P, _P, C.c_double, C.c_int64, C.c_int32,
                               C.POINTER(SpxOptions)]),
    'spx_batch_create': (C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(_P), C.POINTER(C.c_int64),
                                   C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(_P),
                                   C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(SpxOptions),
                                   C.POINTER(_P)]),
    'spx_batch_launch': (C.c_int, [_P, _P]),
    'spx_batch_synchronize': (C.c_int, [_P, C.POINTER(C.c_double)]),
    'spx_batch_destroy': (C.c_int, [_P]),
    'spx_batch_last_error': (C.c_char_p, [_P]),
    'spx_surrogate_create': (C.c_int, [C.POINTER(_P), C.c_int, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_uint64]),
    'spx_surrogate_destroy': (C.c_int, [_P]),
    'spx_surrogate_num_params': (C.c_int64, [_P]),
    'spx_surrogate_features': (C.c_int, [_P, C.c_int64, _P, _P, _P]),
    'spx_surrogate_train': (C.c_int, [_P, C.c_int64, _P, _P, _P, C.c_int32, C.c_float,
                                      C.POINTER(C.c_float)]),
    'spx_surrogate_predict': (C.c_int, [_P, C.c_int64, _P, _P, _P]),
    'spx_surrogate_gradients': (C.c_int, [_P, C.c_int64, _P, _P, _P, C.POINTER(C.c_float),
                                          C.POINTER(C.c_float)]),
    'spx_surrogate_get_params': (C.c_int, [_P, C.POINTER(C.c_float)]),
    'spx_surrogate_set_params': (C.c_int, [_P, C.POINTER(C.c_float)]),
    'spx_surrogate_last_error': (C.c_char_p, [_P]),
    'spx_synchronize': (C.c_int, [_P]),
    'spx_get_stream': (_P, [_P]),
    'spx_get_stats': (C.c_int, [_P, C.POINTER(SpxStats)]),
    'spx_status_string': (C.c_char_p, [C.c_int]),
    'spx_last_error': (C.c_char_p, [_P]),
    'spx_version': (C.c_char_p, []),
}


class SpxError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f'spinach_gpu error {code}: {message}')
        self.code = code


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the engine library and bind every declared entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f'{path} is missing: build it with spinach_gb300.build.build_library()')
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


class _CscHolder:
    """Keeps numpy buffers of one MATLAB-layout CSC matrix alive."""

    def __init__(self, A, n: int):
        A = sp.csc_matrix(A, shape=(n, n)).astype(np.complex128)
        A.sort_indices()
        self.colptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
        self.rowidx = np.ascontiguousarray(A.indices, dtype=np.int64)
        self.values = np.ascontiguousarray(A.data.view(np.float64) if A.nnz else np.zeros(2))
        self.struct = SpxCsc(n, self.colptr.ctypes.data_as(C.POINTER(C.c_int64)),
                             self.rowidx.ctypes.data_as(C.POINTER(C.c_int64)), _dptr(self.values))


@dataclass
class HostSystem:
    """A spin system in the C ABI's host layout: I and every Q as
    MATLAB-style CSC arrays (int64 column pointers and row indices,
    interleaved complex values), R likewise or absent, rho0 and coil as
    interleaved complex vectors."""
    n: int
    nterms: int
    holders: list
    Qarr: object
    rank: np.ndarray
    kk: np.ndarray
    mm: np.ndarray
    Rh: object
    rho0: np.ndarray
    coil: np.ndarray


def host_system(I, terms: dict, R=None, rho0=None, coil=None) -> HostSystem:
    """Lay out ``I``, the rotational-basis terms ``{(rank, k, m): Q}`` (0-based k,
    m), ``R`` (or None) and the states as the C ABI takes them."""
    n = I.shape[0]
    keys = sorted(terms)
    holders = [_CscHolder(I, n)] + [_CscHolder(terms[k], n) for k in keys]
    Qarr = (SpxCsc * max(1, len(keys)))(*[h.struct for h in holders[1:]])
    return HostSystem(
        n=n, nterms=len(keys), holders=holders, Qarr=Qarr,
        rank=np.array([k[0] for k in keys] or [0], np.int32),
        kk=np.array([k[1] for k in keys] or [0], np.int32),
        mm=np.array([k[2] for k in keys] or [0], np.int32),
        Rh=_CscHolder(R, n) if R is not None else None,
        rho0=np.ascontiguousarray(np.asarray(rho0, np.complex128).view(np.float64)),
        coil=np.ascontiguousarray(np.asarray(coil, np.complex128).view(np.float64)))


@dataclass
class PowderResult:
    fid: np.ndarray                    # (nsteps+1,) complex128
    fids: np.ndarray | None            # (n_orient, nsteps+1) complex128 or None
    stats: dict


class Engine:
    """One device handle with one uploaded spin system."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        self._check(self.lib.spx_create(C.byref(h), device), None)
        self.h = h
        self.dim = None

    def _check(self, status: int, handle):
        if status != 0:
            detail = self.lib.spx_last_error(handle).decode() if handle else ''
            raise SpxError(status, f'{self.lib.spx_status_string(status).decode()}: {detail}')

    def close(self):
        if getattr(self, 'h', None):
            self.lib.spx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, I, terms: dict, R=None, rho0=None, coil=None):
        """Upload ``I`` and the rotational-basis terms ``{(rank, k, m): Q}`` (0-based
        k, m), the relaxation superoperator ``R`` (or None), and the states."""
        self.upload_host(host_system(I, terms, R, rho0, coil))

    def upload_host(self, hs: 'HostSystem'):
        """spx_upload_system from host buffers already in the C ABI's layout
        (MATLAB-style CSC matrices, interleaved complex states)."""
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        self._check(self.lib.spx_upload_system(
            self.h, C.byref(hs.holders[0].struct), hs.nterms, ip(hs.rank), ip(hs.kk), ip(hs.mm), hs.Qarr,
            C.byref(hs.Rh.struct) if hs.Rh else None, _dptr(hs.rho0), _dptr(hs.coil)), self.h)
        self._host_system = hs             # the library reads the buffers during the call only
        self.dim = hs.n
        self.nchan = 1

    def build_system(self, hm, r_diag=None, rho0=None, coil=None) -> float:
        """Build I and Q on the GPU from ``hm`` (spin_system.HamiltonianMonomials)
        and upload the system with the relaxation diagonal and the states.
        Returns the device time of the construction (ms)."""
        i32 = lambda a: np.ascontiguousarray(a, np.int32)
        i64 = lambda a: np.ascontiguousarray(a, np.int64)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        lp = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
        mults, keys, radix = i32(hm.mults), i64(hm.keys), i64(hm.radix)
        rank = i32([t[0] for t in hm.terms] or [0])
        kk = i32([t[1] for t in hm.terms] or [0])
        mm = i32([t[2] for t in hm.terms] or [0])
        mt, ms, mc = i32(hm.mono_term), i32(hm.mono_spins), i32(hm.mono_codes)
        mf = np.ascontiguousarray(np.asarray(hm.mono_coefs, np.complex128).view(np.float64))
        n = keys.size
        rd = None if r_diag is None else np.ascontiguousarray(r_diag, np.float64)
        rho0 = np.ascontiguousarray(np.asarray(rho0, np.complex128).view(np.float64))
        coil = np.ascontiguousarray(np.asarray(coil, np.complex128).view(np.float64))
        ms_out = C.c_double(0.0)
        self._check(self.lib.spx_build_system(
            self.h, mults.size, ip(mults), n, lp(keys), lp(radix), len(hm.terms), ip(rank), ip(kk), ip(mm),
            mt.size, ip(mt), ip(ms), ip(mc), _dptr(mf), _dptr(rd) if rd is not None else None, _dptr(rho0),
            _dptr(coil), C.byref(ms_out)), self.h)
        self.dim = n
        self.nchan = 1
        return ms_out.value

    def set_initial_states(self, states):
        """One initial state per orientation (powder.m 'aniso_eq' or a function
        handle rho0): an (n_orient, dim) array; None returns to the single rho0."""
        if states is None:
            self._check(self.lib.spx_set_initial_states(self.h, 0, None), self.h)
            return
        arr = np.ascontiguousarray(np.asarray(states, np.complex128))
        flat = arr.view(np.float64).ravel()
        self._check(self.lib.spx_set_initial_states(self.h, arr.shape[0], _dptr(flat)), self.h)

    def upload_coils(self, coils):
        """Several detection states (evolution.m 'multichannel'): ``coils`` is
        a list of Liouville vectors or an (nchan, dim) array.  Runs then return
        one FID per channel (``fid`` of shape (nchan, nsteps+1))."""
        cs = np.atleast_2d(np.asarray(coils, np.complex128))
        arr = np.ascontiguousarray(cs.view(np.float64).ravel())      # column c = row c of cs
        self._check(self.lib.spx_upload_coils(self.h, cs.shape[0], _dptr(arr)), self.h)
        self.nchan = cs.shape[0]

    def run(self, alphas, betas, gammas, weights, dt: float, nsteps: int, precision: int = FP32,
            per_orientation: bool = False, chunk_steps: int = 0, threads: int = 0,
            series_tol: float = 0.0, cluster: int = 0, chunk_target: float = 0.0,
            lanczos_its: int = 0, fp32_check: bool = True, promote: bool = True) -> PowderResult:
        """spx_run_powder.  FP32 runs re-run two orientations in FP64 and report
        their larger relative error (stats['fp32_rel_error']) and the powder
        error it implies (stats['fp32_powder_error']); above half of 1e-5 the
        whole grid is re-run in FP64 (stats['promoted_fp64']) unless
        ``promote`` is false."""
        al = np.ascontiguousarray(alphas, np.float64)
        be = np.ascontiguousarray(betas, np.float64)
        ga = np.ascontiguousarray(gammas, np.float64)
        w = np.ascontiguousarray(weights, np.float64)
        no = al.size
        nch = getattr(self, 'nchan', 1)
        fid = np.zeros(2 * (nsteps + 1) * nch)
        fids = np.zeros(2 * (nsteps + 1) * nch * no) if per_orientation else None
        flags = (0 if fp32_check else FLAG_NO_FP32_CHECK) | (0 if promote else FLAG_NO_PROMOTE)
        opt = SpxOptions(precision, chunk_steps, threads, cluster, series_tol, chunk_target, lanczos_its, flags)
        self._check(self.lib.spx_run_powder(self.h, no, _dptr(al), _dptr(be), _dptr(ga), _dptr(w),
                                            float(dt), int(nsteps), C.byref(opt), _dptr(fid),
                                            _dptr(fids) if fids is not None else None), self.h)
        f = fid.view(np.complex128)
        fs = None if fids is None else fids.view(np.complex128).reshape(no, nch, nsteps + 1)
        if nch == 1:
            fs = None if fs is None else fs[:, 0, :]
        else:
            f = f.reshape(nch, nsteps + 1)
        return PowderResult(f, fs, self.stats())

    def run_cpmg(self, alphas, betas, gammas, weights, dt: float, npoints: int, nloops: int, pulse_op,
                 precision: int = FP32, threads: int = 0, cluster: int = 0,
                 per_orientation: bool = False) -> PowderResult:
        """CPMG echo train (experiments/cpmg.m): 90-degree pulse about ``pulse_op``
        (a commutation superoperator), npoints-1 steps, then ``nloops`` times a
        180-degree pulse and 2*npoints-1 steps.  ``fid`` holds the concatenated
        powder FIDs, npoints*(1 + 2*nloops) points."""
        al = np.ascontiguousarray(alphas, np.float64)
        be = np.ascontiguousarray(betas, np.float64)
        ga = np.ascontiguousarray(gammas, np.float64)
        w = np.ascontiguousarray(weights, np.float64)
        npts = npoints * (1 + 2 * nloops)
        fid = np.zeros(2 * npts)
        fids = np.zeros(2 * npts * al.size) if per_orientation else None
        P = _CscHolder(pulse_op, self.dim)
        opt = SpxOptions(precision, 0, threads, cluster, 0.0, 0.0, 0, 0)
        self._check(self.lib.spx_run_cpmg(self.h, al.size, _dptr(al), _dptr(be), _dptr(ga), _dptr(w), float(dt),
                                          int(npoints), int(nloops), C.byref(P.struct), C.byref(opt), _dptr(fid),
                                          _dptr(fids) if fids is not None else None), self.h)
        fs = None if fids is None else fids.view(np.complex128).reshape(al.size, npts)
        return PowderResult(fid.view(np.complex128), fs, self.stats())

    def run_sequence(self, alphas, betas, gammas, weights, pulse_ops, program, precision: int = FP32,
                     threads: int = 0, cluster: int = 0, per_orientation: bool = False) -> PowderResult:
        """A pulse program (spx_run_sequence): ``pulse_ops`` a list of
        commutation superoperators, ``program`` a list of ``('pulse', index,
        angle)`` and ``('evolve', nsteps, dt[, record])`` entries.  ``fid`` is
        the concatenation of the recorded segments' powder FIDs."""
        al = np.ascontiguousarray(alphas, np.float64)
        be = np.ascontiguousarray(betas, np.float64)
        ga = np.ascontiguousarray(gammas, np.float64)
        w = np.ascontiguousarray(weights, np.float64)
        holders = [_CscHolder(P, self.dim) for P in pulse_ops]
        parr = (SpxCsc * max(1, len(holders)))(*[hd.struct for hd in holders])
        ops = []
        npts = 0
        for op in program:
            if op[0] == 'pulse':
                ops.append(SpxSeqOp(SEQ_PULSE, int(op[1]), float(op[2]), 0, 0.0, 0, 0))
            elif op[0] == 'evolve':
                rec = 1 if (len(op) < 4 or op[3]) else 0
                ops.append(SpxSeqOp(SEQ_EVOLVE, 0, 0.0, int(op[1]), float(op[2]), rec, 0))
                npts += (int(op[1]) + 1) if rec else 0
            else:
                raise ValueError(f'unknown program entry {op[0]!r}')
        oarr = (SpxSeqOp * max(1, len(ops)))(*ops)
        fid = np.zeros(2 * max(npts, 1))
        fids = np.zeros(2 * max(npts, 1) * al.size) if per_orientation else None
        opt = SpxOptions(precision, 0, threads, cluster, 0.0, 0.0, 0, 0)
        self._check(self.lib.spx_run_sequence(self.h, al.size, _dptr(al), _dptr(be), _dptr(ga), _dptr(w),
                                              len(holders), parr, len(ops), oarr, C.byref(opt), _dptr(fid),
                                              _dptr(fids) if fids is not None else None), self.h)
        fs = None if fids is None else fids.view(np.complex128)[:npts * al.size].reshape(al.size, npts)
        return PowderResult(fid.view(np.complex128)[:npts], fs, self.stats())

    def run_eseem(self, alphas, betas, gammas, weights, timestep: float, npoints: int, pulse_op,
                  precision: int = FP32, threads: int = 0, cluster: int = 0,
                  per_orientation: bool = False, out_of_phase: bool = False) -> PowderResult:
        """Two-pulse echo (experiments/esr_dipolar/eseem.m): ``fid[n]`` is the powder
        echo after a 90-degree pulse, n steps of timestep/2, a 180-degree pulse
        and n more steps (npoints values).  out_of_phase: the 45-degree first
        pulse of experiments/esr_dipolar/oopeseem.m (spx_run_oopeseem)."""
        al = np.ascontiguousarray(alphas, np.float64)
        be = np.ascontiguousarray(betas, np.float64)
        ga = np.ascontiguousarray(gammas, np.float64)
        w = np.ascontiguousarray(weights, np.float64)
        fid = np.zeros(2 * npoints)
        fids = np.zeros(2 * npoints * al.size) if per_orientation else None
        P = _CscHolder(pulse_op, self.dim)
        opt = SpxOptions(precision, 0, threads, cluster, 0.0, 0.0, 0, 0)
        fn = self.lib.spx_run_oopeseem if out_of_phase else self.lib.spx_run_eseem
        self._check(fn(self.h, al.size, _dptr(al), _dptr(be), _dptr(ga), _dptr(w), float(timestep), int(npoints),
                       C.byref(P.struct), C.byref(opt), _dptr(fid), _dptr(fids) if fids is not None else None),
                    self.h)
        fs = None if fids is None else fids.view(np.complex128).reshape(al.size, npoints)
        return PowderResult(fid.view(np.complex128), fs, self.stats())

    def run_deer(self, alphas, betas, gammas, weights, stepsize: float, nsteps: int, ex_prob, ex_pump,
                 precision: int = FP32, threads: int = 0, cluster: int = 0,
                 per_orientation: bool = False) -> PowderResult:
        """Three-pulse DEER with hard pulses (experiments/esr_dipolar/deer_3p_hard_deer.m,
        'brief'): ``fid[j]`` is the powder DEER trace with the pump pulse j steps
        after the first probe pulse (nsteps+1 values), divided by the 2-norm of
        the uploaded (probe) coil."""
        al = np.ascontiguousarray(alphas, np.float64)
        be = np.ascontiguousarray(betas, np.float64)
        ga = np.ascontiguousarray(gammas, np.float64)
        w = np.ascontiguousarray(weights, np.float64)
        npts = int(nsteps) + 1
        fid = np.zeros(2 * npts)
        fids = np.zeros(2 * npts * al.size) if per_orientation else None
        Pp, Pu = _CscHolder(ex_prob, self.dim), _CscHolder(ex_pump, self.dim)
        opt = SpxOptions(precision, 0, threads, cluster, 0.0, 0.0, 0, 0)
        self._check(self.lib.spx_run_deer(self.h, al.size, _dptr(al), _dptr(be), _dptr(ga), _dptr(w),
                                          float(stepsize), int(nsteps), C.byref(Pp.struct), C.byref(Pu.struct),
                                          C.byref(opt), _dptr(fid), _dptr(fids) if fids is not None else None),
                    self.h)
        fs = None if fids is None else fids.view(np.complex128).reshape(al.size, npts)
        return PowderResult(fid.view(np.complex128), fs, self.stats())

    def run_device(self, d_alphas: int, d_betas: int, d_gammas: int, d_weights: int, n_orient: int,
                   dt: float, nsteps: int, d_fid: int, precision: int = FP32, chunk_steps: int = 0,
                   threads: int = 0, series_tol: float = 0.0, cluster: int = 0, fp32_check: bool = True):
        """Enqueue a run on device-resident buffers (raw device pointers); no
        sync.  FP32 runs report their FP64-checked error in the stats."""
        opt = SpxOptions(precision, chunk_steps, threads, cluster, series_tol, 0.0, 0,
                         0 if fp32_check else FLAG_NO_FP32_CHECK)
        self._check(self.lib.spx_run_powder_device(self.h, n_orient, d_alphas, d_betas, d_gammas,
                                                   d_weights, float(dt), int(nsteps), C.byref(opt),
                                                   d_fid), self.h)

    def run_noalloc(self, d_alphas: int, d_betas: int, d_gammas: int, d_weights: int, n_orient: int,
                    dt: float, nsteps: int, d_fid: int, precision: int = FP32):
        """Blocking run that allocates no memory: every intermediate lives in the
        library's static device scratch array (spx_run_powder_noalloc)."""
        self._check(self.lib.spx_run_powder_noalloc(self.h, n_orient, d_alphas, d_betas, d_gammas,
                                                     d_weights, float(dt), int(nsteps), int(precision),
                                                     d_fid), self.h)

    def autotune(self, d_alphas: int, d_betas: int, d_gammas: int, n_orient: int, dt: float, nsteps: int,
                 precision: int = FP32) -> dict:
        """Time candidate launch shapes on device-resident orientations; later
        runs with default options use the fastest.  Returns the chosen options."""
        best = SpxOptions()
        self._check(self.lib.spx_autotune(self.h, n_orient, d_alphas, d_betas, d_gammas, float(dt), int(nsteps),
                                          precision, C.byref(best)), self.h)
        return {'threads': best.threads, 'cluster': best.cluster, 'chunk_target': best.chunk_target}

    def synchronize(self):
        self._check(self.lib.spx_synchronize(self.h), self.h)

    @property
    def stream(self) -> int:
        return self.lib.spx_get_stream(self.h) or 0

    def stats(self) -> dict:
        st = SpxStats()
        self._check(self.lib.spx_get_stats(self.h, C.byref(st)), self.h)
        return st.as_dict()


class Surrogate:
    """Device MLP over spherical-harmonic features of (beta, gamma) (spx_surrogate_*).

    Device buffers are passed as raw pointers (ints), e.g. torch ``data_ptr()``."""

    def __init__(self, device: int = 0, lmax: int = 12, hidden: int = 256, layers: int = 4,
                 n_out: int = 128, seed: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.spx_surrogate_create(C.byref(h), device, lmax, hidden, layers, n_out, seed)
        if st != 0:
            raise SpxError(st, self.lib.spx_status_string(st).decode())
        self.h = h
        self.lmax, self.hidden, self.layers, self.n_out = lmax, hidden, layers, n_out
        self.n_in = (lmax + 1) ** 2
        self.n_params = int(self.lib.spx_surrogate_num_params(h))

    def _check(self, st):
        if st != 0:
            raise SpxError(st, f'{self.lib.spx_status_string(st).decode()}: '
                               f'{self.lib.spx_surrogate_last_error(self.h).decode()}')

    def close(self):
        if getattr(self, 'h', None):
            self.lib.spx_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def features(self, n, d_beta, d_gamma, d_out):
        self._check(self.lib.spx_surrogate_features(self.h, n, d_beta, d_gamma, d_out))

    def train(self, n, d_beta, d_gamma, d_targets, epochs: int, lr: float) -> np.ndarray:
        loss = np.zeros(epochs, np.float32)
        self._check(self.lib.spx_surrogate_train(self.h, n, d_beta, d_gamma, d_targets, epochs, lr,
                                                 loss.ctypes.data_as(C.POINTER(C.c_float))))
        return loss

    def predict(self, n, d_beta, d_gamma, d_out):
        self._check(self.lib.spx_surrogate_predict(self.h, n, d_beta, d_gamma, d_out))

    def gradients(self, n, d_beta, d_gamma, d_targets):
        g = np.zeros(self.n_params, np.float32)
        loss = np.zeros(1, np.float32)
        self._check(self.lib.spx_surrogate_gradients(self.h, n, d_beta, d_gamma, d_targets,
                                                     g.ctypes.data_as(C.POINTER(C.c_float)),
                                                     loss.ctypes.data_as(C.POINTER(C.c_float))))
        return float(loss[0]), g

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        self._check(self.lib.spx_surrogate_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self._check(self.lib.spx_surrogate_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))


class Batch:
    """One CUDA graph running a powder of every engine (spx_batch_*).

    ``runs`` holds, per engine, (engine, n_orient, d_alphas, d_betas, d_gammas,
    d_weights, dt, nsteps, d_fid, precision) with raw device pointers."""

    def __init__(self, runs):
        self.lib = load_library()
        n = len(runs)
        P = _P * n
        self.engines = [r[0] for r in runs]
        hs = P(*[r[0].h for r in runs])
        no = (C.c_int64 * n)(*[r[1] for r in runs])
        al, be, ga, wt = (P(*[r[i] for r in runs]) for i in (2, 3, 4, 5))
        dts = (C.c_double * n)(*[r[6] for r in runs])
        ns = (C.c_int64 * n)(*[r[7] for r in runs])
        out = P(*[r[8] for r in runs])
        opts = (SpxOptions * n)(*[SpxOptions(r[9], 0, 0, 0, 0.0, 0.0) for r in runs])
        h = C.c_void_p()
        st = self.lib.spx_batch_create(C.byref(h), n, hs, no, al, be, ga, wt, dts, ns, opts, out)
        if st != 0:
            raise SpxError(st, f'{self.lib.spx_status_string(st).decode()}: '
                               f'{self.lib.spx_batch_last_error(None).decode()}')
        self.h = h

    def _check(self, st):
        if st != 0:
            raise SpxError(st, f'{self.lib.spx_status_string(st).decode()}: '
                               f'{self.lib.spx_batch_last_error(self.h).decode()}')

    def launch(self, stream: int = 0):
        self._check(self.lib.spx_batch_launch(self.h, stream or None))

    def synchronize(self) -> float:
        ms = C.c_double()
        self._check(self.lib.spx_batch_synchronize(self.h, C.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, 'h', None):
            self.lib.spx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
