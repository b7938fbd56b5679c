"""In-tree build of the engine library for sm_103a (nvcc, no cmake)."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SOURCES = [os.path.join(HERE, 'csrc', f) for f in
           ['engine.cu', 'builder.cu', 'surrogate.cu'] +
           [f'kern_{p}_{c}{t}.cu' for p in ('f32r', 'f32c', 'f64r', 'f64c') for c in ('sc', 'dc') for t in ('', '_t')]]
DEPS = SOURCES + [os.path.join(HERE, 'csrc', 'kernels.cuh'), os.path.join(HERE, 'csrc', 'builder.h'), os.path.join(HERE, 'csrc', 'kern_inst.inc'),
                  os.path.join(ROOT, 'include', 'spinach_gpu.h')]
LIB = os.path.join(HERE, 'lib', 'libspinach_gpu.so')
NVCC_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a', '-O3', '-lineinfo', '-std=c++17',
              '-Xcompiler', '-fPIC', '-shared', '-diag-suppress', '550']


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile libspinach_gpu.so if it is missing or older than its sources."""
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    nvcc = os.environ.get('NVCC', 'nvcc')
    inc = ['-I', os.path.join(ROOT, 'include')]
    objs, procs = [], []
    for src in SOURCES:                       # translation units compile in parallel
        obj = os.path.join(os.path.dirname(LIB), os.path.basename(src) + '.o')
        objs.append(obj)
        procs.append(subprocess.Popen([nvcc, *NVCC_FLAGS, '-c', *inc, src, '-o', obj],
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    logs = [p.communicate()[0] for p in procs]
    if any(p.returncode for p in procs):
        raise RuntimeError('nvcc failed:\n' + '\n'.join(logs))
    res = subprocess.run([nvcc, *NVCC_FLAGS, *objs, '-o', LIB + '.tmp'], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc link failed:\n' + res.stdout + res.stderr)
    if verbose:
        print('\n'.join(logs) + res.stdout + res.stderr)
    os.replace(LIB + '.tmp', LIB)
    return LIB


if __name__ == '__main__':
    print(build_library(force=True, verbose=True))
