"""The MEX gateway (spinach_gb300/mex/spinach_powder_gpu.cpp) compiled against a
host-only mx stand-in and a recording engine: marshalling of I, Q{r}{k,m}, R,
states, grid and options into the C ABI, outputs, and error identifiers
(mirrors the fake-mex approach of the reference's
tests/kernel/test_dynamic_integrity_includes_mex_suite.m:410-460)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, 'tests', 'mex_stub')


@pytest.mark.skipif(shutil.which('g++') is None, reason='needs g++')
def test_gateway_marshalling(tmp_path):
    exe = tmp_path / 'gateway_test'
    srcs = [os.path.join(ROOT, 'spinach_gb300', 'mex', 'spinach_powder_gpu.cpp'),
            os.path.join(STUB, 'mex_stub.cpp'), os.path.join(STUB, 'fake_engine.cpp'),
            os.path.join(STUB, 'gateway_test.cpp')]
    cmd = ['g++', '-std=c++17', '-O1', '-Wall', '-I', STUB, '-I', os.path.join(ROOT, 'include'), *srcs, '-o', str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stdout + res.stderr
    assert 'PASS' in res.stdout
