"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/spinach_gpu.h (no GPU needed)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'spinach_gpu.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(spx_[a-z_]+)\s*\(', src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert 'spx_create' in syms and 'spx_run_powder' in syms and len(syms) >= 10


def test_library_exports_declared_symbols(engine_lib):
    from spinach_gb300 import engine
    out = subprocess.run(['nm', '-D', '--defined-only', engine.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r'\bT (spx_\w+)', out))
    missing = set(declared_symbols()) - exported
    assert not missing, missing
    assert set(engine.SIGNATURES) == set(declared_symbols())


def test_status_strings_without_gpu(engine_lib):
    assert engine_lib.spx_status_string(0) == b'success'
    assert engine_lib.spx_version().startswith(b'spinach-gb300')
    assert engine_lib.spx_last_error(None) == b'NULL handle'


def test_create_without_gpu_fails_cleanly(engine_lib):
    import ctypes
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    h = ctypes.c_void_p()
    st = engine_lib.spx_create(ctypes.byref(h), 0)
    assert st != 0 and not h.value
