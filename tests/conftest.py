import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')
    config.addinivalue_line('markers', 'slow: longer CPU oracle runs')


@pytest.fixture(scope='session')
def engine_lib():
    """Build (if needed) and load the engine library."""
    from spinach_gb300.build import build_library
    from spinach_gb300 import engine
    build_library()
    return engine.load_library()


@pytest.fixture(scope='session')
def gpu_engine(engine_lib):
    from spinach_gb300 import engine
    eng = engine.Engine(0)
    yield eng
    eng.close()
