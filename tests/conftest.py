import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, 'oracle')):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the native library')


@pytest.fixture(scope='session')
def native():
    """The native solver library, built if needed (GPU tests only)."""
    from gprmax_gb300 import _native
    return _native.lib()
