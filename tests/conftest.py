import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')
    config.addinivalue_line('markers', 'slow: runs longer than a few seconds')


@pytest.fixture(scope='session')
def lib():
    """The built C-ABI library (built in-tree on first use)."""
    from festung_gb300.build import build as build_lib
    from festung_gb300 import _lib
    build_lib()
    return _lib.load()
