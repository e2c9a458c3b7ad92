import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")
    config.addinivalue_line("markers", "slow: longer CPU-side checks")


@pytest.fixture(scope="session")
def lib():
    from ubootgl_gb300 import build as B
    B.build()
    from ubootgl_gb300 import _lib
    return _lib.load()
