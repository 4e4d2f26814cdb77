import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def lib():
    """The built CUDA library (C ABI).  GPU tests need it; a missing build is an error."""
    from bayesnewton_gb300 import _lib
    return _lib.load()
