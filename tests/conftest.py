import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import loader
    return loader.load()


@pytest.fixture(scope="session")
def native():
    """The CUDA library's context on device 0 (GPU tests only)."""
    from kiyosi_gb300 import _native
    return _native.context(0)
