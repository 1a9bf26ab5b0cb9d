import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpulib():
    """The built C-ABI library; GPU tests fail (not skip) when it cannot load."""
    from cpfft_gb300 import build
    build.build()
    import cpfft_gb300
    cpfft_gb300.load_library()
    return cpfft_gb300
