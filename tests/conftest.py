import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsimmd.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build, pyoracle
    build.build_oracle()
    return pyoracle


@pytest.fixture(scope="session")
def simlib():
    """libsimmd.so loaded through ctypes (built on demand)."""
    from simulationcode_gb300 import build, _lib
    build.build()
    return _lib.load()
