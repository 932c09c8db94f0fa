import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def engine():
    """The built engine library (compiled on first use)."""
    from tomoj_gb300 import _abi
    from tomoj_gb300.build import build
    build()
    return _abi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    O.lib()
    return O
