import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library; GPU tests fail loudly if it is missing."""
    from cubez_gb300 import build as cb
    cb.build()
    from cubez_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    return O.lib()
