import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")
    config.addinivalue_line("markers", "slow: long CPU oracle run")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def native():
    """The sm_103a library, built in-tree if needed.  GPU tests only."""
    from cfd__gb300 import _native, build
    build.build()
    return _native.load()
