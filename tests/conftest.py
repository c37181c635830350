import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def lib():
    from cpic_gb300 import build, load
    build.build()
    return load()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    return oracle.load()
