import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if os.path.dirname(os.path.abspath(__file__)) not in sys.path:
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgb_cs.so")


@pytest.fixture(scope="session")
def gbo():
    from oracle import gbo as m

    return m


@pytest.fixture(scope="session")
def gb():
    import gaga_gb300 as m

    m._lib.load()
    return m
