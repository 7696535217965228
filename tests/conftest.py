import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def lib():
    from song_gb300 import build, capi
    build.build()
    return capi.load()


@pytest.fixture(scope="session")
def olib():
    import oracle
    oracle.build()
    return oracle.load()
