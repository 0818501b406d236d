import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU oracle case")


@pytest.fixture(scope="session")
def lib():
    from gpuintegration_gb300 import _build, load_library
    if not os.path.exists(_build.LIB):
        _build.build()
    return load_library()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def ctx(lib):
    import gpuintegration_gb300 as pg
    c = pg.Context(0)
    yield c
    c.close()
