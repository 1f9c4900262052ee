import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle_ffi import load_oracle
    return load_oracle()


@pytest.fixture(scope="session")
def engine():
    from locarna_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()
