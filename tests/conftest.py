import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def gblib():
    from diffrg_gb300 import build as B

    B.build()
    from diffrg_gb300 import capi

    return capi.load()


@pytest.fixture(scope="session")
def ctx(gblib):
    from diffrg_gb300.engine import Context

    c = Context(0)
    yield c
    c.close()
