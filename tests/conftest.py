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


def reference_checkout():
    """The DiFfRG checkout the reference-reading tests use: $GBINT_REFERENCE_DIR, else a directory
    named 'reference' beside this repository; None when neither holds DiFfRG's sources."""
    cands = [os.environ.get("GBINT_REFERENCE_DIR"), os.path.join(os.path.dirname(ROOT), "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "Examples")):
            return c
    return None


@pytest.fixture(scope="session")
def reference_dir():
    d = reference_checkout()
    if d is None:
        pytest.skip("no DiFfRG checkout (set GBINT_REFERENCE_DIR)")
    return d
