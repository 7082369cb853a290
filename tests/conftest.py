import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (incremental)."""
    from gmlib_gb300 import build as gbuild
    from oracle import build as obuild
    gbuild.build()
    obuild.build_oracle()
    yield


@pytest.fixture(scope="session")
def G():
    import gmlib_gb300
    return gmlib_gb300


@pytest.fixture(scope="session")
def O():
    import oracle
    return oracle


@pytest.fixture
def gpu(G):
    """A GMlib instance on device 0, stopped after the test."""
    g = G.lib.GmlInit(0)
    if not g:
        pytest.fail("GmlInit(0) failed on a GPU test")
    yield g
    G.lib.GmlStop(g)


PARAMS = b"typedef struct {\n   int   foo;\n   float res;\n}GmlParSct;\n"
