import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """Builds the CUDA library and the oracle once per session (incremental)."""
    import __graft_entry__ as g
    g.build_library_and_oracle()
    yield


@pytest.fixture
def ctx():
    import suminc_gb300 as sg
    c = sg.Context(0)
    yield c
    c.close()
