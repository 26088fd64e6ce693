import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cloud-renderer_gb300")
for p in (PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (incremental)."""
    import __graft_entry__
    __graft_entry__.build()
    yield


@pytest.fixture(scope="session")
def ctx():
    import cloudgb
    c = cloudgb.Context(0)
    yield c
    c.close()
