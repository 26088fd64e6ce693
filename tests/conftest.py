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


@pytest.fixture(autouse=True)
def _bounds_checked(request):
    """With CG_BOUNDS_CHECK=1 (the bounds-check library, built by
    `CG_BOUNDS_CHECK=1 python cloud-renderer_gb300/build.py`), every GPU test
    must end with no out-of-range index in any kernel."""
    yield
    if os.environ.get("CG_BOUNDS_CHECK") != "1" or request.node.get_closest_marker("gpu") is None:
        return
    import ctypes

    import cloudgb
    from cloudgb import _lib
    lib = _lib.load()
    assert lib.cg_bounds_check_build() == 1, "CG_BOUNDS_CHECK=1 but the normal library is loaded"
    c = request.getfixturevalue("ctx")
    n = ctypes.c_uint64()
    site = ctypes.create_string_buffer(256)
    _lib.check(lib.cg_context_bounds_violations(c.handle, ctypes.byref(n), site, 256),
               "cg_context_bounds_violations")
    assert n.value == 0, f"{n.value} out-of-range accesses, first at {site.value.decode()}"
