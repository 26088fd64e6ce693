"""The C-ABI library loads, exports every declared entry point, and rejects
bad arguments without touching a GPU."""
import ctypes
import os
import re

import pytest

import cloudgb
from cloudgb import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "cloudgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(cg_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_expected_surface():
    names = declared_functions()
    for must in ["cg_context_create", "cg_volume_create", "cg_volume_set_billboards",
                 "cg_voxelize", "cg_render", "cg_trace_cones", "cg_volume_read_level"]:
        assert must in names


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_every_declared_symbol_is_bound():
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_status_strings_and_version():
    lib = _lib.load()
    assert lib.cg_abi_version() == 2
    assert lib.cg_status_string(0) == b"ok"
    assert lib.cg_status_string(5) == b"not ready"


def test_defaults():
    p = _lib.cg_render_params()
    _lib.load().cg_render_params_default(ctypes.byref(p))
    assert p.view_steps == 64 and p.sun_steps == 24
    assert abs(p.cone_half_angle - 0.03) < 1e-9
    assert p.use_mlp == 0
    assert tuple(p.noise.offset) == (0.0, 0.0, 0.0)


def test_null_arguments_are_rejected():
    lib = _lib.load()
    assert lib.cg_context_create(0, None) == 1
    assert b"NULL" in lib.cg_last_error()
    pos = (ctypes.c_float * 3)(0, 0, 0)
    out = ctypes.c_void_p()
    assert lib.cg_volume_create(None, 64, -0.5, 0.5, pos, 7, 0, ctypes.byref(out)) == 1
    assert lib.cg_voxelize(None, None, None) == 1
    assert lib.cg_render(None, None, None, None, None, 0, None) == 1
    assert lib.cg_volume_set_billboards(None, None, None, None, 0, 1.0) == 1


def test_shader_rejects_unknown_parameter():
    with pytest.raises(AttributeError):
        cloudgb.ConeTraceShader(notAParameter=1)
