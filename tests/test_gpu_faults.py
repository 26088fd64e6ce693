"""Failure detection on the GPU without a fault: the tensor-core kernel's
bounded mbarrier wait is made to run out (a barrier nothing arrives on), the
host reads the error status, and the context keeps working."""
import ctypes

import numpy as np
import pytest

import cloudgb
from cloudgb import _lib, configs, workload

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_survives(ctx):
    lib = _lib.load()
    waited = ctypes.c_uint64()
    st = lib.cg_context_check_wait_timeout(ctx.handle, 20000, ctypes.byref(waited))
    assert st == 6, "CG_ERR_DEVICE_FAULT expected: the bound must fire"
    assert b"ran out" in lib.cg_last_error()
    assert 20000 <= waited.value < 500000, waited.value  # ~20 ms, not forever
    # invalid limits are refused before any launch
    assert lib.cg_context_check_wait_timeout(ctx.handle, 0, ctypes.byref(waited)) == 2
    # the context is still usable: a render after the probe is deterministic
    cfg = configs.SMALL_64
    wl = workload.build(cfg, boards=16, width=48, height=32)
    vol = cloudgb.CloudVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION,
                              cfg["mips"], ctx=ctx)
    vol.set_billboards(wl.positions, wl.scales, wl.densities)
    vol.update()
    cloudgb.VoxelizeShader().voxelize(vol, cloudgb.Sun(wl.sun_direction, *wl.sun_map))
    sh = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    cam = workload.make_camera(wl.cameras[0])
    a = sh.coneTrace(vol, cam)
    assert np.array_equal(a, sh.coneTrace(vol, cam)) and a[..., 3].max() > 0
    vol.close()
