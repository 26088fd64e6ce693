"""cg_sun_map_noalloc, the allocation-free sun-view map entry point.

Some callers cannot call cudaMalloc: an engine or plugin host that hands out
all device memory from its own fixed budget, or a real-time render thread
that cannot take the device-wide synchronisation cudaMalloc may cause.  For
them the library offers this one entry point, which allocates nothing: it
keeps its per-texel depth keys in a fixed array compiled into the library,
and the caller passes the boards and the outputs in device memory it owns.

These tests call it through the C ABI twice in a row, on two different
scenes, and check that each result equals what the allocating path
(cg_voxelize, read back with cg_volume_read_sun_map / cg_volume_read_highlight)
produces: bit for bit, the tolerance used for all index work.  The second call
also checks that the shared array is reset between calls.  This file is named
to be collected last.
"""
import ctypes

import numpy as np
import pytest

import cloudgb
from cloudgb import _lib, configs, workload

pytestmark = pytest.mark.gpu


def _device_boards(positions, scales, fluffiness):
    # world centre = volume position + board position, radius = scale * fluffiness,
    # computed in float32 exactly as the library does
    cw = np.asarray(configs.VOLUME_POSITION, np.float32)[None, :] + positions.astype(np.float32)
    r = scales.astype(np.float32) * np.float32(fluffiness)
    arr = np.ascontiguousarray(np.concatenate([cw, r[:, None]], axis=1), np.float32)
    buf = cloudgb.DeviceBuffer(max(16, arr.nbytes))
    if arr.size:
        buf.upload(arr)
    return buf


def _noalloc(dim, positions, scales, sun, fluffiness=1.0):
    lib = _lib.load()
    boards = _device_boards(positions, scales, fluffiness)
    W, H = sun.map_width, sun.map_height
    d_pos = cloudgb.DeviceBuffer(W * H * 16)
    d_mask = cloudgb.DeviceBuffer(dim ** 3)
    vpos = (ctypes.c_float * 3)(*configs.VOLUME_POSITION)
    csun = sun._c()
    _lib.check(lib.cg_sun_map_noalloc(dim, configs.VOLUME_BOUNDS[0], configs.VOLUME_BOUNDS[1],
                                      vpos, boards.ptr, positions.shape[0], ctypes.byref(csun),
                                      d_pos.ptr, d_mask.ptr, None), "cg_sun_map_noalloc")
    return d_pos.download((H, W, 4)), d_mask.download((dim, dim, dim), np.uint8)


def _allocating(ctx, dim, mips, positions, scales, densities, sun, fluffiness=1.0):
    vol = cloudgb.CloudVolume(dim, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, mips, ctx=ctx)
    vol.set_billboards(positions, scales, densities)
    vol.fluffiness = fluffiness
    vol.update()
    cloudgb.VoxelizeShader().voxelize(vol, sun)
    _, pos = vol.read_sun_map(sun)
    return pos, vol.read_highlight()


def test_two_calls_in_a_row_match_voxelize(ctx):
    wl = workload.build(configs.SMALL_64)
    scenes = [
        (64, 7, wl.positions, wl.scales, wl.densities, cloudgb.Sun(wl.sun_direction, 1280, 720),
         1.0),
        (96, 7, wl.positions[:40] * 0.8, wl.scales[:40], wl.densities[:40],
         cloudgb.Sun((-0.5, 0.7, 0.4), 640, 480), 1.25),
    ]
    for dim, mips, pos, sc, den, sun, fl in scenes:
        got_pos, got_mask = _noalloc(dim, pos, sc, sun, fl)
        ref_pos, ref_mask = _allocating(ctx, dim, mips, pos, sc, den, sun, fl)
        assert np.array_equal(got_pos, ref_pos), "position map differs from cg_voxelize's"
        assert np.array_equal(got_mask, ref_mask), "highlight mask differs from cg_voxelize's"
        assert got_mask.sum() > 0


def test_rejects_a_map_beyond_the_fixed_array(ctx):
    lib = _lib.load()
    sun = cloudgb.Sun((0.3, 1.0, 0.2), 2048, 1024)  # 2^21 texels > CG_NOALLOC_MAX_TEXELS
    assert sun.map_width * sun.map_height > _lib.NOALLOC_MAX_TEXELS
    boards = cloudgb.DeviceBuffer(16)
    d_pos = cloudgb.DeviceBuffer(16)
    d_mask = cloudgb.DeviceBuffer(64 ** 3)
    vpos = (ctypes.c_float * 3)(*configs.VOLUME_POSITION)
    csun = sun._c()
    rc = lib.cg_sun_map_noalloc(64, -0.5, 0.5, vpos, boards.ptr, 1, ctypes.byref(csun),
                                d_pos.ptr, d_mask.ptr, None)
    assert rc == 2  # CG_ERR_OUT_OF_RANGE
    assert b"CG_NOALLOC_MAX_TEXELS" in lib.cg_last_error()
