"""ctypes binding of oracle/_ref/libref_shaders.so: the reference's own shader
code (compiled through oracle/ref_shim/) run on the CPU.  TEST INFRASTRUCTURE
ONLY -- used by tests/golden/make_golden.py and by the tests that check the
oracle against it where the library exists."""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_shaders.so")
FP = ctypes.POINTER(ctypes.c_float)
IP = ctypes.POINTER(ctypes.c_int)
LP = ctypes.POINTER(ctypes.c_long)
_lib = None


def available():
    return os.path.exists(LIB)


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(LIB)
        lib.ref_sun_pass.restype = ctypes.c_long
        lib.ref_sun_pass.argtypes = [FP, FP, ctypes.c_int, FP, ctypes.c_float, ctypes.c_float, FP,
                                     ctypes.c_int, ctypes.c_int, FP, IP, FP]
        lib.ref_second_pass.restype = None
        lib.ref_second_pass.argtypes = [FP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_float, ctypes.c_float, FP, ctypes.c_void_p]
        lib.ref_compat_render.restype = ctypes.c_long
        lib.ref_compat_render.argtypes = [FP, FP, ctypes.c_int, FP, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_int, FP, IP, LP, ctypes.c_int,
                                          FP, FP, FP, FP, ctypes.c_float, ctypes.c_int,
                                          ctypes.c_int, FP, ctypes.c_void_p, FP]
        lib.ref_trace_cone.restype = ctypes.c_float
        lib.ref_trace_cone.argtypes = [FP, IP, LP, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                       ctypes.c_float, FP, FP, FP, ctypes.c_int, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_float, ctypes.c_float, FP]
        _lib = lib
    return _lib


def _f(a):
    return np.ascontiguousarray(a, np.float32)


def sun_pass(board_pos, board_scale, vol_pos, bounds, sun_dir, W, H):
    """first_voxelize (+ billboard_vert_instanced) over the boards ->
    (posmap (H, W, 4), winner (H, W), depth (H, W), fragments shaded)."""
    lib = load()
    bp, bs = _f(board_pos).reshape(-1, 3), _f(board_scale).reshape(-1)
    pm = np.empty((H, W, 4), np.float32)
    win = np.empty((H, W), np.int32)
    dep = np.empty((H, W), np.float32)
    vp, sd = _f(vol_pos), _f(sun_dir)
    n = lib.ref_sun_pass(bp.ctypes.data_as(FP), bs.ctypes.data_as(FP), bp.shape[0],
                         vp.ctypes.data_as(FP), float(bounds[0]), float(bounds[1]),
                         sd.ctypes.data_as(FP), W, H, pm.ctypes.data_as(FP),
                         win.ctypes.data_as(IP), dep.ctypes.data_as(FP))
    return pm, win, dep, int(n)


def second_pass(posmap, D, vol_pos, bounds):
    """second_voxelize over a position map -> (D, D, D) uint8 marks (1 = stored)."""
    lib = load()
    pm = _f(posmap)
    H, W = pm.shape[:2]
    marks = np.empty((D, D, D), np.uint8)
    vp = _f(vol_pos)
    lib.ref_second_pass(pm.ctypes.data_as(FP), W, H, D, float(bounds[0]), float(bounds[1]),
                        vp.ctypes.data_as(FP), marks.ctypes.data)
    return (marks > 0).astype(np.uint8)


def trace_cone(levels, D, vol_pos, bounds, world_pos, direction, steps, cone_angle, cone_h0,
               lod_offset=0.0, down_scaling=1.0):
    """traceCone over a one-channel mip chain (list of (n, n, n) arrays) ->
    (value, voxel-space start position)."""
    lib = load()
    flat = _f(np.concatenate([np.asarray(l, np.float32).reshape(-1) for l in levels]))
    dims = np.array([l.shape[0] for l in levels], np.int32)
    offs = np.zeros(len(levels), np.int64)
    offs[1:] = np.cumsum([l.size for l in levels])[:-1]
    offs = offs.astype(np.int64)
    vp, wp, dr = _f(vol_pos), _f(world_pos), _f(direction)
    out = np.empty(3, np.float32)
    v = lib.ref_trace_cone(flat.ctypes.data_as(FP), dims.ctypes.data_as(IP),
                           offs.ctypes.data_as(LP), len(levels), D, float(bounds[0]),
                           float(bounds[1]), vp.ctypes.data_as(FP), wp.ctypes.data_as(FP),
                           dr.ctypes.data_as(FP), int(steps), float(cone_angle), float(cone_h0),
                           float(lod_offset), float(down_scaling), out.ctypes.data_as(FP))
    return float(v), out


def compat_render(board_pos, board_scale, vol_pos, bounds, D, light_levels, noise_map, eye,
                  target, up, fov_deg, W, H, sun_dir, params):
    """The reference's cone-trace pass (billboards shaded by its fragment
    shader, sorted and blended as its host code does) -> ((H, W, 4) float32
    image, row 0 = top; fragments shaded).  light_levels: the light channel's
    mip chain; params: an or_compat_params (or the same layout)."""
    lib = load()
    bp, bs = _f(board_pos).reshape(-1), _f(board_scale).reshape(-1)
    flat = _f(np.concatenate([np.asarray(l, np.float32).reshape(-1) for l in light_levels]))
    dims = np.array([l.shape[0] for l in light_levels], np.int32)
    offs = np.zeros(len(light_levels), np.int64)
    offs[1:] = np.cumsum([l.size for l in light_levels])[:-1]
    nm = _f(noise_map).reshape(-1)
    out = np.empty((H, W, 4), np.float32)
    f3 = [_f(x) for x in (vol_pos, eye, target, up, sun_dir)]
    pbuf = ctypes.create_string_buffer(bytes(params), len(bytes(params)))
    shaded = lib.ref_compat_render(
        bp.ctypes.data_as(FP), bs.ctypes.data_as(FP), int(bs.shape[0]), f3[0].ctypes.data_as(FP),
        float(bounds[0]), float(bounds[1]), int(D), flat.ctypes.data_as(FP),
        dims.ctypes.data_as(IP), offs.ctypes.data_as(LP), len(light_levels),
        nm.ctypes.data_as(FP), f3[1].ctypes.data_as(FP), f3[2].ctypes.data_as(FP),
        f3[3].ctypes.data_as(FP), float(fov_deg), int(W), int(H), f3[4].ctypes.data_as(FP),
        ctypes.cast(pbuf, ctypes.c_void_p), out.ctypes.data_as(FP))
    return out, int(shaded)
