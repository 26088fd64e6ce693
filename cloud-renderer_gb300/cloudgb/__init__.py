"""cloudgb -- host-side mirror of the reference's cloud-rendering classes over
the libcloudgb C ABI (include/cloudgb.h).

Class and field names follow the reference (jaafersheriff/Cloud-Renderer):
CloudVolume (src/CloudVolume.hpp:12-55), Sun (src/Sun.hpp:10-44), Camera
(src/Camera.hpp:12-46), VoxelizeShader (src/Shaders/VoxelizeShader.hpp:10-35)
and ConeTraceShader (src/Shaders/ConeTraceShader.hpp:8-44).  Every call runs on
the GPU through libcloudgb.so; errors raise CloudError with the library's
message.
"""
import ctypes
import math

import numpy as np

from . import _lib
from ._lib import (CONE_REFERENCE, CONE_TRANSMITTANCE, FORMAT_BF16_FP16, FORMAT_RGBA32F,
                   CloudError, check, load)

__all__ = ["Context", "CloudVolume", "Sun", "Camera", "VoxelizeShader", "ConeTraceShader",
           "CompatShader", "FrameGraph", "CloudError", "FORMAT_RGBA32F", "FORMAT_BF16_FP16", "CONE_TRANSMITTANCE",
           "CONE_REFERENCE", "default_context", "HostBuffer", "DeviceBuffer"]


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class Context:
    """One device and its stream (the GL context of Window::init, Window.cpp:54-106)."""

    def __init__(self, device=0):
        self._lib = load()
        h = ctypes.c_void_p()
        check(self._lib.cg_context_create(device, ctypes.byref(h)), "cg_context_create")
        self.handle = h
        self.device = device

    def synchronize(self):
        check(self._lib.cg_context_synchronize(self.handle), "cg_context_synchronize")

    @property
    def launch_count(self):
        return int(self._lib.cg_context_launch_count(self.handle))

    def set_timing(self, on=True):
        check(self._lib.cg_context_set_timing(self.handle, 1 if on else 0), "cg_context_set_timing")

    def stage_times(self):
        """{stage: ms} of the last voxelize/render call made with timing on."""
        ms = (ctypes.c_float * 32)()
        n = ctypes.c_int()
        names = ctypes.create_string_buffer(1024)
        check(self._lib.cg_context_stage_times(self.handle, ms, 32, ctypes.byref(n), names, 1024),
              "cg_context_stage_times")
        keys = names.value.decode().split(";") if n.value else []
        return {k: float(ms[i]) for i, k in enumerate(keys)}

    def mlp_fallbacks(self):
        v = ctypes.c_uint64()
        check(self._lib.cg_context_mlp_fallbacks(self.handle, ctypes.byref(v)),
              "cg_context_mlp_fallbacks")
        return int(v.value)

    def last_samples(self):
        """View samples the last surrogate render shaded."""
        v = ctypes.c_uint64()
        check(self._lib.cg_context_last_samples(self.handle, ctypes.byref(v)),
              "cg_context_last_samples")
        return int(v.value)

    def error_stats(self, image, reference):
        """GPU FP64 error statistics of an (H, W, 4) float32 image against a
        reference of the same shape (float64 or float32): dict of max-abs and
        RMSE per channel and overall."""
        img = np.ascontiguousarray(image, np.float32)
        ref = np.asarray(reference)
        f64 = ref.dtype == np.float64
        ref = np.ascontiguousarray(ref, np.float64 if f64 else np.float32)
        if img.shape != ref.shape or img.shape[-1] != 4:
            raise ValueError("error_stats: image and reference must be (..., 4) of equal shape")
        out = (ctypes.c_double * 10)()
        check(self._lib.cg_image_error_stats(self.handle, img.ctypes.data_as(ctypes.c_void_p),
                                             ref.ctypes.data_as(ctypes.c_void_p), 1 if f64 else 0,
                                             img.size // 4, 0, out, None),
              "cg_image_error_stats")
        return {"max_abs": list(out[0:4]), "rmse": list(out[4:8]), "max_abs_all": out[8],
                "rmse_all": out[9]}

    # ---- many volumes and views per frame
    @staticmethod
    def _views(views):
        def addr(p):
            return p.value if isinstance(p, ctypes.c_void_p) else int(p)
        arr = (_lib.cg_batch_view * len(views))()
        for i, (vol, cam, out) in enumerate(views):
            arr[i].volume = addr(vol.handle)
            arr[i].camera = cam._c()
            arr[i].rgba_out = addr(out.ptr)
        return arr

    def render_batch(self, views, shader, config=None, stream=None):
        """Render [(CloudVolume, Camera, DeviceBuffer)] in one persistent
        launch (plain FP32 method).  config: (lanes_per_ray, step_unroll,
        brick) or None for the context's."""
        arr = self._views(views)
        p = shader.params()
        cfg = None
        if config is not None:
            cfg = _lib.cg_trace_config(*config)
        check(self._lib.cg_render_batch(self.handle, arr, len(views), ctypes.byref(p),
                                        ctypes.byref(cfg) if cfg is not None else None,
                                        stream),
              "cg_render_batch")

    @property
    def trace_config(self):
        c = _lib.cg_trace_config()
        check(self._lib.cg_context_get_trace_config(self.handle, ctypes.byref(c)),
              "cg_context_get_trace_config")
        return (c.lanes_per_ray, c.step_unroll, c.brick)

    @trace_config.setter
    def trace_config(self, config):
        c = _lib.cg_trace_config(*config)
        check(self._lib.cg_context_set_trace_config(self.handle, ctypes.byref(c)),
              "cg_context_set_trace_config")

    def autotune(self, views, shader, repeats=3):
        """Time the 36 launch shapes on a batch; returns (best, {config: ms})."""
        arr = self._views(views)
        p = shader.params()
        best = _lib.cg_trace_config()
        ms = (ctypes.c_float * 36)()
        check(self._lib.cg_autotune(self.handle, arr, len(views), ctypes.byref(p), int(repeats),
                                    ctypes.byref(best), ms), "cg_autotune")
        table, k = {}, 0
        for lanes in (1, 4, 8, 32):
            for unroll in (1, 2, 4):
                for brick in (4, 8, 16):
                    table[(lanes, unroll, brick)] = float(ms[k])
                    k += 1
        return (best.lanes_per_ray, best.step_unroll, best.brick), table

    def close(self):
        if self.handle:
            self._lib.cg_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class HostBuffer:
    """Pinned host memory from cg_host_alloc, viewed as a numpy array."""

    def __init__(self, shape, dtype=np.float32):
        self._lib = load()
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = ctypes.c_void_p()
        check(self._lib.cg_host_alloc(self.nbytes, ctypes.byref(p)), "cg_host_alloc")
        self.ptr = p
        buf = (ctypes.c_char * self.nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self._lib.cg_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DeviceBuffer:
    """Device memory from cg_device_alloc."""

    def __init__(self, nbytes):
        self._lib = load()
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        check(self._lib.cg_device_alloc(self.nbytes, ctypes.byref(p)), "cg_device_alloc")
        self.ptr = p

    def upload(self, arr):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        check(self._lib.cg_memcpy(self.ptr, arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes,
                                  _lib.MEMCPY_H2D), "cg_memcpy")

    def download(self, shape, dtype=np.float32):
        out = np.empty(shape, dtype)
        check(self._lib.cg_memcpy(out.ctypes.data_as(ctypes.c_void_p), self.ptr, out.nbytes,
                                  _lib.MEMCPY_D2H), "cg_memcpy")
        return out

    def free(self):
        if self.ptr:
            self._lib.cg_device_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Sun:
    """Directional sun (Sun.hpp:10-44).  `direction` points toward the sun;
    the sun-view position map is map_width x map_height texels (the reference
    sizes it to the window, 1280x720, main.cpp:25-26)."""

    def __init__(self, direction=(0.3, 1.0, 0.2), map_width=1280, map_height=720):
        d = np.asarray(direction, np.float64)
        self.direction = tuple(float(x) for x in (d / np.sqrt((d * d).sum())))
        self.map_width = int(map_width)
        self.map_height = int(map_height)

    def _c(self):
        s = _lib.cg_sun()
        s.direction[:] = [float(x) for x in self.direction]
        s.map_width = self.map_width
        s.map_height = self.map_height
        return s


class Camera:
    """Pinhole camera (Camera::getP/getV, Camera.cpp:59-60)."""

    def __init__(self, eye, target, up=(0.0, 1.0, 0.0), fov_y_degrees=60.0, width=256,
                 height=256):
        self.eye = tuple(float(x) for x in eye)
        self.target = tuple(float(x) for x in target)
        self.up = tuple(float(x) for x in up)
        self.fov_y_degrees = float(fov_y_degrees)
        self.width = int(width)
        self.height = int(height)

    def _c(self):
        c = _lib.cg_camera()
        c.eye[:] = list(self.eye)
        c.target[:] = list(self.target)
        c.up[:] = list(self.up)
        c.fov_y_degrees = self.fov_y_degrees
        c.width = self.width
        c.height = self.height
        return c

    def getPosition(self):
        return self.eye


class CloudVolume:
    """CloudVolume(int dim, vec2 bounds, vec3 position, int mips) (CloudVolume.cpp:7-55).

    The world box is position + [bounds[0], bounds[1]]^3.  Billboards hold
    positions relative to `position`, radii (`scales`) and per-board
    densities; `fluffiness` multiplies the radii at upload."""

    def __init__(self, dim, bounds, position, mips, fmt=FORMAT_RGBA32F, ctx=None):
        self.ctx = ctx or default_context()
        self._lib = self.ctx._lib
        self.dimension = int(dim)
        self.position = tuple(float(x) for x in position)
        self.xBounds = self.yBounds = self.zBounds = (float(bounds[0]), float(bounds[1]))
        self.levels = int(mips)
        self.format = int(fmt)
        r = self.xBounds[1] - self.xBounds[0]
        self.range = (r, r, r)
        self.voxelSize = tuple(x / self.dimension for x in self.range)
        self.fluffiness = 1.0
        self.positions = np.zeros((0, 3), np.float32)
        self.scales = np.zeros((0,), np.float32)
        self.densities = np.zeros((0,), np.float32)
        self._regen = None
        pos = (ctypes.c_float * 3)(*self.position)
        h = ctypes.c_void_p()
        check(self._lib.cg_volume_create(self.ctx.handle, self.dimension, self.xBounds[0],
                                         self.xBounds[1], pos, self.levels, self.format,
                                         ctypes.byref(h)), "cg_volume_create")
        self.handle = h

    # -- billboards (CloudVolume.cpp:58-62, 120-164) --
    @property
    def count(self):
        return int(self.positions.shape[0])

    def set_billboards(self, positions, scales, densities=None):
        self.positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        self.scales = np.ascontiguousarray(scales, np.float32).reshape(-1)
        if densities is None:
            densities = np.ones(self.scales.shape, np.float32)
        self.densities = np.ascontiguousarray(densities, np.float32).reshape(-1)

    def addCloudBoard(self, pos, scale, density=1.0):
        self.positions = np.concatenate([self.positions, np.asarray([pos], np.float32)])
        self.scales = np.concatenate([self.scales, np.asarray([scale], np.float32)])
        self.densities = np.concatenate([self.densities, np.asarray([density], np.float32)])

    def regenerateBillboards(self, count, minOffset, maxOffset, minScale, maxScale, seed=0):
        """Uniform offsets in [minOffset, maxOffset] and scales in
        [minScale, maxScale] (CloudVolume.cpp:120-133), from a seeded stream."""
        from .scene import SplitMix64
        rng = SplitMix64(seed)
        lo = np.asarray(minOffset, np.float64) * np.ones(3)
        hi = np.asarray(maxOffset, np.float64) * np.ones(3)
        u = rng.uniform(3 * count).reshape(count, 3)
        pos = (lo + (hi - lo) * u).astype(np.float32)
        sc = rng.uniform_range(count, minScale, maxScale).astype(np.float32)
        self._regen = (count, minOffset, maxOffset, minScale, maxScale, seed)
        self.set_billboards(pos, sc)

    def resetBillboards(self):
        if self._regen:
            self.regenerateBillboards(*self._regen)

    def sortBoards(self, point):
        """Far-to-near order by distance to `point` (CloudVolume.cpp:65-82).
        The renderer composites front to back per pixel and does not need it;
        it only changes which board wins a sun-map depth tie."""
        c = np.asarray(self.position, np.float32) + self.positions
        d = np.sqrt(((c - np.asarray(point, np.float32)) ** 2).sum(axis=1))
        order = np.argsort(-d, kind="stable")
        self.set_billboards(self.positions[order], self.scales[order], self.densities[order])

    def update(self):
        """Upload the billboard list (CloudVolume::update, CloudVolume.cpp:84-93)."""
        self.uploadBillboards()

    def uploadBillboards(self):
        n = self.count
        check(self._lib.cg_volume_set_billboards(self.handle, _fptr(self.positions),
                                                 _fptr(self.scales), _fptr(self.densities), n,
                                                 float(self.fluffiness)),
              "cg_volume_set_billboards")

    def clearGPU(self):
        """The volume is cleared by every voxelize (CloudVolume.cpp:96-100)."""

    # -- index helpers (CloudVolume.cpp:103-118) --
    def get3DIndices(self, index):
        line = self.dimension
        sl = self.dimension * line
        z = index // sl
        y = (index - z * sl) // line
        x = index - z * sl - y * line
        return (x, y, z)

    def reverseVoxelIndex(self, idx):
        return tuple(float(idx[a]) * self.range[a] / self.dimension + self.xBounds[0]
                     for a in range(3))

    # -- readback (VoxelShader::updateVoxelData, VoxelShader.cpp:102-133) --
    def set_occupancy_brick(self, brick):
        """Edge (4, 8 or 16 texels) of the empty-space bricks; images do not
        depend on it."""
        check(self._lib.cg_volume_set_occupancy_brick(self.handle, int(brick)),
              "cg_volume_set_occupancy_brick")

    def info(self):
        inf = _lib.cg_volume_info()
        check(self._lib.cg_volume_get_info(self.handle, ctypes.byref(inf)), "cg_volume_get_info")
        return inf

    def read_level(self, level):
        n = max(1, self.dimension >> level)
        if self.format == FORMAT_RGBA32F:
            out = np.empty((n, n, n, 4), np.float32)
        else:
            out = np.empty((n, n, n), np.uint32)
        check(self._lib.cg_volume_read_level(self.handle, level,
                                             out.ctypes.data_as(ctypes.c_void_p), out.nbytes),
              "cg_volume_read_level")
        return out

    def read_coverage(self):
        D = self.dimension
        cnt = np.empty((D, D, D), np.uint32)
        dq = np.empty((D, D, D), np.uint32)
        check(self._lib.cg_volume_read_coverage(
            self.handle, cnt.ctypes.data_as(_lib.U32P), dq.ctypes.data_as(_lib.U32P)),
            "cg_volume_read_coverage")
        return cnt, dq

    def read_sun_map(self, sun):
        keys = np.empty((sun.map_height, sun.map_width), np.uint64)
        pos = np.empty((sun.map_height, sun.map_width, 4), np.float32)
        check(self._lib.cg_volume_read_sun_map(self.handle, keys.ctypes.data_as(_lib.U64P),
                                               _fptr(pos)), "cg_volume_read_sun_map")
        return keys, pos

    def read_highlight(self):
        D = self.dimension
        m = np.empty((D, D, D), np.uint8)
        check(self._lib.cg_volume_read_highlight(self.handle, m.ctypes.data_as(_lib.U8P)),
              "cg_volume_read_highlight")
        return m

    def activeVoxels(self):
        v = ctypes.c_uint64()
        check(self._lib.cg_volume_active_voxels(self.handle, ctypes.byref(v)),
              "cg_volume_active_voxels")
        return int(v.value)

    def close(self):
        if self.handle:
            self._lib.cg_volume_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class VoxelizeShader:
    """VoxelizeShader::voxelize(CloudVolume*) (VoxelizeShader.cpp:18-31)."""

    def voxelize(self, volume, sun, stream=None):
        s = sun._c()
        check(self._lib().cg_voxelize(volume.handle, ctypes.byref(s), stream), "cg_voxelize")

    @staticmethod
    def _lib():
        return load()


class ConeTraceShader:
    """ConeTraceShader::coneTrace(CloudVolume*) (ConeTraceShader.cpp:15-82).

    Field names follow ConeTraceShader.hpp:15-32.  vctConeAngle is the full
    cone aperture as in the reference (its half is the cone half-angle);
    freqStep / persStep are the fBm lacunarity / gain.  The noise domain moves
    with the wind: offset = windVel * runTime in base-frequency lattice units
    (the reference's octaveOffsets, ConeTraceShader.cpp:55-61, with runTime its
    Window::runTime, here set by the caller)."""

    def __init__(self, **kw):
        p = _lib.cg_render_params()
        load().cg_render_params_default(ctypes.byref(p))
        self.viewSteps = p.view_steps
        self.vctSteps = p.sun_steps
        self.vctConeAngle = 2.0 * p.cone_half_angle
        self.vctConeInitialHeight = p.cone_initial_height
        self.vctConeMinRadius = p.cone_min_radius
        self.vctLodOffset = p.lod_offset
        self.vctDownScaling = p.down_scaling
        self.densityScale = p.density_scale
        self.ambient = p.ambient
        self.sunColor = tuple(p.sun_color)
        self.transmittanceCutoff = p.transmittance_cutoff
        self.coneMode = p.cone_mode
        self.noiseSeed = p.noise.seed
        self.numOctaves = p.noise.octaves
        self.noiseFrequency = p.noise.frequency
        self.freqStep = p.noise.lacunarity
        self.persStep = p.noise.gain
        self.windVel = (0.01, 0.0, 0.0)
        self.runTime = 0.0
        self.useMlp = False
        self.mlp = None
        self.pipeline = p.pipeline
        self.coneLanes = p.cone_lanes
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"ConeTraceShader has no parameter {k!r}")
            setattr(self, k, v)

    def params(self):
        p = _lib.cg_render_params()
        p.view_steps = int(self.viewSteps)
        p.sun_steps = int(self.vctSteps)
        p.cone_half_angle = float(self.vctConeAngle) / 2.0
        p.cone_initial_height = float(self.vctConeInitialHeight)
        p.cone_min_radius = float(self.vctConeMinRadius)
        p.lod_offset = float(self.vctLodOffset)
        p.down_scaling = float(self.vctDownScaling)
        p.density_scale = float(self.densityScale)
        p.ambient = float(self.ambient)
        p.sun_color[:] = [float(x) for x in self.sunColor]
        p.transmittance_cutoff = float(self.transmittanceCutoff)
        p.cone_mode = int(self.coneMode)
        p.noise.seed = int(self.noiseSeed) & 0xFFFFFFFF
        p.noise.octaves = int(self.numOctaves)
        p.noise.frequency = float(self.noiseFrequency)
        p.noise.lacunarity = float(self.freqStep)
        p.noise.gain = float(self.persStep)
        p.noise.offset[:] = [float(w) * float(self.runTime) for w in self.windVel]
        p.use_mlp = 1 if self.useMlp else 0
        p.mlp = self.mlp.handle if (self.useMlp and self.mlp is not None) else None
        p.pipeline = int(self.pipeline)
        p.cone_lanes = int(self.coneLanes)
        return p

    def coneTrace(self, volume, camera, out=None, stream=None):
        """Render `camera`'s view of `volume`; returns an H x W x 4 float32 image
        (row 0 = top).  `out` may be a numpy array, a HostBuffer (pinned) or a
        DeviceBuffer (result left on the device)."""
        p = self.params()
        c = camera._c()
        lib = load()
        if isinstance(out, DeviceBuffer):
            check(lib.cg_render(volume.ctx.handle, volume.handle, ctypes.byref(c), ctypes.byref(p),
                                out.ptr, 1, stream), "cg_render")
            return out
        if isinstance(out, HostBuffer):
            arr = out.array
        elif out is None:
            arr = np.empty((camera.height, camera.width, 4), np.float32)
        else:
            arr = out
        assert arr.dtype == np.float32 and arr.flags["C_CONTIGUOUS"]
        assert arr.size >= camera.width * camera.height * 4
        check(lib.cg_render(volume.ctx.handle, volume.handle, ctypes.byref(c), ctypes.byref(p),
                            arr.ctypes.data_as(ctypes.c_void_p), 0, stream), "cg_render")
        return arr

    def renderStats(self, volume, camera):
        """Executed-work counters of one render: view samples, sun cones,
        sun-cone samples, pixels whose ray met the box."""
        p = self.params()
        c = camera._c()
        out = (ctypes.c_uint64 * 4)()
        check(load().cg_render_stats(volume.ctx.handle, volume.handle, ctypes.byref(c),
                                     ctypes.byref(p), out), "cg_render_stats")
        return dict(view_samples=int(out[0]), sun_cones=int(out[1]), sun_samples=int(out[2]),
                    hit_pixels=int(out[3]))

    def traceCone(self, volume, positions, direction):
        """traceCone at level-0 voxel-space positions (conetrace_frag.glsl:64-79)."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        out = np.empty((pos.shape[0],), np.float32)
        d = (ctypes.c_float * 3)(*[float(x) for x in direction])
        p = self.params()
        check(load().cg_trace_cones(volume.handle, pos.ctypes.data_as(ctypes.c_void_p),
                                    pos.shape[0], d, ctypes.byref(p),
                                    out.ctypes.data_as(ctypes.c_void_p), 0, None),
              "cg_trace_cones")
        return out

    @staticmethod
    def half_angle_to_cone_angle(half):
        return 2.0 * half


class CompatShader:
    """The reference's own image formation (ConeTraceShader::coneTrace,
    ConeTraceShader.cpp:15-82): one camera-facing billboard per board shaded
    by its fragment program (soft-particle noise, traceCone from the sphere
    surface) and blended in distance order over the clear colour.  Field
    names and defaults follow ConeTraceShader.hpp:15-32; octaveOffsets =
    windVel * runTime (ConeTraceShader.cpp:55-61)."""

    _FIELDS = dict(showQuad="show_quad", doNoiseSample="do_noise", doConeTrace="do_cone_trace",
                   stepSize="step_size", noiseOpacity="noise_opacity", numOctaves="num_octaves",
                   freqStep="freq_step", persStep="pers_step", adjustSize="adjust_size",
                   minNoiseSteps="min_noise_steps", maxNoiseSteps="max_noise_steps",
                   minNoiseColor="min_noise_color", noiseColorScale="noise_color_scale",
                   noiseSeed="noise_seed", vctSteps="vct_steps", vctConeAngle="vct_cone_angle",
                   vctConeInitialHeight="vct_cone_initial_height",
                   vctLodOffset="vct_lod_offset", vctDownScaling="vct_down_scaling",
                   nearPlane="near_plane", transmittanceCutoff="transmittance_cutoff")

    def __init__(self, **kw):
        p = _lib.cg_compat_params()
        load().cg_compat_params_default(ctypes.byref(p))
        for name, field in self._FIELDS.items():
            v = getattr(p, field)
            setattr(self, name, bool(v) if field in ("show_quad", "do_noise", "do_cone_trace")
                    else v)
        self.clearColor = tuple(p.clear_color)
        self.windVel = (0.01, 0.0, 0.0)
        self.runTime = 0.0
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"CompatShader has no parameter {k!r}")
            setattr(self, k, v)

    def params(self):
        p = _lib.cg_compat_params()
        for name, field in self._FIELDS.items():
            v = getattr(self, name)
            ftype = dict(p._fields_)[field]
            setattr(p, field, int(v) & 0xFFFFFFFF if field == "noise_seed" else
                    (int(v) if ftype is ctypes.c_int else float(v)))
        p.clear_color[:] = [float(x) for x in self.clearColor]
        p.octave_offsets[:] = [float(w) * float(self.runTime) for w in self.windVel]
        return p

    def coneTrace(self, volume, camera, out=None, stream=None):
        """The compat image of camera over volume's boards: H x W x 4 float32
        (row 0 = top); `out` as in ConeTraceShader.coneTrace."""
        p = self.params()
        c = camera._c()
        lib = load()
        if isinstance(out, DeviceBuffer):
            check(lib.cg_render_compat(volume.ctx.handle, volume.handle, ctypes.byref(c),
                                       ctypes.byref(p), out.ptr, 1, stream), "cg_render_compat")
            return out
        if isinstance(out, HostBuffer):
            arr = out.array
        elif out is None:
            arr = np.empty((camera.height, camera.width, 4), np.float32)
        else:
            arr = out
        assert arr.dtype == np.float32 and arr.flags["C_CONTIGUOUS"]
        assert arr.size >= camera.width * camera.height * 4
        check(lib.cg_render_compat(volume.ctx.handle, volume.handle, ctypes.byref(c),
                                   ctypes.byref(p), arr.ctypes.data_as(ctypes.c_void_p), 0,
                                   stream), "cg_render_compat")
        return arr

    @staticmethod
    def noise_map(seed):
        """The decoded 32^3 RGBA noise map of a seed: (32, 32, 32, 4) float32."""
        out = np.empty((32, 32, 32, 4), np.float32)
        check(load().cg_compat_noise_map(int(seed) & 0xFFFFFFFF,
                                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
              "cg_compat_noise_map")
        return out


def deg(x):
    return math.degrees(x)


class FrameGraph:
    """A frame (voxelize every volume, then one batch render of the views) as
    one CUDA graph, replayed by launch()."""

    def __init__(self, ctx, volumes, sun, views, shader):
        self.ctx = ctx
        self._lib = load()
        vols = (ctypes.c_void_p * len(volumes))(
            *[v.handle.value if isinstance(v.handle, ctypes.c_void_p) else v.handle
              for v in volumes])
        arr = Context._views(views)
        p = shader.params()
        s = sun._c()
        h = ctypes.c_void_p()
        check(self._lib.cg_frame_graph_create(ctx.handle, vols, len(volumes), ctypes.byref(s), arr,
                                              len(views), ctypes.byref(p), ctypes.byref(h)),
              "cg_frame_graph_create")
        self.handle = h

    def launch(self, stream=None):
        check(self._lib.cg_frame_graph_launch(self.handle, stream), "cg_frame_graph_launch")

    def close(self):
        if self.handle:
            self._lib.cg_frame_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

