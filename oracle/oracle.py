"""ctypes wrapper of the CPU oracle (oracle/cloud_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never loads it.
Parity status: see the header of cloud_oracle.c.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBS = {64: os.path.join(HERE, "liboracle64.so"), 32: os.path.join(HERE, "liboracle32.so")}


class or_params(ctypes.Structure):
    _fields_ = [("view_steps", ctypes.c_int), ("sun_steps", ctypes.c_int),
                ("cone_half_angle", ctypes.c_float), ("cone_initial_height", ctypes.c_float),
                ("cone_min_radius", ctypes.c_float), ("lod_offset", ctypes.c_float),
                ("down_scaling", ctypes.c_float), ("density_scale", ctypes.c_float),
                ("ambient", ctypes.c_float), ("sun_color", ctypes.c_float * 3),
                ("transmittance_cutoff", ctypes.c_float), ("cone_mode", ctypes.c_int),
                ("noise_seed", ctypes.c_uint32), ("noise_octaves", ctypes.c_int),
                ("noise_frequency", ctypes.c_float), ("noise_lacunarity", ctypes.c_float),
                ("noise_gain", ctypes.c_float), ("noise_offset", ctypes.c_float * 3)]


class or_sun_frame(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("right", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3), ("fwd", ctypes.c_float * 3),
                ("t", ctypes.c_float * 3), ("lo", ctypes.c_float), ("hi", ctypes.c_float),
                ("near_z", ctypes.c_float), ("clip", ctypes.c_float), ("W", ctypes.c_int),
                ("H", ctypes.c_int)]


class or_compat_params(ctypes.Structure):
    """Mirror of or_compat_params (the same layout as the product's
    cg_compat_params)."""
    _fields_ = [("show_quad", ctypes.c_int), ("do_noise", ctypes.c_int),
                ("do_cone_trace", ctypes.c_int), ("step_size", ctypes.c_float),
                ("noise_opacity", ctypes.c_float), ("num_octaves", ctypes.c_int),
                ("freq_step", ctypes.c_float), ("pers_step", ctypes.c_float),
                ("adjust_size", ctypes.c_float), ("min_noise_steps", ctypes.c_int),
                ("max_noise_steps", ctypes.c_int), ("min_noise_color", ctypes.c_float),
                ("noise_color_scale", ctypes.c_float), ("octave_offsets", ctypes.c_float * 3),
                ("noise_seed", ctypes.c_uint32), ("vct_steps", ctypes.c_int),
                ("vct_cone_angle", ctypes.c_float), ("vct_cone_initial_height", ctypes.c_float),
                ("vct_lod_offset", ctypes.c_float), ("vct_down_scaling", ctypes.c_float),
                ("clear_color", ctypes.c_float * 4), ("near_plane", ctypes.c_float),
                ("transmittance_cutoff", ctypes.c_float)]


class or_camera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_double * 3), ("target", ctypes.c_double * 3),
                ("up", ctypes.c_double * 3), ("fov_y_degrees", ctypes.c_double),
                ("width", ctypes.c_int), ("height", ctypes.c_int)]


_libs = {}
P = ctypes.c_void_p
I = ctypes.c_int
F = ctypes.c_float
FP = ctypes.POINTER(ctypes.c_float)
DP = ctypes.POINTER(ctypes.c_double)


def load(bits=64):
    if bits in _libs:
        return _libs[bits]
    path = LIBS[bits]
    if not os.path.exists(path):
        raise ImportError(f"{path} missing: run `python oracle/build_oracle.py`")
    lib = ctypes.CDLL(path)
    sig = {
        "or_volume_new": (P, [I, F, F, FP, I]),
        "or_volume_free": (None, [P]),
        "or_volume_total": (I, [P]),
        "or_volume_level_offset": (ctypes.c_long, [P, I]),
        "or_volume_level_dim": (I, [P, I]),
        "or_volume_set_boards": (I, [P, FP, FP, FP, I, F]),
        "or_volume_get_quantized": (None, [P, P, P, P, P, P]),
        "or_volume_voxelize": (I, [P, FP, I, I, I]),
        "or_volume_get_coverage": (None, [P, P, P]),
        "or_volume_get_mask": (None, [P, P]),
        "or_volume_get_sun_map": (None, [P, P, P]),
        "or_volume_get_frame": (None, [P, ctypes.POINTER(or_sun_frame)]),
        "or_volume_get_pyramid": (None, [P, DP]),
        "or_volume_set_pyramid": (None, [P, DP]),
        "or_volume_rebuild_mips": (None, [P, I]),
        "or_sun_frame_make": (I, [FP, F, F, FP, I, I, ctypes.POINTER(or_sun_frame)]),
        "or_highlight_offset": (F, [P]),
        "or_highlight_posmap": (None, [P, FP, I, I, P]),
        "or_sample": (ctypes.c_double, [P, DP, ctypes.c_double, I, I]),
        "or_trace_cone": (ctypes.c_double, [P, DP, DP, ctypes.POINTER(or_params)]),
        "or_pcg3d": (None, [ctypes.POINTER(ctypes.c_uint32)]),
        "or_lattice": (ctypes.c_double, [I, I, I, ctypes.c_uint32, I]),
        "or_fbm": (ctypes.c_double, [DP, ctypes.POINTER(or_params)]),
        "or_render": (I, [P, ctypes.POINTER(or_camera), ctypes.POINTER(or_params), FP, I, I, I,
                          I, DP, P, I]),
        "or_real_bytes": (I, []),
        "or_compat_noise_map": (None, [ctypes.c_uint32, FP]),
        "or_compat_render": (I, [P, ctypes.POINTER(or_camera), ctypes.POINTER(or_compat_params),
                                 FP, FP, DP, I]),
        "or_mlp_features": (None, [P, DP, DP, I, ctypes.c_double, DP]),
        "or_mlp_forward": (ctypes.c_double, [DP, DP, DP, DP, I]),
        "or_mlp_loss_grad": (ctypes.c_double, [DP, DP, DP, ctypes.c_double, ctypes.c_double, DP,
                                               DP, I, DP, I]),
        "or_adam_step": (None, [DP, DP, DP, DP, I, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, I]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _libs[bits] = lib
    return lib


def _f3(v):
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def _d3(v):
    return (ctypes.c_double * 3)(*[float(x) for x in v])


def params_from_shader(shader):
    """or_params from a cloudgb.ConeTraceShader (same field meanings)."""
    p = or_params()
    p.view_steps = int(shader.viewSteps)
    p.sun_steps = int(shader.vctSteps)
    p.cone_half_angle = float(shader.vctConeAngle) / 2.0
    p.cone_initial_height = float(shader.vctConeInitialHeight)
    p.cone_min_radius = float(shader.vctConeMinRadius)
    p.lod_offset = float(shader.vctLodOffset)
    p.down_scaling = float(shader.vctDownScaling)
    p.density_scale = float(shader.densityScale)
    p.ambient = float(shader.ambient)
    p.sun_color[:] = [float(x) for x in shader.sunColor]
    p.transmittance_cutoff = float(shader.transmittanceCutoff)
    p.cone_mode = int(shader.coneMode)
    p.noise_seed = int(shader.noiseSeed) & 0xFFFFFFFF
    p.noise_octaves = int(shader.numOctaves)
    p.noise_frequency = float(shader.noiseFrequency)
    p.noise_lacunarity = float(shader.freqStep)
    p.noise_gain = float(shader.persStep)
    wind = getattr(shader, "windVel", (0.0, 0.0, 0.0))
    p.noise_offset[:] = [float(w) * float(getattr(shader, "runTime", 0.0)) for w in wind]
    return p


def make_params(**kw):
    p = or_params()
    defaults = dict(view_steps=64, sun_steps=24, cone_half_angle=0.03, cone_initial_height=1.0,
                    cone_min_radius=2.0, lod_offset=0.0, down_scaling=1.0, density_scale=4.0,
                    ambient=0.3, sun_color=(1.0, 1.0, 1.0), transmittance_cutoff=1e-5,
                    cone_mode=0, noise_seed=1, noise_octaves=0, noise_frequency=4.0,
                    noise_lacunarity=2.0, noise_gain=0.5)
    defaults.update(kw)
    for k, v in defaults.items():
        if k in ("sun_color", "noise_offset"):
            getattr(p, k)[:] = [float(x) for x in v]
        else:
            setattr(p, k, v)
    return p


class OracleVolume:
    def __init__(self, D, bounds, position, mips, bits=64):
        self.lib = load(bits)
        self.D, self.L = int(D), int(mips)
        self.h = self.lib.or_volume_new(self.D, float(bounds[0]), float(bounds[1]),
                                        _f3(position), self.L)
        if not self.h:
            raise ValueError("or_volume_new failed")
        self.map_size = None

    def __del__(self):
        try:
            if self.h:
                self.lib.or_volume_free(self.h)
                self.h = None
        except Exception:
            pass

    def set_boards(self, positions, scales, densities=None, fluffiness=1.0):
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        sc = np.ascontiguousarray(scales, np.float32).reshape(-1)
        self.n = pos.shape[0]
        dp = None
        if densities is not None:
            self._dens = np.ascontiguousarray(densities, np.float32).reshape(-1)
            dp = self._dens.ctypes.data_as(FP)
        rc = self.lib.or_volume_set_boards(self.h, pos.ctypes.data_as(FP), sc.ctypes.data_as(FP),
                                           dp, self.n, float(fluffiness))
        return rc

    def quantized(self):
        n = self.n
        q = np.empty((n, 3), np.int64)
        rq = np.empty(n, np.int64)
        thr = np.empty(n, np.uint64)
        dq = np.empty(n, np.uint32)
        cul = np.empty(n, np.uint8)
        self.lib.or_volume_get_quantized(self.h, q.ctypes.data, rq.ctypes.data, thr.ctypes.data,
                                         dq.ctypes.data, cul.ctypes.data)
        return q, rq, thr, dq, cul

    def voxelize(self, sun_dir, W=1280, H=720, threads=None):
        threads = threads or os.cpu_count() or 1
        self.map_size = (W, H)
        return self.lib.or_volume_voxelize(self.h, _f3(sun_dir), W, H, threads)

    def coverage(self):
        D = self.D
        c = np.empty((D, D, D), np.uint32)
        d = np.empty((D, D, D), np.uint32)
        self.lib.or_volume_get_coverage(self.h, c.ctypes.data, d.ctypes.data)
        return c, d

    def mask(self):
        D = self.D
        m = np.empty((D, D, D), np.uint8)
        self.lib.or_volume_get_mask(self.h, m.ctypes.data)
        return m

    def sun_map(self):
        W, H = self.map_size
        k = np.empty((H, W), np.uint64)
        p = np.empty((H, W, 4), np.float32)
        self.lib.or_volume_get_sun_map(self.h, k.ctypes.data, p.ctypes.data)
        return k, p

    def highlight_posmap(self, posmap):
        """Pass 2 alone over a given (H, W, 4) position map -> (D, D, D) marks."""
        pm = np.ascontiguousarray(posmap, np.float32)
        H, W = pm.shape[:2]
        m = np.empty((self.D,) * 3, np.uint8)
        self.lib.or_highlight_posmap(self.h, pm.ctypes.data_as(FP), W, H, m.ctypes.data)
        return m

    def frame(self):
        fr = or_sun_frame()
        self.lib.or_volume_get_frame(self.h, ctypes.byref(fr))
        return fr

    def pyramid(self):
        total = self.lib.or_volume_total(self.h)
        flat = np.empty(total * 4, np.float64)
        self.lib.or_volume_get_pyramid(self.h, flat.ctypes.data_as(DP))
        levels = []
        for l in range(self.L):
            off = self.lib.or_volume_level_offset(self.h, l)
            n = self.lib.or_volume_level_dim(self.h, l)
            levels.append(flat[off * 4:(off + n ** 3) * 4].reshape(n, n, n, 4))
        return levels

    def set_pyramid(self, levels):
        flat = np.ascontiguousarray(np.concatenate([l.reshape(-1) for l in levels]), np.float64)
        self.lib.or_volume_set_pyramid(self.h, flat.ctypes.data_as(DP))

    def rebuild_mips(self, threads=1):
        self.lib.or_volume_rebuild_mips(self.h, threads)

    def sample(self, p, lod, channel=0, border=1):
        return self.lib.or_sample(self.h, _d3(p), float(lod), int(channel), int(border))

    def trace_cone(self, p, direction, params):
        return self.lib.or_trace_cone(self.h, _d3(p), _d3(direction), ctypes.byref(params))

    def trace_cones(self, positions, direction, params):
        return np.array([self.trace_cone(p, direction, params) for p in positions])

    def render(self, camera, params, sun_dir, rect=None, threads=None, stats=False):
        """Render camera (a cloudgb.Camera-like object) over rect = (x0, y0, w, h)."""
        threads = threads or os.cpu_count() or 1
        c = or_camera()
        c.eye[:] = [float(x) for x in camera.eye]
        c.target[:] = [float(x) for x in camera.target]
        c.up[:] = [float(x) for x in camera.up]
        c.fov_y_degrees = float(camera.fov_y_degrees)
        c.width, c.height = int(camera.width), int(camera.height)
        x0, y0, w, h = rect if rect else (0, 0, camera.width, camera.height)
        out = np.zeros((h, w, 4), np.float64)
        st = np.zeros((h, 2), np.int64)
        self.lib.or_render(self.h, ctypes.byref(c), ctypes.byref(params), _f3(sun_dir), x0, y0, w,
                           h, out.ctypes.data_as(DP), st.ctypes.data_as(ctypes.c_void_p), threads)
        return (out, st) if stats else out


    def compat_render(self, camera, params, sun_dir, noise_map, threads=None):
        """The compat (billboard) image of camera over the volume's boards;
        params an or_compat_params (or a product cg_compat_params: same
        layout), noise_map from compat_noise_map."""
        threads = threads or os.cpu_count() or 1
        c = or_camera()
        c.eye[:] = [float(x) for x in camera.eye]
        c.target[:] = [float(x) for x in camera.target]
        c.up[:] = [float(x) for x in camera.up]
        c.fov_y_degrees = float(camera.fov_y_degrees)
        c.width, c.height = int(camera.width), int(camera.height)
        p = or_compat_params.from_buffer_copy(bytes(params))
        tab = np.ascontiguousarray(noise_map, np.float32)
        out = np.zeros((camera.height, camera.width, 4), np.float64)
        self.lib.or_compat_render(self.h, ctypes.byref(c), ctypes.byref(p), _f3(sun_dir),
                                  tab.ctypes.data_as(FP), out.ctypes.data_as(DP), threads)
        return out


def compat_noise_map(seed, bits=64):
    """The decoded 32^3 RGBA noise map (32, 32, 32, 4) float32, z-major."""
    out = np.zeros((32, 32, 32, 4), np.float32)
    load(bits).or_compat_noise_map(int(seed) & 0xFFFFFFFF, out.ctypes.data_as(FP))
    return out


def _dp(a):
    return a.ctypes.data_as(DP)


class OracleMLP:
    """FP64 forward / loss gradient / Adam of the surrogate (or_mlp_*) with 1,
    2 or 3 hidden layers."""

    NPARAM = 9473

    def __init__(self, params, mean, stddev, tau_scale, layers=3):
        self.lib = load(64)
        self.P = np.ascontiguousarray(params, np.float64)
        self.mu = np.ascontiguousarray(mean, np.float64)
        self.sd = np.ascontiguousarray(stddev, np.float64)
        self.tau_scale = float(tau_scale)
        self.layers = int(layers)

    def forward(self, feats):
        f = np.ascontiguousarray(feats, np.float64).reshape(-1, 16)
        return np.array([self.lib.or_mlp_forward(_dp(self.P), _dp(self.mu), _dp(self.sd),
                                                 _dp(np.ascontiguousarray(row)), self.layers)
                         for row in f])

    def loss_grad(self, feats, tau, sigma, params=None):
        P = self.P if params is None else np.ascontiguousarray(params, np.float64)
        f = np.ascontiguousarray(feats, np.float64).reshape(-1, 16)
        t = np.ascontiguousarray(tau, np.float64).reshape(-1)
        g = np.zeros(self.NPARAM, np.float64)
        loss = self.lib.or_mlp_loss_grad(_dp(P), _dp(self.mu), _dp(self.sd), self.tau_scale,
                                         float(sigma), _dp(f), _dp(t), f.shape[0], _dp(g),
                                         self.layers)
        return loss, g


def adam_step(w, m, v, g, lr, b1, b2, eps, t):
    w = np.ascontiguousarray(w, np.float64).copy()
    m = np.ascontiguousarray(m, np.float64).copy()
    v = np.ascontiguousarray(v, np.float64).copy()
    g = np.ascontiguousarray(g, np.float64)
    load(64).or_adam_step(_dp(w), _dp(m), _dp(v), _dp(g), w.shape[0], lr, b1, b2, eps, int(t))
    return w, m, v


def mlp_features(vol, positions, direction, base_level, initial_height):
    d = np.asarray(direction, np.float64)
    d = d / np.sqrt((d * d).sum())
    out = np.zeros((len(positions), 16))
    for i, p in enumerate(positions):
        o = np.zeros(16)
        vol.lib.or_mlp_features(vol.h, _d3(p), _d3(d), int(base_level), float(initial_height),
                                _dp(o))
        out[i] = o
    return out


def fbm(p, params, bits=64):
    return load(bits).or_fbm(_d3(p), ctypes.byref(params))


def lattice(ix, iy, iz, seed, octave, bits=64):
    return load(bits).or_lattice(int(ix), int(iy), int(iz), int(seed) & 0xFFFFFFFF, int(octave))


def pcg3d(v):
    a = (ctypes.c_uint32 * 3)(*[int(x) & 0xFFFFFFFF for x in v])
    load(64).or_pcg3d(a)
    return tuple(int(x) for x in a)


def sun_frame(position, bounds, direction, W, H, bits=64):
    fr = or_sun_frame()
    rc = load(bits).or_sun_frame_make(_f3(position), float(bounds[0]), float(bounds[1]),
                                      _f3(direction), int(W), int(H), ctypes.byref(fr))
    return rc, fr
