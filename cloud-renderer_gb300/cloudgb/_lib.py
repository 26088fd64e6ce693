"""ctypes binding of include/cloudgb.h (libcloudgb.so, built for sm_103a).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# the bounds-check build (CG_BOUNDS_CHECK=1 at build time) is loaded instead
# when CG_BOUNDS_CHECK=1 is set at run time
LIB_PATH = os.path.join(_HERE, "libcloudgb_check.so" if os.environ.get("CG_BOUNDS_CHECK") == "1"
                        else "libcloudgb.so")

CG_OK = 0
STATUS_NAMES = {
    0: "CG_OK", 1: "CG_ERR_INVALID_ARGUMENT", 2: "CG_ERR_OUT_OF_RANGE",
    3: "CG_ERR_OUT_OF_MEMORY", 4: "CG_ERR_CUDA", 5: "CG_ERR_NOT_READY",
    6: "CG_ERR_DEVICE_FAULT", 7: "CG_ERR_IO", 8: "CG_ERR_BAD_CHECKPOINT",
    9: "CG_ERR_UNSUPPORTED",
}
FORMAT_RGBA32F = 0
FORMAT_BF16_FP16 = 1
CONE_TRANSMITTANCE = 0
CONE_REFERENCE = 1
MEMCPY_H2D, MEMCPY_D2H, MEMCPY_D2D = 1, 2, 3


class CloudError(RuntimeError):
    """A libcloudgb call returned a non-OK cg_status."""

    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class cg_sun(ctypes.Structure):
    _fields_ = [("direction", ctypes.c_float * 3), ("map_width", ctypes.c_int),
                ("map_height", ctypes.c_int)]


class cg_camera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("target", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3), ("fov_y_degrees", ctypes.c_float),
                ("width", ctypes.c_int), ("height", ctypes.c_int)]


class cg_noise(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint32), ("octaves", ctypes.c_int),
                ("frequency", ctypes.c_float), ("lacunarity", ctypes.c_float),
                ("gain", ctypes.c_float), ("offset", ctypes.c_float * 3)]


class cg_render_params(ctypes.Structure):
    _fields_ = [("view_steps", ctypes.c_int), ("sun_steps", ctypes.c_int),
                ("cone_half_angle", ctypes.c_float), ("cone_initial_height", ctypes.c_float),
                ("cone_min_radius", ctypes.c_float), ("lod_offset", ctypes.c_float),
                ("down_scaling", ctypes.c_float), ("density_scale", ctypes.c_float),
                ("ambient", ctypes.c_float), ("sun_color", ctypes.c_float * 3),
                ("transmittance_cutoff", ctypes.c_float), ("cone_mode", ctypes.c_int),
                ("noise", cg_noise), ("use_mlp", ctypes.c_int), ("mlp", ctypes.c_void_p),
                ("pipeline", ctypes.c_int), ("cone_lanes", ctypes.c_int)]


PIPELINE_FUSED = 0
PIPELINE_DEFERRED = 1
PIPELINE_PERSISTENT = 2
MLP_FEATURES = 16
MLP_PARAMS = 9473
MLP_MAX_LAYERS = 3
MLP_DEFAULT_LAYERS = 3


class cg_mlp_config(ctypes.Structure):
    _fields_ = [("base_level", ctypes.c_int), ("initial_height", ctypes.c_float),
                ("dimension", ctypes.c_int), ("sun_steps", ctypes.c_int),
                ("cone_half_angle", ctypes.c_float), ("cone_initial_height", ctypes.c_float),
                ("cone_min_radius", ctypes.c_float), ("lod_offset", ctypes.c_float),
                ("mean", ctypes.c_float * 16), ("stddev", ctypes.c_float * 16),
                ("feature_min", ctypes.c_float * 16), ("feature_max", ctypes.c_float * 16),
                ("tau_scale", ctypes.c_float)]


class cg_train_params(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("batch", ctypes.c_int), ("lr", ctypes.c_float),
                ("beta1", ctypes.c_float), ("beta2", ctypes.c_float), ("eps", ctypes.c_float),
                ("sigma", ctypes.c_float), ("seed", ctypes.c_uint64),
                ("separate_adam", ctypes.c_int)]


class cg_trace_config(ctypes.Structure):
    _fields_ = [("lanes_per_ray", ctypes.c_int), ("step_unroll", ctypes.c_int),
                ("brick", ctypes.c_int)]


class cg_batch_view(ctypes.Structure):
    _fields_ = [("volume", ctypes.c_void_p), ("camera", cg_camera), ("rgba_out", ctypes.c_void_p)]


class cg_compat_params(ctypes.Structure):
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


class cg_volume_info(ctypes.Structure):
    _fields_ = [("dimension", ctypes.c_int), ("mips", ctypes.c_int), ("format", ctypes.c_int),
                ("board_count", ctypes.c_int), ("world_min", ctypes.c_float * 3),
                ("world_max", ctypes.c_float * 3), ("level_dim", ctypes.c_int * 16),
                ("level_offset", ctypes.c_size_t * 16), ("bytes_per_voxel", ctypes.c_size_t),
                ("pyramid_bytes", ctypes.c_size_t)]


P = ctypes.c_void_p
PP = ctypes.POINTER(ctypes.c_void_p)
I = ctypes.c_int
F = ctypes.c_float
FP = ctypes.POINTER(ctypes.c_float)
U32P = ctypes.POINTER(ctypes.c_uint32)
U64P = ctypes.POINTER(ctypes.c_uint64)
U8P = ctypes.POINTER(ctypes.c_uint8)
SZ = ctypes.c_size_t

# (name, restype, argtypes) for every function declared in include/cloudgb.h
SIGNATURES = [
    ("cg_status_string", ctypes.c_char_p, [I]),
    ("cg_last_error", ctypes.c_char_p, []),
    ("cg_abi_version", I, []),
    ("cg_context_create", I, [I, PP]),
    ("cg_context_destroy", None, [P]),
    ("cg_context_synchronize", I, [P]),
    ("cg_context_launch_count", ctypes.c_uint64, [P]),
    ("cg_render_params_default", None, [ctypes.POINTER(cg_render_params)]),
    ("cg_context_set_timing", I, [P, I]),
    ("cg_context_stage_times", I, [P, FP, I, ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, SZ]),
    ("cg_host_alloc", I, [SZ, PP]),
    ("cg_host_free", None, [P]),
    ("cg_device_alloc", I, [SZ, PP]),
    ("cg_device_free", None, [P]),
    ("cg_memcpy", I, [P, P, SZ, I]),
    ("cg_volume_create", I, [P, I, F, F, FP, I, I, PP]),
    ("cg_volume_destroy", None, [P]),
    ("cg_volume_set_billboards", I, [P, FP, FP, FP, I, F]),
    ("cg_voxelize", I, [P, ctypes.POINTER(cg_sun), P]),
    ("cg_render", I, [P, P, ctypes.POINTER(cg_camera), ctypes.POINTER(cg_render_params), P, I, P]),
    ("cg_render_stats", I, [P, P, ctypes.POINTER(cg_camera), ctypes.POINTER(cg_render_params),
                            U64P]),
    ("cg_trace_cones", I, [P, P, I, FP, ctypes.POINTER(cg_render_params), P, I, P]),
    ("cg_volume_get_info", I, [P, ctypes.POINTER(cg_volume_info)]),
    ("cg_volume_read_level", I, [P, I, P, SZ]),
    ("cg_volume_read_coverage", I, [P, U32P, U32P]),
    ("cg_volume_read_sun_map", I, [P, U64P, FP]),
    ("cg_volume_read_highlight", I, [P, U8P]),
    ("cg_volume_active_voxels", I, [P, U64P]),
    ("cg_sun_map_noalloc", I, [I, F, F, FP, P, I, ctypes.POINTER(cg_sun), P, P, P]),
    ("cg_march_samples", I, [P, P, ctypes.POINTER(cg_camera), ctypes.POINTER(cg_render_params),
                             FP, FP, I, ctypes.POINTER(ctypes.c_int)]),
    ("cg_mlp_config_default", None, [ctypes.POINTER(cg_mlp_config)]),
    ("cg_train_params_default", None, [ctypes.POINTER(cg_train_params)]),
    ("cg_mlp_param_count", I, []),
    ("cg_mlp_create", I, [P, ctypes.c_uint64, PP]),
    ("cg_mlp_create_layers", I, [P, ctypes.c_uint64, I, PP]),
    ("cg_mlp_hidden_layers", I, [P]),
    ("cg_mlp_destroy", None, [P]),
    ("cg_mlp_configure", I, [P, ctypes.POINTER(cg_mlp_config)]),
    ("cg_mlp_get_config", I, [P, ctypes.POINTER(cg_mlp_config)]),
    ("cg_mlp_features", I, [P, P, P, I, FP, P, I, P]),
    ("cg_mlp_infer", I, [P, P, I, P, I, P]),
    ("cg_mlp_gradient", I, [P, P, P, I, F, FP, FP, I]),
    ("cg_mlp_train", I, [P, P, P, ctypes.c_longlong, ctypes.POINTER(cg_train_params), FP]),
    ("cg_mlp_check_train_timeout", I, [P, P, P, ctypes.c_longlong, I, ctypes.c_uint32]),
    ("cg_mlp_get_params", I, [P, FP, FP, FP, ctypes.POINTER(ctypes.c_int)]),
    ("cg_mlp_set_params", I, [P, FP, FP, FP, I]),
    ("cg_mlp_save", I, [P, ctypes.c_char_p]),
    ("cg_mlp_load", I, [P, ctypes.c_char_p, PP]),
    ("cg_context_mlp_fallbacks", I, [P, U64P]),
    ("cg_context_last_samples", I, [P, U64P]),
    ("cg_image_error_stats", I, [P, P, P, I, ctypes.c_uint64, I, ctypes.POINTER(ctypes.c_double), P]),
    ("cg_volume_set_occupancy_brick", I, [P, I]),
    ("cg_render_batch", I, [P, ctypes.POINTER(cg_batch_view), I, ctypes.POINTER(cg_render_params),
                            ctypes.POINTER(cg_trace_config), P]),
    ("cg_context_set_trace_config", I, [P, ctypes.POINTER(cg_trace_config)]),
    ("cg_context_get_trace_config", I, [P, ctypes.POINTER(cg_trace_config)]),
    ("cg_autotune", I, [P, ctypes.POINTER(cg_batch_view), I, ctypes.POINTER(cg_render_params), I,
                        ctypes.POINTER(cg_trace_config), FP]),
    ("cg_frame_graph_create", I, [P, PP, I, ctypes.POINTER(cg_sun), ctypes.POINTER(cg_batch_view),
                                  I, ctypes.POINTER(cg_render_params), PP]),
    ("cg_frame_graph_launch", I, [P, P]),
    ("cg_frame_graph_destroy", None, [P]),
    ("cg_compat_params_default", None, [ctypes.POINTER(cg_compat_params)]),
    ("cg_context_check_wait_timeout", I, [P, ctypes.c_uint32, U64P]),
    ("cg_bounds_check_build", I, []),
    ("cg_context_bounds_violations", I, [P, U64P, ctypes.c_char_p, I]),
    ("cg_compat_noise_map", I, [ctypes.c_uint32, FP]),
    ("cg_render_compat", I, [P, P, ctypes.POINTER(cg_camera), ctypes.POINTER(cg_compat_params), P,
                             I, P]),
]
NOALLOC_MAX_TEXELS = 1 << 20

_lib = None


def load():
    """Load libcloudgb.so and bind every declared entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`")
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, what=""):
    if status != CG_OK:
        msg = load().cg_last_error().decode(errors="replace")
        raise CloudError(status, f"{what}: {msg}" if what else msg)
