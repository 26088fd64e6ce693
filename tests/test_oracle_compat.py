"""The compat render's oracle (or_compat_render: the reference's billboard
image formation restated in C) against the reference's own shaders.

tests/golden/reference_compat.npz holds images the reference's
billboard_vert_instanced.glsl + conetrace_frag.glsl produced, compiled as C++
through oracle/ref_shim/ and driven as ConeTraceShader::coneTrace drives them
(tests/golden/make_compat_golden.py).  The oracle, fed the same seeded scene,
must reproduce them to within FP32-vs-FP64 rounding (1e-4 on 99.9 % of the
pixel values; the FP32 shader and the FP64 oracle may disagree on a rare
fragment whose discard test or noise step count sits on a threshold).
"""
import ctypes
import os
import sys

import numpy as np
import pytest

from cloudgb import _lib, configs, workload
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_compat_golden as G  # noqa: E402

GOLD = os.path.join(HERE, "golden", "reference_compat.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


class Cam:
    def __init__(self, eye, target, fov, w, h):
        self.eye, self.target, self.up = tuple(eye), tuple(target), (0.0, 1.0, 0.0)
        self.fov_y_degrees, self.width, self.height = fov, w, h


def camera_of(gold, name):
    c = gold[f"{name}_camera"]
    W, H = (int(x) for x in gold["size"])
    return Cam(c[:3], c[3:6], float(c[6]), W, H)


def close_enough(a, b, tol=1e-4, frac=1e-3):
    err = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    return float(np.quantile(err, 1.0 - frac)) <= tol, float(err.max()), float(np.quantile(err, 0.999))


@pytest.mark.parametrize("name", list(G.CASES))
def test_oracle_matches_reference_compat_pass(gold, name):
    cam_spec, n, kw = G.CASES[name]
    wl, c, ov = G.case_inputs(cam_spec, n)
    P = O.or_compat_params.from_buffer_copy(gold[f"{name}_params"].tobytes())
    img = ov.compat_render(camera_of(gold, name), P, wl.sun_direction,
                           O.compat_noise_map(P.noise_seed))
    ok, mx, q = close_enough(img, gold[f"{name}_image"])
    assert ok, f"{name}: 99.9% quantile {q}, max {mx}"
    assert int(gold[f"{name}_shaded"][0]) > 1000  # the case draws fragments


def test_golden_inputs_are_reproducible(gold):
    """The fixture's parameter blocks are what the generator's cases say."""
    for name, (_, n, kw) in G.CASES.items():
        assert bytes(G.compat_params(**kw)) == gold[f"{name}_params"].tobytes()
        assert int(gold[f"{name}_boards"][0]) == n


@pytest.mark.parametrize("seed", [0, 1, 9, 0xDEADBEEF])
def test_product_noise_map_equals_oracle(seed):
    """The library's host-side noise map (integer-exact) is the oracle's."""
    lib = _lib.load()
    out = np.empty((32, 32, 32, 4), np.float32)
    assert lib.cg_compat_noise_map(seed, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    ref = O.compat_noise_map(seed)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    # GL_RGBA8_SNORM decode: multiples of 1/127 in [-1, 1]; RGB of unit length
    assert np.all(np.abs(out) <= 1.0)
    q = out * 127.0
    assert np.allclose(q, np.round(q), atol=1e-4)
    nrm = np.linalg.norm(out[..., :3], axis=-1)
    assert np.all((nrm == 0) | (np.abs(nrm - 128.0 / 127.0) < 0.03))


def test_compat_defaults_are_the_reference_fields():
    p = _lib.cg_compat_params()
    _lib.load().cg_compat_params_default(ctypes.byref(p))
    assert (p.show_quad, p.do_noise, p.do_cone_trace) == (0, 1, 1)
    assert abs(p.step_size - 0.01) < 1e-9 and p.noise_opacity == 4.0 and p.num_octaves == 4
    assert p.freq_step == 3.0 and p.pers_step == 0.5 and p.adjust_size == 40.0
    assert (p.min_noise_steps, p.max_noise_steps) == (2, 8)
    assert abs(p.min_noise_color - 0.2) < 1e-7 and abs(p.noise_color_scale - 0.45) < 1e-7
    assert p.vct_steps == 16 and abs(p.vct_cone_angle - 0.9) < 1e-7
    assert abs(p.vct_cone_initial_height - 0.1) < 1e-7
    assert tuple(round(x, 6) for x in p.clear_color) == (0.2, 0.3, 0.5, 1.0)
    assert ctypes.sizeof(p) == ctypes.sizeof(O.or_compat_params)


def test_oracle_edge_cases():
    cfg = configs.COMPAT_REF
    wl = workload.build_compat(cfg, boards=20, width=24, height=16)
    cam = wl.cameras[0]
    c = Cam(cam["eye"], cam["target"], cam["fov"], 24, 16)
    tab = O.compat_noise_map(1)
    clear = np.array([0.2, 0.3, 0.5, 1.0])
    # no boards: the clear colour
    ov = O.OracleVolume(cfg["dim"], cfg["bounds"], cfg["position"], cfg["mips"])
    ov.set_boards(np.zeros((0, 3), np.float32), np.zeros(0, np.float32), np.zeros(0, np.float32))
    ov.voxelize(wl.sun_direction, 64, 64)
    img = ov.compat_render(c, G.compat_params(), wl.sun_direction, tab)
    assert np.allclose(img, clear, atol=1e-7)
    # every stage off: the pass returns before drawing
    _, _, ov = G.case_inputs(0, 20)
    img = ov.compat_render(c, G.compat_params(do_noise=0, do_cone_trace=0), wl.sun_direction, tab)
    assert np.allclose(img, clear, atol=1e-7)
    # boards behind the camera are clipped: looking away from the cloud
    away = Cam(cam["eye"], tuple(2 * np.array(cam["eye"]) - np.array(cam["target"])), 60.0, 24, 16)
    img = ov.compat_render(away, G.compat_params(), wl.sun_direction, tab)
    assert np.allclose(img, clear, atol=1e-7)
    # and drawn when facing it
    img = ov.compat_render(c, G.compat_params(), wl.sun_direction, tab)
    assert np.abs(img - clear).max() > 0.05


@pytest.mark.skipif(not __import__("oracle.ref_shaders", fromlist=["x"]).available(),
                    reason="reference shaders not built here")
@pytest.mark.parametrize("seed", [3, 4])
def test_live_reference_compat_random_scenes(seed):
    """Random parameter draws on the reference-scale scene, oracle vs the
    reference's shaders run live (only where the reference is present)."""
    from oracle import ref_shaders as R
    rng = np.random.default_rng(seed)
    kw = dict(noise_opacity=float(rng.uniform(1, 6)), num_octaves=int(rng.integers(1, 4)),
              freq_step=float(rng.uniform(1.5, 3.5)), pers_step=float(rng.uniform(0.3, 0.7)),
              adjust_size=float(rng.uniform(20, 60)), min_noise_steps=int(rng.integers(2, 4)),
              max_noise_steps=int(rng.integers(5, 10)), vct_steps=int(rng.integers(4, 30)),
              vct_cone_angle=float(rng.uniform(0.2, 1.2)), noise_seed=int(rng.integers(0, 99)),
              octave_offsets=tuple(float(x) for x in rng.uniform(-1, 1, 3)))
    cfg = configs.COMPAT_REF
    wl, c, ov = G.case_inputs(int(rng.integers(0, 8)), 150)
    P = G.compat_params(**kw)
    light = [lv[..., 1].astype(np.float32) for lv in ov.pyramid()]
    tab = O.compat_noise_map(P.noise_seed)
    ref, _ = R.compat_render(wl.positions, wl.scales, cfg["position"], cfg["bounds"], cfg["dim"],
                             light, tab, c["eye"], c["target"], (0.0, 1.0, 0.0), c["fov"],
                             G.W, G.H, wl.sun_direction, P)
    img = ov.compat_render(Cam(c["eye"], c["target"], c["fov"], G.W, G.H), P, wl.sun_direction,
                           tab)
    ok, mx, q = close_enough(img, ref)
    assert ok, (q, mx)
