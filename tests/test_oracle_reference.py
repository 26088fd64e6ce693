"""The oracle against the reference's own shader code.

tests/golden/reference_shaders.npz holds what the reference's shaders
(res/billboard_vert_instanced.glsl, first_voxelize.glsl, second_voxelize.glsl
and traceCone of conetrace_frag.glsl, compiled as C++ through
oracle/ref_shim/) computed on seeded scenes; tests/golden/make_golden.py made
it.  Bars:
  * sun-view map: the same covered texels and the same winning board per
    texel, surface positions within 1e-5 (the oracle works in sun-view space,
    the shaders in world space through matrices: rounding differs);
  * highlight marks over the same position map: bit-exact;
  * traceCone: within 2e-5 relative (FP64 oracle vs the FP32 shader).
Where the library itself was built (oracle/_ref/), more seeded cases run live.
"""
import os

import numpy as np
import pytest

from cloudgb import configs, scene
from oracle import oracle as O
from oracle import ref_shaders as R

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                    "reference_shaders.npz")
BOUNDS = configs.VOLUME_BOUNDS
VPOS = configs.VOLUME_POSITION
SCENES = ["small", "oblique", "edge"]
CONE_PARAMS = [(16, 0.1, 1.0, 0.0, 1.0), (24, 0.6, 2.0, 0.5, 2.0)]


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def levels_of(D):
    return int(np.floor(np.log2(D))) + 1


def scene_of(gold, name):
    n, D, W, H = (int(x) for x in gold[f"sun_{name}_meta"])
    s = gold[f"sun_{name}_scene"]
    pos, rad, dens = s[:3 * n].reshape(n, 3), s[3 * n:4 * n], s[4 * n:5 * n]
    return n, D, W, H, pos, rad, dens, tuple(float(x) for x in gold[f"sun_{name}_dir"])


def oracle_volume(D, pos, rad, dens, sun, W, H):
    ov = O.OracleVolume(D, BOUNDS, VPOS, levels_of(D))
    ov.set_boards(pos, rad, dens)
    ov.voxelize(sun, W, H)
    return ov


def cone_params(steps, ang, h0, lodo, ds):
    return O.make_params(sun_steps=steps, cone_half_angle=ang / 2.0, cone_initial_height=h0,
                         lod_offset=lodo, down_scaling=ds, cone_mode=1)


def check_sun_map(ov, texels, winner, posw, W, H):
    keys, pm = ov.sun_map()
    k = keys.reshape(-1)
    covered = np.flatnonzero(k != np.uint64(0xFFFFFFFFFFFFFFFF))
    np.testing.assert_array_equal(covered, texels)
    np.testing.assert_array_equal((k[covered] & np.uint64(0xFFFFFFFF)).astype(np.int64),
                                  winner.astype(np.int64))
    d = np.abs(pm.reshape(-1, 4)[covered, :3].astype(np.float64) - posw.astype(np.float64))
    assert d.max() <= 1e-5, d.max()


def marks_volume(idx, D):
    m = np.zeros(D * D * D, np.uint8)
    m[idx] = 1
    return m.reshape(D, D, D)


@pytest.mark.parametrize("name", SCENES)
def test_sun_map_matches_reference_shaders(gold, name):
    n, D, W, H, pos, rad, dens, sun = scene_of(gold, name)
    ov = oracle_volume(D, pos, rad, dens, sun, W, H)
    check_sun_map(ov, gold[f"sun_{name}_texels"], gold[f"sun_{name}_winner"],
                  gold[f"sun_{name}_pos"], W, H)


@pytest.mark.parametrize("name", SCENES)
def test_highlight_marks_match_reference_shaders(gold, name):
    n, D, W, H, pos, rad, dens, sun = scene_of(gold, name)
    ov = oracle_volume(D, pos, rad, dens, sun, W, H)
    pm = np.zeros((W * H, 4), np.float32)
    tex = gold[f"sun_{name}_texels"]
    pm[tex, :3] = gold[f"sun_{name}_pos"]
    pm[tex, 3] = 1.0
    want = marks_volume(gold[f"marks_{name}"], D)
    np.testing.assert_array_equal(ov.highlight_posmap(pm.reshape(H, W, 4)), want)
    # and from the oracle's own map: a store index can only move when a
    # position lies within its 1e-5 of a voxel face
    own = ov.mask()
    assert (own != want).sum() <= 0.001 * want.sum(), (own != want).sum()


def test_highlight_marks_random_map(gold):
    D, W, H = (int(x) for x in gold["marks_rand_meta"])
    ov = O.OracleVolume(D, BOUNDS, VPOS, 1)
    got = ov.highlight_posmap(gold["marks_rand_posmap"])
    np.testing.assert_array_equal(got, marks_volume(gold["marks_rand"], D))


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("k", [0, 1])
def test_trace_cone_reference_mode_scene(gold, name, k):
    n, D, W, H, pos, rad, dens, sun = scene_of(gold, name)
    ov = oracle_volume(D, pos, rad, dens, sun, W, H)
    P = cone_params(*CONE_PARAMS[k])
    vp = gold[f"cone_{name}_{k}_voxpos"].astype(np.float64)
    want = gold[f"cone_{name}_{k}_value"].astype(np.float64)
    got = ov.trace_cones(vp, sun, P)
    assert np.abs(want).max() > 0
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=2e-5)


@pytest.mark.parametrize("k", [0, 1])
def test_trace_cone_reference_mode_random_volume(gold, k):
    lv0 = gold["cone_rand_level0"].astype(np.float64)
    D = lv0.shape[0]
    ov = O.OracleVolume(D, BOUNDS, VPOS, 5)
    levels = [np.zeros((D >> l,) * 3 + (4,)) for l in range(5)]
    levels[0][..., 1] = lv0
    ov.set_pyramid(levels)
    ov.rebuild_mips()
    P = cone_params(*CONE_PARAMS[k])
    vp = gold[f"cone_rand_{k}_voxpos"].astype(np.float64)
    dirs = gold["cone_rand_dirs"].astype(np.float64)
    got = np.array([ov.trace_cone(p, d, P) for p, d in zip(vp, dirs)])
    want = gold[f"cone_rand_{k}_value"].astype(np.float64)
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=2e-5)


live = pytest.mark.skipif(not R.available(), reason="oracle/_ref/libref_shaders.so not built")


@live
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_live_reference_shaders(seed):
    """Fresh seeded scenes through the reference's shaders and the oracle."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(16, 160))
    D = int(rng.choice([24, 32, 40, 64]))
    W, H = int(rng.integers(48, 140)), int(rng.integers(40, 120))
    sun = rng.normal(size=3)
    sun[1] = abs(sun[1]) + 0.2
    sun = tuple(sun / np.linalg.norm(sun))
    pos, rad, dens = scene.billboards(seed, n, radius_scale=float(rng.uniform(0.4, 1.0)),
                                      volume_position=VPOS)
    pm, win, dep, _ = R.sun_pass(pos, rad, VPOS, BOUNDS, sun, W, H)
    ov = oracle_volume(D, pos, rad, dens, sun, W, H)
    tex = np.flatnonzero(win.reshape(-1) >= 0)
    check_sun_map(ov, tex, win.reshape(-1)[tex], pm.reshape(-1, 4)[tex, :3], W, H)
    np.testing.assert_array_equal(ov.highlight_posmap(pm), R.second_pass(pm, D, VPOS, BOUNDS))
    G = [l[..., 1] for l in ov.pyramid()]
    P = cone_params(*CONE_PARAMS[seed % 2])
    for p in rng.uniform(0.2, 0.8, (24, 3)):
        v, vp = R.trace_cone(G, D, VPOS, BOUNDS, p, sun, *CONE_PARAMS[seed % 2])
        assert abs(ov.trace_cone(vp.astype(np.float64), sun, P) - v) <= 2e-5 * max(1.0, abs(v))
