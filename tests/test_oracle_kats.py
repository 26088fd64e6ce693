"""Known-answer tests that pin the CPU oracle where the reference has no code
or fixtures: coverage of a single ball, permutation invariance, mips, the
sampler, the sun cone, front-to-back compositing and the noise hash."""
import math

import numpy as np
import pytest

from oracle import oracle as O

BOUNDS = (-0.5, 0.5)
POS = (0.5, 0.5, 0.5)


def vol_with(boards, D=64, L=7, dens=None, sun=(0.3, 1.0, 0.2), map_size=(256, 256), bits=64):
    v = O.OracleVolume(D, BOUNDS, POS, L, bits=bits)
    pos = np.asarray([b[0] for b in boards], np.float32).reshape(-1, 3)
    rad = np.asarray([b[1] for b in boards], np.float32)
    assert v.set_boards(pos, rad, dens) == 0
    assert v.voxelize(sun, *map_size) == 0
    return v


@pytest.mark.parametrize("r", [0.1, 0.2, 0.33])
def test_single_ball_coverage_volume(r):
    D = 64
    v = vol_with([((0.013, -0.021, 0.007), r)], D=D)
    cnt, dq = v.coverage()
    n = int((cnt > 0).sum())
    rv = r * D
    exact = 4.0 / 3.0 * math.pi * rv ** 3
    # lattice-point count of a ball: error bounded by a few surface layers
    assert abs(n - exact) <= 3.0 * 4.0 * math.pi * rv ** 2 * 0.25 + 10
    assert cnt.max() == 1
    assert np.array_equal(dq[cnt > 0], np.full(n, 65536, np.uint32))


def test_coverage_voxel_centre_rule():
    # ball centred on a voxel corner with radius exactly one voxel: the 8
    # surrounding voxel centres lie at sqrt(3)/2 voxel -> inside
    D = 16
    v = vol_with([((0.0, 0.0, 0.0), 1.0 / D)], D=D, L=5)
    cnt, _ = v.coverage()
    assert int(cnt.sum()) == 8
    assert cnt[7:9, 7:9, 7:9].sum() == 8


def test_coverage_permutation_invariant():
    rng = np.random.default_rng(3)
    boards = [((rng.uniform(-0.3, 0.3, 3)), rng.uniform(0.05, 0.15)) for _ in range(40)]
    dens = rng.uniform(0.5, 1.0, 40).astype(np.float32)
    v1 = vol_with(boards, dens=dens)
    perm = rng.permutation(40)
    v2 = vol_with([boards[i] for i in perm], dens=dens[perm])
    c1, d1 = v1.coverage()
    c2, d2 = v2.coverage()
    assert np.array_equal(c1, c2) and np.array_equal(d1, d2)


def test_density_sum_is_q16():
    v = vol_with([((0, 0, 0), 0.2), ((0.05, 0, 0), 0.2)], dens=np.array([0.5, 0.25], np.float32))
    cnt, dq = v.coverage()
    both = cnt == 2
    assert both.any()
    assert np.all(dq[both] == 32768 + 16384)


def test_mip_of_constant_is_constant():
    v = vol_with([], D=32, L=6)
    lv = v.pyramid()
    lv[0][...] = 0.375
    v.set_pyramid(lv)
    v.rebuild_mips()
    for l in v.pyramid():
        assert np.allclose(l, 0.375, atol=0, rtol=0)


def test_mip_of_single_voxel():
    v = vol_with([], D=32, L=6)
    lv = v.pyramid()
    for l in lv:
        l[...] = 0
    lv[0][5, 9, 17, 0] = 1.0
    v.set_pyramid(lv)
    v.rebuild_mips()
    out = v.pyramid()
    for l in range(1, 6):
        assert out[l][..., 0].max() == pytest.approx(1.0 / 8 ** l)
        assert out[l][..., 0].sum() == pytest.approx(1.0 / 8 ** l)


def test_npot_mip_drops_last_child():
    v = O.OracleVolume(6, BOUNDS, POS, 3)
    v.set_boards(np.zeros((0, 3), np.float32), np.zeros(0, np.float32))
    v.voxelize((0.3, 1, 0.2), 16, 16)
    lv = v.pyramid()
    assert [l.shape[0] for l in lv] == [6, 3, 1]
    lv[1][...] = 0
    lv[1][2, 2, 2, 0] = 1.0  # the dropped child of 3 -> 1
    lv[0][...] = 0
    v.set_pyramid(lv)
    lv2 = v.pyramid()
    # rebuild from level 0 zeroes level 1; check directly that 3 -> 1 averages children 0,1
    lv2[0][...] = 0
    v.set_pyramid(lv2)
    v.rebuild_mips()
    assert v.pyramid()[2].max() == 0.0


def test_trilinear_at_texel_centres():
    v = vol_with([], D=16, L=5)
    lv = v.pyramid()
    rng = np.random.default_rng(1)
    for l in lv:
        l[...] = rng.uniform(0, 1, l.shape)
    v.set_pyramid(lv)
    for (x, y, z) in [(0, 0, 0), (3, 7, 11), (15, 15, 15)]:
        p = (x + 0.5, y + 0.5, z + 0.5)
        assert v.sample(p, 0.0, 0) == pytest.approx(lv[0][z, y, x, 0], abs=1e-12)
        assert v.sample(p, 0.0, 1) == pytest.approx(lv[0][z, y, x, 1], abs=1e-12)
    # level 2 texel centre (i + 0.5) * 4 in level-0 voxels
    assert v.sample((6.0, 2.0, 10.0), 2.0, 0) == pytest.approx(lv[2][2, 0, 1, 0], abs=1e-12)
    # halfway in lod blends the two levels linearly
    p = (2.0, 2.0, 2.0)
    a, b = v.sample(p, 1.0, 0), v.sample(p, 2.0, 0)
    assert v.sample(p, 1.5, 0) == pytest.approx(0.5 * (a + b), abs=1e-12)


def test_border_reads_zero_outside():
    v = vol_with([], D=16, L=5)
    lv = v.pyramid()
    for l in lv:
        l[...] = 1.0
    v.set_pyramid(lv)
    assert v.sample((8, 8, 8), 0, 0, border=1) == pytest.approx(1.0)
    assert v.sample((-1.0, 8, 8), 0, 0, border=1) == 0.0
    assert v.sample((0.0, 8, 8), 0, 0, border=1) == pytest.approx(0.5)
    assert v.sample((-1.0, 8, 8), 0, 0, border=0) == pytest.approx(1.0)


def test_sun_cone_empty_volume_is_zero():
    v = vol_with([], D=32, L=6)
    P = O.make_params(sun_steps=24)
    assert v.trace_cone((16, 16, 16), (0.3, 1, 0.2), P) == 0.0


def test_sun_cone_uniform_medium():
    """Constant density rho: tau = rho * sum(dh) * voxel_world while inside."""
    D, L = 64, 7
    v = vol_with([], D=D, L=L)
    lv = v.pyramid()
    rho = 0.7
    for l in lv:
        l[...] = 0
        l[..., 0] = rho
    v.set_pyramid(lv)
    P = O.make_params(sun_steps=8, cone_half_angle=0.05, cone_initial_height=1.0,
                      cone_min_radius=1.0)
    # march along +x from x = 4: total reach stays well inside the box at lod <= 1
    tau = v.trace_cone((4.0, 32.0, 32.0), (1, 0, 0), P)
    h, s = 1.0, 0.0
    for _ in range(8):
        r = max(h * math.tan(0.05), 1.0)
        s += r
        h += r
    assert h < 32
    assert tau == pytest.approx(rho * s / D, rel=1e-12)


def test_reference_cone_mode_weights():
    """CG_CONE_REFERENCE sums the light channel with weights i/(steps*down)."""
    v = vol_with([], D=32, L=6)
    lv = v.pyramid()
    for l in lv:
        l[...] = 0
        l[..., 1] = 1.0
    v.set_pyramid(lv)
    P = O.make_params(sun_steps=16, cone_mode=1, cone_half_angle=0.45, cone_initial_height=0.1,
                      down_scaling=2.0)
    got = v.trace_cone((16, 16, 16), (0.3, 1, 0.2), P)
    assert got == pytest.approx(sum(i / (16 * 2.0) for i in range(1, 17)), rel=1e-12)


def test_front_to_back_uniform_slab():
    """Uniform medium along a ray: alpha = 1 - exp(-sigma rho L)."""
    D, L = 64, 7
    v = vol_with([], D=D, L=L)
    lv = v.pyramid()
    rho = 0.5
    for l in lv:
        l[...] = 0
        l[..., 0] = rho
    v.set_pyramid(lv)

    class Cam:
        eye = (0.5, 0.5, -1.0)
        target = (0.5, 0.5, 0.5)
        up = (0.0, 1.0, 0.0)
        fov_y_degrees = 1e-3
        width = height = 2

    sigma = 1.5
    P = O.make_params(view_steps=8, sun_steps=0, density_scale=sigma, ambient=1.0,
                      transmittance_cutoff=0.0)
    img = v.render(Cam(), P, (0.3, 1, 0.2))
    # the chord through the unit cube is 1; every sample is 4 voxels or more inside
    expect = 1.0 - math.exp(-sigma * rho * 1.0)
    assert img[..., 3] == pytest.approx(np.full((2, 2), expect), abs=1e-9)
    # with no sun steps T_sun = 1, so colour = alpha (ambient 1)
    assert img[..., 0] == pytest.approx(np.full((2, 2), expect), abs=1e-9)


def _pcg3d_py(v):
    M = 0xFFFFFFFF
    x, y, z = [(a * 1664525 + 1013904223) & M for a in v]
    x = (x + y * z) & M
    y = (y + z * x) & M
    z = (z + x * y) & M
    x ^= x >> 16
    y ^= y >> 16
    z ^= z >> 16
    x = (x + y * z) & M
    y = (y + z * x) & M
    z = (z + x * y) & M
    return x, y, z


def test_pcg3d_matches_published_algorithm():
    for v in [(0, 0, 0), (1, 2, 3), (0xFFFFFFFF, 12345, 987654321)]:
        assert O.pcg3d(v) == _pcg3d_py(v)


def test_noise_is_deterministic_and_seeded():
    a = [O.lattice(i, 2 * i, 3 * i, 7, 0) for i in range(50)]
    b = [O.lattice(i, 2 * i, 3 * i, 7, 0) for i in range(50)]
    c = [O.lattice(i, 2 * i, 3 * i, 8, 0) for i in range(50)]
    d = [O.lattice(i, 2 * i, 3 * i, 7, 1) for i in range(50)]
    assert a == b and a != c and a != d
    assert all(0.0 <= x < 1.0 for x in a)
    assert 0.35 < np.mean(a + c + d) < 0.65


def test_fbm_range_and_continuity():
    P = O.make_params(noise_octaves=4, noise_seed=7)
    rng = np.random.default_rng(0)
    vals = [O.fbm(rng.uniform(0, 1, 3), P) for _ in range(200)]
    assert 0.0 <= min(vals) and max(vals) < 1.0
    # continuous across a lattice boundary (x*4 = 1)
    lo = O.fbm((0.25 - 1e-9, 0.3, 0.7), P)
    hi = O.fbm((0.25 + 1e-9, 0.3, 0.7), P)
    assert abs(lo - hi) < 1e-6
    assert O.fbm((0.3, 0.3, 0.3), O.make_params(noise_octaves=0)) == 1.0


def test_fbm_wind_offset_is_a_domain_shift():
    """octaveOffsets (base-frequency lattice units) move the whole fBm: with
    offset o and frequency f, fbm_o(p) = fbm_0(p + o / f), every octave alike."""
    f = np.float32(4.0)
    off = np.float32([0.37, -1.25, 2.5])
    P0 = O.make_params(noise_octaves=4, noise_seed=7, noise_frequency=float(f))
    P1 = O.make_params(noise_octaves=4, noise_seed=7, noise_frequency=float(f),
                       noise_offset=off)
    rng = np.random.default_rng(3)
    for p in rng.uniform(-1, 1, (50, 3)):
        q = p + off.astype(np.float64) / np.float64(f)
        assert O.fbm(p, P1) == O.fbm(q, P0)
    # a whole lattice cell of offset at the base frequency is a shift by one
    # base cell (1 / f world units), not the identity
    P2 = O.make_params(noise_octaves=4, noise_seed=7, noise_frequency=float(f),
                       noise_offset=(1.0, 0.0, 0.0))
    p = np.array([0.1, 0.2, 0.3])
    assert O.fbm(p, P2) == O.fbm(p + np.array([0.25, 0.0, 0.0]), P0)
    assert O.fbm(p, P2) != O.fbm(p, P0)


def test_sun_frame_orthonormal():
    rc, fr = O.sun_frame(POS, BOUNDS, (0.3, 1.0, 0.2), 1280, 720)
    assert rc == 0
    r, u, f = (np.array(fr.right[:]), np.array(fr.up[:]), np.array(fr.fwd[:]))
    for a in (r, u, f):
        assert abs(np.linalg.norm(a) - 1) < 1e-6
    assert abs(r @ u) < 1e-6 and abs(r @ f) < 1e-6 and abs(u @ f) < 1e-6
    s = np.array([0.3, 1.0, 0.2]) / np.linalg.norm([0.3, 1.0, 0.2])
    assert np.allclose(f, -s, atol=1e-6)
    assert fr.lo == -1.0 and fr.hi == 1.0
    # the sun straight overhead is degenerate for lookAt with up = +y
    assert O.sun_frame(POS, BOUNDS, (0, 1, 0), 64, 64)[0] == -1


def test_fp32_build_tracks_fp64_oracle():
    """The FP32 CPU baseline agrees with the FP64 oracle on the small scene."""
    import cloudgb.configs as C
    from cloudgb import workload
    cfg = C.SMALL_64
    wl = workload.build(cfg, width=64, height=64)
    imgs = []
    for bits in (64, 32):
        v = O.OracleVolume(cfg["dim"], C.VOLUME_BOUNDS, C.VOLUME_POSITION, cfg["mips"], bits=bits)
        v.set_boards(wl.positions, wl.scales, wl.densities)
        v.voxelize(wl.sun_direction, *wl.sun_map)
        cam = _cam(wl.cameras[0])
        P = O.make_params(view_steps=cfg["view_steps"], sun_steps=cfg["sun_steps"],
                          cone_half_angle=cfg["cone_half_angle"],
                          density_scale=cfg["density_scale"])
        imgs.append(v.render(cam, P, wl.sun_direction))
    assert np.abs(imgs[0] - imgs[1]).max() < 1e-4


class _cam:
    def __init__(self, c):
        self.eye, self.target, self.up = c["eye"], c["target"], (0.0, 1.0, 0.0)
        self.fov_y_degrees, self.width, self.height = c["fov"], c["width"], c["height"]


def test_index_paths_identical_in_both_builds():
    """Coverage, sun-map keys and highlights do not depend on the float type."""
    rng = np.random.default_rng(11)
    boards = [((rng.uniform(-0.3, 0.3, 3)), rng.uniform(0.03, 0.1)) for _ in range(60)]
    a = vol_with(boards, bits=64)
    b = vol_with(boards, bits=32)
    assert np.array_equal(a.coverage()[0], b.coverage()[0])
    assert np.array_equal(a.sun_map()[0], b.sun_map()[0])
    assert np.array_equal(a.mask(), b.mask())
