"""GPU parity through the C ABI against the CPU oracle.

Bit-exact: quantized boards, coverage counts, Q16.16 density sums, sun-view
depth keys (winner boards), position map, highlight mask, level-0 texels.
Tolerance: mips (FP32 vs FP64, 1e-6 relative), traceCone (1e-5 relative),
and the FP32 image vs the FP64 oracle: max-abs <= 1e-4 per RGBA channel.
"""
import numpy as np
import pytest

import cloudgb
from cloudgb import configs, workload
from oracle import oracle as O

pytestmark = pytest.mark.gpu

IMAGE_TOL = 1e-4


def make_pair(ctx, dim, mips, positions, scales, densities, sun_dir, sun_map, fmt=0,
              fluffiness=1.0):
    vol = cloudgb.CloudVolume(dim, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, mips, fmt=fmt,
                              ctx=ctx)
    vol.set_billboards(positions, scales, densities)
    vol.fluffiness = fluffiness
    vol.update()
    sun = cloudgb.Sun(sun_dir, *sun_map)
    cloudgb.VoxelizeShader().voxelize(vol, sun)
    ov = O.OracleVolume(dim, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, mips)
    assert ov.set_boards(positions, scales, densities, fluffiness) == 0
    assert ov.voxelize(sun.direction, *sun_map) == 0
    return vol, sun, ov


def random_scene(seed, n, spread=0.3, rmin=0.02, rmax=0.12):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
    rad = rng.uniform(rmin, rmax, n).astype(np.float32)
    den = rng.uniform(0.5, 1.0, n).astype(np.float32)
    return pos, rad, den


def assert_voxelize_exact(vol, sun, ov):
    cnt, dq = vol.read_coverage()
    ocnt, odq = ov.coverage()
    assert np.array_equal(cnt, ocnt), f"count mismatch at {np.argwhere(cnt != ocnt)[:5]}"
    assert np.array_equal(dq, odq), "density mismatch"
    keys, pos = vol.read_sun_map(sun)
    okeys, opos = ov.sun_map()
    assert np.array_equal(keys, okeys), f"{int((keys != okeys).sum())} sun-map keys differ"
    assert np.array_equal(pos, opos), "position map differs"
    assert np.array_equal(vol.read_highlight(), ov.mask()), "highlight mask differs"


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_voxelize_random_scenes_bit_exact(ctx, seed):
    pos, rad, den = random_scene(seed, 48)
    vol, sun, ov = make_pair(ctx, 64, 7, pos, rad, den, (0.3, 1.0, 0.2), (320, 180))
    assert_voxelize_exact(vol, sun, ov)


def test_voxelize_small_config_bit_exact(ctx):
    cfg = configs.SMALL_64
    wl = workload.build(cfg)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    assert_voxelize_exact(vol, sun, ov)
    lv0 = vol.read_level(0)
    olv = ov.pyramid()
    assert np.array_equal(lv0, olv[0].astype(np.float32)), "level-0 texels differ"
    for l in range(1, cfg["mips"]):
        g = vol.read_level(l).astype(np.float64)
        np.testing.assert_allclose(g, olv[l], rtol=1e-6, atol=1e-7)
    assert vol.activeVoxels() == int(((ov.coverage()[0] > 0) | (ov.mask() > 0)).sum())


def test_voxelize_full_1080p_scene_bit_exact(ctx):
    cfg = configs.PLAIN_1080P
    wl = workload.build(cfg)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    assert_voxelize_exact(vol, sun, ov)


# 264^3: 33^3 = 35937 bricks, more than one pass of the brick-count scan
# (32768 per pass) with a ragged last pass
@pytest.mark.parametrize("dim,mips", [(2, 2), (20, 3), (96, 7), (128, 8), (264, 4)])
def test_voxelize_odd_sizes(ctx, dim, mips):
    pos, rad, den = random_scene(dim, 30, rmin=0.05, rmax=0.2)
    vol, sun, ov = make_pair(ctx, dim, mips, pos, rad, den, (-0.4, 0.8, 0.5), (97, 61))
    assert_voxelize_exact(vol, sun, ov)
    olv = ov.pyramid()
    for l in range(mips):
        np.testing.assert_allclose(vol.read_level(l).astype(np.float64), olv[l], rtol=1e-6,
                                   atol=1e-7)


def test_voxelize_edge_cases(ctx):
    # boards outside the box (culled from coverage but present in the sun
    # map), zero radius, a board touching the box face, fluffiness
    pos = np.array([[5.0, 5.0, 5.0], [0.0, 0.0, 0.0], [0.49, 0.0, 0.0], [-0.7, 0.1, 0.0],
                    [0.0, 0.3, 0.0]], np.float32)
    rad = np.array([0.3, 0.0, 0.1, 0.25, 0.05], np.float32)
    den = np.array([1.0, 1.0, 0.75, 0.5, 2.0], np.float32)
    vol, sun, ov = make_pair(ctx, 32, 6, pos, rad, den, (0.2, 0.9, -0.3), (128, 72),
                             fluffiness=1.5)
    assert_voxelize_exact(vol, sun, ov)


def test_empty_volume(ctx):
    z = np.zeros((0, 3), np.float32)
    vol, sun, ov = make_pair(ctx, 32, 6, z, np.zeros(0, np.float32), np.zeros(0, np.float32),
                             (0.3, 1, 0.2), (64, 64))
    cnt, dq = vol.read_coverage()
    assert cnt.sum() == 0 and dq.sum() == 0
    cam = cloudgb.Camera((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=32, height=32)
    img = cloudgb.ConeTraceShader().coneTrace(vol, cam)
    assert np.all(img == 0)


@pytest.mark.parametrize("fmt", [0, 1])
def test_revoxelize_rewrites_vacated_bricks(ctx, fmt):
    # bricks that held a cloud in one voxelize and hold nothing in the next are
    # rewritten (zeros), bricks empty in both are left alone: the pyramid and
    # its texture copies equal a fresh volume's after every voxelize
    sun = cloudgb.Sun((0.3, 1.0, 0.2), 96, 64)
    scenes = [random_scene(s, 24, spread=0.35) for s in (11, 12)] + [
        (np.zeros((0, 3), np.float32), np.zeros(0, np.float32), np.zeros(0, np.float32)),
        random_scene(13, 24, spread=0.35)]
    reused = cloudgb.CloudVolume(64, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, 7, fmt=fmt,
                                 ctx=ctx)
    cam = cloudgb.Camera((0.5, 0.6, -1.2), (0.5, 0.5, 0.5), width=48, height=40)
    shader = cloudgb.ConeTraceShader(viewSteps=32, vctSteps=8)
    for pos, rad, den in scenes:
        reused.set_billboards(pos, rad, den)
        reused.update()
        cloudgb.VoxelizeShader().voxelize(reused, sun)
        fresh = cloudgb.CloudVolume(64, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, 7,
                                    fmt=fmt, ctx=ctx)
        fresh.set_billboards(pos, rad, den)
        fresh.update()
        cloudgb.VoxelizeShader().voxelize(fresh, sun)
        for l in range(7):
            assert np.array_equal(reused.read_level(l), fresh.read_level(l)), l
        assert np.array_equal(shader.coneTrace(reused, cam), shader.coneTrace(fresh, cam))
        fresh.close()
    reused.close()


def test_error_paths(ctx):
    vol = cloudgb.CloudVolume(16, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, 5, ctx=ctx)
    cam = cloudgb.Camera((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=8, height=8)
    with pytest.raises(cloudgb.CloudError) as e:
        cloudgb.ConeTraceShader().coneTrace(vol, cam)
    assert e.value.status == 5  # not voxelized
    with pytest.raises(cloudgb.CloudError) as e:
        vol.set_billboards([[0, 0, np.nan]], [0.1])
        vol.update()
    assert e.value.status == 1
    with pytest.raises(cloudgb.CloudError) as e:
        vol.set_billboards([[0, 0, 0]], [2.0])  # radius beyond the box extent
        vol.update()
    assert e.value.status == 2
    vol.set_billboards([[0, 0, 0]], [0.2])
    vol.update()
    with pytest.raises(cloudgb.CloudError):
        cloudgb.VoxelizeShader().voxelize(vol, cloudgb.Sun((0, 1, 0), 16, 16))
    with pytest.raises(cloudgb.CloudError):
        cloudgb.CloudVolume(1024, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, 5, ctx=ctx)
    with pytest.raises(cloudgb.CloudError):
        cloudgb.CloudVolume(16, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, 9, ctx=ctx)
    cloudgb.VoxelizeShader().voxelize(vol, cloudgb.Sun((0.3, 1, 0.2), 16, 16))
    with pytest.raises(cloudgb.CloudError):
        cloudgb.ConeTraceShader(viewSteps=0).coneTrace(vol, cam)
    with pytest.raises(cloudgb.CloudError):
        cloudgb.ConeTraceShader(vctSteps=65).coneTrace(vol, cam)


def _oracle_image(ov, shader, cam, sun_dir, rect=None):
    return ov.render(cam, O.params_from_shader(shader), sun_dir, rect=rect)


def test_render_small_config_full_image(ctx):
    cfg = configs.SMALL_64
    wl = workload.build(cfg)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    cam = workload.make_camera(wl.cameras[0])
    img = shader.coneTrace(vol, cam).astype(np.float64)
    ref = _oracle_image(ov, shader, cam, sun.direction)
    err = np.abs(img - ref).max(axis=(0, 1))
    assert np.all(err <= IMAGE_TOL), f"max-abs per channel {err}"
    assert ref[..., 3].max() > 0.5  # the cloud is in view


@pytest.mark.parametrize("view", [0, 5, 11])
def test_render_1080p_scene_sampled_tiles(ctx, view):
    """Plain FP32 path on the 256^3 / 4096-board / noise scene; the oracle
    checks 32x32 tiles of the 1920x1080 image."""
    cfg = configs.PLAIN_1080P
    wl = workload.build(cfg)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    cam = workload.make_camera(wl.cameras[view])
    img = shader.coneTrace(vol, cam).astype(np.float64)
    alpha = img[..., 3]
    ys, xs = np.nonzero(alpha > 0.2)
    rng = np.random.default_rng(view)
    picks = [(960 - 16, 540 - 16)]
    for k in rng.choice(len(xs), size=min(3, len(xs)), replace=False):
        picks.append((int(min(max(xs[k] - 16, 0), 1920 - 32)), int(min(max(ys[k] - 16, 0), 1080 - 32))))
    for (x0, y0) in picks:
        ref = _oracle_image(ov, shader, cam, sun.direction, rect=(x0, y0, 32, 32))
        got = img[y0:y0 + 32, x0:x0 + 32]
        err = np.abs(got - ref).max(axis=(0, 1))
        assert np.all(err <= IMAGE_TOL), f"tile {x0},{y0}: max-abs {err}"


@pytest.mark.parametrize("cone_mode", [0, 1])
def test_cooperative_cones_match_fused_and_oracle(ctx, cone_mode):
    """Warp-cooperative sun cones (cone_lanes 1, 8, 32): the same samples and
    compositing order as the default fused trace, only a cooperative cone's
    terms are summed by a shuffle tree -- images within 1e-6 of the default
    and within the 1e-4 bar of the FP64 oracle; both cone modes, the noise
    scene at 200 x 120 and 32 x 32 tiles of a 1080p view."""
    cfg = configs.PLAIN_1080P
    wl = workload.build(cfg, width=200, height=120)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    kw = dict(wl.shader_kwargs(), coneMode=cone_mode)
    cam = workload.make_camera(wl.cameras[2])
    base = cloudgb.ConeTraceShader(coneLanes=0, **kw).coneTrace(vol, cam)
    ref = _oracle_image(ov, cloudgb.ConeTraceShader(**kw), cam, sun.direction)
    assert base[..., 3].max() > 0.2
    for lanes in (1, 8, 32):
        img = cloudgb.ConeTraceShader(coneLanes=lanes, **kw).coneTrace(vol, cam)
        assert np.abs(img - base).max() <= 1e-6, (lanes, float(np.abs(img - base).max()))
        err = np.abs(img.astype(np.float64) - ref).max()
        assert err <= IMAGE_TOL, (lanes, err)
    big = workload.make_camera(dict(wl.cameras[2], width=1920, height=1080))
    a = cloudgb.ConeTraceShader(coneLanes=0, **kw).coneTrace(vol, big)
    b = cloudgb.ConeTraceShader(coneLanes=32, **kw).coneTrace(vol, big)
    assert np.abs(a - b).max() <= 1e-6
    with pytest.raises(cloudgb.CloudError):
        cloudgb.ConeTraceShader(coneLanes=33, **kw).coneTrace(vol, cam)


def test_trace_cones_match_oracle(ctx):
    cfg = configs.SMALL_64
    wl = workload.build(cfg)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    rng = np.random.default_rng(5)
    pts = rng.uniform(8, 56, (500, 3)).astype(np.float32)
    for mode, kw in [(0, dict(vctSteps=16, vctConeAngle=0.1)),
                     (1, dict(vctSteps=16, vctConeAngle=0.9, vctConeInitialHeight=0.1,
                              vctDownScaling=1.0))]:
        shader = cloudgb.ConeTraceShader(coneMode=mode, **kw)
        got = shader.traceCone(vol, pts, sun.direction).astype(np.float64)
        ref = ov.trace_cones(pts.astype(np.float64), sun.direction, O.params_from_shader(shader))
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
        assert ref.max() > 0


def _unpack_bf16_fp16(packed):
    r = (packed.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    g = (packed >> 16).astype(np.uint16).view(np.float16).astype(np.float64)
    return r, g


def test_bf16_volume_sampling_and_rmse(ctx):
    """BF16 density + FP16 light storage: (a) the GPU image equals the oracle
    rendering the same quantized pyramid within the FP32 tolerance; (b) the
    image RMSE against the full-precision FP64 oracle stays within 1e-2."""
    cfg = configs.SMALL_64
    wl = workload.build(cfg)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map, fmt=cloudgb.FORMAT_BF16_FP16)
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    cam = workload.make_camera(wl.cameras[0])
    img = shader.coneTrace(vol, cam).astype(np.float64)
    full = _oracle_image(ov, shader, cam, sun.direction)
    rmse = float(np.sqrt(((img - full) ** 2).mean()))
    assert rmse <= 1e-2, f"RMSE vs FP64 oracle {rmse}"
    # feed the oracle the GPU's quantized pyramid
    levels = ov.pyramid()
    for l in range(cfg["mips"]):
        r, g = _unpack_bf16_fp16(vol.read_level(l))
        levels[l][..., 0] = r
        levels[l][..., 1] = g
        # the FP32 mips of levels <= 3 were rounded once from FP32 values
        np.testing.assert_allclose(r, ov.pyramid()[l][..., 0], rtol=2 ** -7, atol=1e-6)
    ov.set_pyramid(levels)
    ref = _oracle_image(ov, shader, cam, sun.direction)
    err = np.abs(img - ref).max(axis=(0, 1))
    assert np.all(err <= IMAGE_TOL), f"max-abs per channel {err}"


def test_noise_scene_small_image_full_parity(ctx):
    """Noise path (table-driven on the GPU, hashed in the oracle) on a full
    image of the 256^3 scene at reduced resolution."""
    cfg = configs.PLAIN_1080P
    wl = workload.build(cfg, width=160, height=90)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    for view in (1, 7):
        cam = workload.make_camera(wl.cameras[view])
        img = shader.coneTrace(vol, cam).astype(np.float64)
        ref = _oracle_image(ov, shader, cam, sun.direction)
        err = np.abs(img - ref).max(axis=(0, 1))
        assert np.all(err <= IMAGE_TOL), f"view {view}: max-abs per channel {err}"
        assert ref[..., 3].max() > 0.5


def test_wind_offset_noise_parity_and_table_reuse(ctx):
    """Wind (octaveOffsets = windVel * runTime) moves the noise domain: each
    image matches the oracle with the same offset; a shift within the tables'
    margin reuses them (one launch fewer), a larger one rebuilds them, and
    either way the image is bit-identical (the tables hold the hashed values)."""
    cfg = configs.PLAIN_1080P
    wl = workload.build(cfg, width=160, height=90)
    vol, sun, ov = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                             wl.sun_direction, wl.sun_map)
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    shader.windVel = (0.8, 0.1, -0.3)
    cam = workload.make_camera(wl.cameras[1])
    imgs, launches = {}, {}
    for t in (0.0, 0.5, 0.7, 3.0):
        shader.runTime = t
        n0 = ctx.launch_count
        imgs[t] = shader.coneTrace(vol, cam)
        launches[t] = ctx.launch_count - n0
        ref = _oracle_image(ov, shader, cam, sun.direction)
        err = np.abs(imgs[t].astype(np.float64) - ref).max(axis=(0, 1))
        assert np.all(err <= IMAGE_TOL), f"runTime {t}: max-abs per channel {err}"
    assert not np.array_equal(imgs[0.5], imgs[0.0])
    assert not np.array_equal(imgs[3.0], imgs[0.5])
    assert launches[0.7] == launches[0.5] - 1   # reused the tables built for 0.5
    assert launches[3.0] == launches[0.5]       # moved past the margin: rebuilt
    shader.runTime = 0.7                        # rebuilt around 0.7 this time
    assert np.array_equal(shader.coneTrace(vol, cam), imgs[0.7])


def test_board_uploads_order_with_voxelize_on_a_user_stream(ctx):
    """Uploads (made on the context's stream) and voxelizes on a caller's
    stream, back to back with no host synchronisation: each voxelize sees its
    own upload, and an upload waits for the voxelize still reading the last
    boards.  The final pyramid equals a default-stream voxelize of the last
    boards."""
    torch = pytest.importorskip("torch")
    cfg = configs.PLAIN_1080P
    wl = workload.build(cfg, width=64, height=36)
    sun = cloudgb.Sun(wl.sun_direction, *wl.sun_map)
    s = torch.cuda.Stream()
    vol = cloudgb.CloudVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION,
                              cfg["mips"], ctx=ctx)
    ref = cloudgb.CloudVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION,
                              cfg["mips"], ctx=ctx)
    rng = np.random.default_rng(5)
    sets = []
    for i in range(6):
        n = len(wl.scales) - 300 * (i % 3)  # board counts (and buffer sizes) change too
        pos = wl.positions[:n] + rng.uniform(-0.02, 0.02, (n, 3)).astype(np.float32)
        sets.append((pos, wl.scales[:n] * (1.0 + 0.2 * (i % 2)), wl.densities[:n]))
    for pos, sc, de in sets:
        vol.set_billboards(pos, sc, de)
        vol.update()
        cloudgb.VoxelizeShader().voxelize(vol, sun, stream=s.cuda_stream)
    ref.set_billboards(*sets[-1])
    ref.update()
    cloudgb.VoxelizeShader().voxelize(ref, sun)
    for l in (0, 2):
        assert np.array_equal(vol.read_level(l), ref.read_level(l)), f"level {l}"
    vol.close()
    ref.close()


def test_render_is_deterministic(ctx):
    cfg = configs.SMALL_64
    wl = workload.build(cfg, width=96, height=64)
    vol, sun, _ = make_pair(ctx, cfg["dim"], cfg["mips"], wl.positions, wl.scales, wl.densities,
                            wl.sun_direction, wl.sun_map)
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    cam = workload.make_camera(wl.cameras[0])
    a = shader.coneTrace(vol, cam)
    b = shader.coneTrace(vol, cam)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["small", "oblique", "edge"])
def test_gpu_matches_reference_shader_fixtures(ctx, name):
    """The GPU path against what the reference's own shaders computed
    (tests/golden/reference_shaders.npz): the same covered sun-map texels and
    winners, positions within 1e-5, highlight marks equal up to stores whose
    point lies within rounding of a voxel face (<= 0.1 %), and traceCone in the
    reference mode within 1e-4 relative (FP32 GPU vs the FP32 shader)."""
    import os
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                "reference_shaders.npz"))
    n, D, W, H = (int(x) for x in gold[f"sun_{name}_meta"])
    s = gold[f"sun_{name}_scene"]
    pos, rad, den = s[:3 * n].reshape(n, 3), s[3 * n:4 * n], s[4 * n:5 * n]
    sun_dir = tuple(float(x) for x in gold[f"sun_{name}_dir"])
    L = int(np.floor(np.log2(D))) + 1
    vol = cloudgb.CloudVolume(D, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, L, ctx=ctx)
    vol.set_billboards(pos, rad, den)
    vol.update()
    sun = cloudgb.Sun(sun_dir, W, H)
    cloudgb.VoxelizeShader().voxelize(vol, sun)
    keys, pm = vol.read_sun_map(sun)
    k = keys.reshape(-1)
    covered = np.flatnonzero(k != np.uint64(0xFFFFFFFFFFFFFFFF))
    np.testing.assert_array_equal(covered, gold[f"sun_{name}_texels"])
    np.testing.assert_array_equal((k[covered] & np.uint64(0xFFFFFFFF)).astype(np.int64),
                                  gold[f"sun_{name}_winner"].astype(np.int64))
    assert np.abs(pm.reshape(-1, 4)[covered, :3] - gold[f"sun_{name}_pos"]).max() <= 1e-5
    want = np.zeros(D ** 3, np.uint8)
    want[gold[f"marks_{name}"]] = 1
    got = vol.read_highlight().reshape(-1)
    assert (got != want).sum() <= 0.001 * want.sum()
    for kk, (steps, ang, h0, lodo, ds) in enumerate([(16, 0.1, 1.0, 0.0, 1.0),
                                                     (24, 0.6, 2.0, 0.5, 2.0)]):
        sh = cloudgb.ConeTraceShader(coneMode=1, vctSteps=steps, vctConeAngle=ang,
                                     vctConeInitialHeight=h0, vctLodOffset=lodo,
                                     vctDownScaling=ds)
        vals = sh.traceCone(vol, gold[f"cone_{name}_{kk}_voxpos"], sun.direction)
        ref = gold[f"cone_{name}_{kk}_value"]
        np.testing.assert_allclose(vals, ref, rtol=1e-4, atol=1e-5)
    vol.close()


def test_error_stats_fp64_on_gpu(ctx):
    """cg_image_error_stats: FP64 GPU reduction against numpy, FP64 and FP32
    references, repeated calls bit-identical (fixed reduction order)."""
    rng = np.random.default_rng(7)
    img = rng.uniform(0, 1, (123, 77, 4)).astype(np.float32)
    ref64 = img.astype(np.float64) + rng.normal(0, 1e-3, img.shape)
    ref32 = ref64.astype(np.float32)
    for ref in (ref64, ref32):
        st = ctx.error_stats(img, ref)
        d = img.astype(np.float64) - ref.astype(np.float64)
        np.testing.assert_array_equal(st["max_abs"], np.abs(d).reshape(-1, 4).max(axis=0))
        np.testing.assert_allclose(st["rmse"], np.sqrt((d ** 2).reshape(-1, 4).mean(axis=0)),
                                   rtol=1e-12)
        assert st["max_abs_all"] == np.abs(d).max()
        np.testing.assert_allclose(st["rmse_all"], np.sqrt((d ** 2).mean()), rtol=1e-12)
        assert ctx.error_stats(img, ref) == st


def test_precision_form_512_4k(ctx):
    """The precision workload (512^3, 16384 boards, 5-octave fBm, 3840x2160,
    128 view steps, 32-step cone): the FP32 volume and the BF16/FP16 volume are
    rendered on the GPU and 48x48 tiles are checked against the FP64 oracle,
    with the error statistics reduced on the GPU in FP64.  FP32: max-abs <= 1e-4
    (the plain-path bar); BF16/FP16: RMSE <= 1e-2, and its error is reported
    against the FP32 run's."""
    cfg = configs.PRECISION_4K
    wl = workload.build(cfg)
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    cam = workload.make_camera(wl.cameras[0])
    W, H = cam.width, cam.height
    sun = cloudgb.Sun(wl.sun_direction, *wl.sun_map)
    ov = O.OracleVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, cfg["mips"])
    assert ov.set_boards(wl.positions, wl.scales, wl.densities) == 0
    assert ov.voxelize(sun.direction, *wl.sun_map) == 0
    images = {}
    for fmt in (cloudgb.FORMAT_RGBA32F, cloudgb.FORMAT_BF16_FP16):
        vol = cloudgb.CloudVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION,
                                  cfg["mips"], fmt=fmt, ctx=ctx)
        vol.set_billboards(wl.positions, wl.scales, wl.densities)
        vol.update()
        cloudgb.VoxelizeShader().voxelize(vol, sun)
        images[fmt] = shader.coneTrace(vol, cam)
        vol.close()
    alpha = images[cloudgb.FORMAT_RGBA32F][..., 3]
    ys, xs = np.nonzero(alpha > 0.2)
    assert len(xs) > 0
    rng = np.random.default_rng(3)
    T = 48
    picks = [(W // 2 - T // 2, H // 2 - T // 2)]
    for k in rng.choice(len(xs), size=3, replace=False):
        picks.append((int(min(max(xs[k] - T // 2, 0), W - T)),
                      int(min(max(ys[k] - T // 2, 0), H - T))))
    refs = [_oracle_image(ov, shader, cam, sun.direction, rect=(x0, y0, T, T))
            for (x0, y0) in picks]
    ref = np.concatenate(refs, axis=0)

    def tiles(img):
        return np.concatenate([img[y0:y0 + T, x0:x0 + T] for (x0, y0) in picks], axis=0)

    st32 = ctx.error_stats(tiles(images[cloudgb.FORMAT_RGBA32F]), ref)
    st16 = ctx.error_stats(tiles(images[cloudgb.FORMAT_BF16_FP16]), ref)
    assert st32["max_abs_all"] <= IMAGE_TOL, st32
    assert st16["rmse_all"] <= 1e-2, st16
    assert st16["rmse_all"] >= st32["rmse_all"]
    print(f"precision form: FP32 max-abs {st32['max_abs_all']:.3g} rmse {st32['rmse_all']:.3g}; "
          f"BF16/FP16 max-abs {st16['max_abs_all']:.3g} rmse {st16['rmse_all']:.3g}")
