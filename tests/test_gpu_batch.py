"""GPU tests of the batching form: many clouds and views per frame in one
persistent launch, every launch shape of the autotuner, the occupancy brick
sizes, and the frame replayed as a CUDA graph.

Bars: every configuration renders the images of the single-view fused
renderer (max-abs <= 1e-6 per channel: same per-sample arithmetic and
compositing order); brick sizes change nothing (empty bricks are exactly 0).
"""
import numpy as np
import pytest

import cloudgb
from cloudgb import _lib, configs, workload

pytestmark = pytest.mark.gpu

TOL = 1e-6


def make_batch(ctx, clouds=3, views=5, max_pixels=160 * 120, fmt=cloudgb.FORMAT_RGBA32F):
    bw = workload.build_batch(configs.BATCH_48x128, clouds=clouds, views=views,
                              max_pixels=max_pixels)
    sun = cloudgb.Sun(bw.sun_direction, 320, 180)
    vols = []
    for c in bw.clouds:
        v = cloudgb.CloudVolume(c["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, c["mips"],
                                fmt=fmt, ctx=ctx)
        v.set_billboards(c["positions"], c["scales"], c["densities"])
        v.update()
        cloudgb.VoxelizeShader().voxelize(v, sun)
        vols.append(v)
    cams = [workload.make_camera(vd) for vd in bw.views]
    outs = [cloudgb.DeviceBuffer(vd["width"] * vd["height"] * 16) for vd in bw.views]
    views = [(vols[vd["cloud"]], cams[i], outs[i]) for i, vd in enumerate(bw.views)]
    shader = cloudgb.ConeTraceShader(viewSteps=48, vctSteps=16, vctConeAngle=0.06,
                                     densityScale=3.0, numOctaves=3, noiseSeed=5)
    return bw, sun, vols, cams, outs, views, shader


def read(out, cam):
    return out.download((cam.height, cam.width, 4))


def test_occupancy_brick_sizes_render_identically(ctx):
    bw, sun, vols, cams, outs, views, shader = make_batch(ctx, clouds=1, views=1)
    vol, cam = vols[0], cams[0]
    images = []
    for brick in (8, 4, 16, 8):
        vol.set_occupancy_brick(brick)
        images.append(shader.coneTrace(vol, cam))
    for img in images[1:]:
        np.testing.assert_array_equal(img, images[0])
    # and after a fresh voxelize with a non-default brick
    vol.set_occupancy_brick(4)
    cloudgb.VoxelizeShader().voxelize(vol, sun)
    np.testing.assert_array_equal(shader.coneTrace(vol, cam), images[0])
    vol.set_occupancy_brick(8)


@pytest.mark.parametrize("lanes", [1, 4, 8, 32])
@pytest.mark.parametrize("unroll", [1, 2, 4])
def test_batch_matches_single_view_renders(ctx, lanes, unroll):
    bw, sun, vols, cams, outs, views, shader = make_batch(ctx)
    ref = [shader.coneTrace(v, c) for (v, c, _) in views]
    ctx.render_batch(views, shader, config=(lanes, unroll, 0))
    ctx.synchronize()
    for (v, c, o), r in zip(views, ref):
        got = read(o, c)
        assert np.abs(got - r).max() <= TOL
    assert max(float(r[..., 3].max()) for r in ref) > 0.1  # the clouds are visible


def test_batch_bf16_volumes(ctx):
    bw, sun, vols, cams, outs, views, shader = make_batch(ctx, fmt=cloudgb.FORMAT_BF16_FP16)
    ref = [shader.coneTrace(v, c) for (v, c, _) in views]
    ctx.render_batch(views, shader, config=(8, 2, 0))
    ctx.synchronize()
    for (v, c, o), r in zip(views, ref):
        assert np.abs(read(o, c) - r).max() <= TOL


def test_batch_rejects_mixed_formats_and_mlp(ctx):
    bw, sun, vols, cams, outs, views, shader = make_batch(ctx, clouds=1, views=1)
    v16 = cloudgb.CloudVolume(64, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, 7,
                              fmt=cloudgb.FORMAT_BF16_FP16, ctx=ctx)
    v16.set_billboards(bw.clouds[0]["positions"][:8], bw.clouds[0]["scales"][:8])
    v16.update()
    cloudgb.VoxelizeShader().voxelize(v16, sun)
    with pytest.raises(_lib.CloudError) as e:
        ctx.render_batch(views + [(v16, cams[0], outs[0])], shader)
    assert e.value.status == 9  # CG_ERR_UNSUPPORTED
    with pytest.raises(_lib.CloudError):
        ctx.render_batch(views, shader, config=(3, 1, 0))
    with pytest.raises(_lib.CloudError):
        ctx.render_batch(views, shader, config=(1, 1, 12))


def test_autotune_picks_a_configuration(ctx):
    bw, sun, vols, cams, outs, views, shader = make_batch(ctx)
    best, table = ctx.autotune(views, shader, repeats=1)
    assert len(table) == 36 and all(t > 0 for t in table.values())
    assert table[best] == min(table.values())
    assert ctx.trace_config == best
    ref = [shader.coneTrace(v, c) for (v, c, _) in views]
    ctx.render_batch(views, shader)  # the tuned configuration
    ctx.synchronize()
    for (v, c, o), r in zip(views, ref):
        assert np.abs(read(o, c) - r).max() <= TOL
    ctx.trace_config = (1, 1, 8)


def test_frame_graph_replay(ctx):
    bw, sun, vols, cams, outs, views, shader = make_batch(ctx)
    g = cloudgb.FrameGraph(ctx, vols, sun, views, shader)
    g.launch()
    ctx.synchronize()
    first = [read(o, c) for (v, c, o) in views]
    ref = [shader.coneTrace(v, c) for (v, c, _) in views]
    for a, r in zip(first, ref):
        assert np.abs(a - r).max() <= TOL
    # moved billboards (same count): the replay voxelizes them again
    c0 = bw.clouds[0]
    vols[0].set_billboards(c0["positions"] + np.float32(0.03), c0["scales"], c0["densities"])
    vols[0].update()
    g.launch()
    ctx.synchronize()
    moved = [read(o, c) for (v, c, o) in views]
    cloudgb.VoxelizeShader().voxelize(vols[0], sun)
    ref2 = [shader.coneTrace(v, c) for (v, c, _) in views]
    for a, r in zip(moved, ref2):
        assert np.abs(a - r).max() <= TOL
    assert any(np.abs(a - b).max() > 1e-3 for a, b in zip(moved, first))
    g.close()


@pytest.mark.parametrize("lanes", [1, 32])
def test_batch_matches_oracle(ctx, lanes):
    """Every view of a batch against the FP64 oracle directly (not only
    through the single-view renderer): max-abs <= 1e-4 per RGBA channel."""
    from oracle import oracle as O
    bw, sun, vols, cams, outs, views, shader = make_batch(ctx)
    ctx.render_batch(views, shader, config=(lanes, 1, 0))
    ctx.synchronize()
    oracles = {}
    P = O.params_from_shader(shader)
    seen = 0.0
    for i, vd in enumerate(bw.views):
        k = vd["cloud"]
        if k not in oracles:
            c = bw.clouds[k]
            ov = O.OracleVolume(c["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, c["mips"])
            ov.set_boards(c["positions"], c["scales"], c["densities"])
            ov.voxelize(sun.direction, sun.map_width, sun.map_height)
            oracles[k] = ov
        ref = oracles[k].render(cams[i], P, sun.direction)
        got = read(outs[i], cams[i]).astype(np.float64)
        err = np.abs(got - ref).max(axis=(0, 1))
        assert np.all(err <= 1e-4), (i, err)
        seen = max(seen, float(ref[..., 3].max()))
    assert seen > 0.1
