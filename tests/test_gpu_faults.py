"""Failure detection on the GPU without a fault: the tensor-core kernels'
bounded mbarrier waits are made to run out (a barrier nothing arrives on), the
host reads the error status, and the context keeps working."""
import ctypes

import numpy as np
import pytest

import cloudgb
from cloudgb import _lib, configs, surrogate, workload

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_survives(ctx):
    lib = _lib.load()
    waited = ctypes.c_uint64()
    st = lib.cg_context_check_wait_timeout(ctx.handle, 20000, ctypes.byref(waited))
    assert st == 6, "CG_ERR_DEVICE_FAULT expected: the bound must fire"
    assert b"ran out" in lib.cg_last_error()
    assert 20000 <= waited.value < 500000, waited.value  # ~20 ms, not forever
    # invalid limits are refused before any launch
    assert lib.cg_context_check_wait_timeout(ctx.handle, 0, ctypes.byref(waited)) == 2
    # the context is still usable: a render after the probe is deterministic
    cfg = configs.SMALL_64
    wl = workload.build(cfg, boards=16, width=48, height=32)
    vol = cloudgb.CloudVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION,
                              cfg["mips"], ctx=ctx)
    vol.set_billboards(wl.positions, wl.scales, wl.densities)
    vol.update()
    cloudgb.VoxelizeShader().voxelize(vol, cloudgb.Sun(wl.sun_direction, *wl.sun_map))
    sh = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    cam = workload.make_camera(wl.cameras[0])
    a = sh.coneTrace(vol, cam)
    assert np.array_equal(a, sh.coneTrace(vol, cam)) and a[..., 3].max() > 0
    vol.close()


def test_training_wait_runs_out_without_update(ctx):
    """The training kernel's layer barrier is never completed (no MMA is
    issued) and its waits are limited to 20 ms: the call must report
    CG_ERR_DEVICE_FAULT, make no update (parameters, Adam moments and step
    unchanged), and the model must keep training afterwards."""
    lib = _lib.load()
    m = surrogate.SunMLP(ctx, seed=21)
    rng = np.random.default_rng(4)
    f = rng.uniform(0, 1, (4096, 16)).astype(np.float32)
    tau = rng.uniform(0, 1, 4096).astype(np.float32)
    m.fit_normalization(f, tau)
    m.train(f, tau, steps=3, batch=1024)
    before = m.get_params()
    df, dt = cloudgb.DeviceBuffer(f.nbytes), cloudgb.DeviceBuffer(tau.nbytes)
    df.upload(f)
    dt.upload(tau)
    st = lib.cg_mlp_check_train_timeout(m.handle, df.ptr, dt.ptr, f.shape[0], 2, 20000)
    assert st == 6, "CG_ERR_DEVICE_FAULT expected: the bound must fire"
    assert b"ran out" in lib.cg_last_error()
    after = m.get_params()
    for a, b in zip(before[:3], after[:3]):
        assert np.array_equal(a, b)
    assert before[3] == after[3] == 3
    # invalid limits are refused before any launch
    assert lib.cg_mlp_check_train_timeout(m.handle, df.ptr, dt.ptr, f.shape[0], 2, 0) == 2
    # the model and the context still work: a normal step updates
    losses = m.train(f, tau, steps=2, batch=1024)
    assert np.isfinite(losses).all()
    assert m.get_params()[3] == 5
    assert not np.array_equal(m.get_params()[0], before[0])
    df.free()
    dt.free()
