"""The C++ host mirror (include/cloudgb.hpp): tests/cpp/frame.cpp builds with
g++ against the headers and libcloudgb.so, its regenerateBillboards stream is
the Python mirror's, and (GPU) its frame -- update, voxelize, coneTrace in the
reference's order -- gives the Python API's image bit for bit."""
import os
import struct
import subprocess

import numpy as np
import pytest

from cloudgb import _lib, configs, scene, workload

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "frame.cpp")


@pytest.fixture(scope="module")
def frame_exe(tmp_path_factory):
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("cpp") / "frame")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir, "-lcloudgb",
           f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_builds_and_links(frame_exe):
    out = subprocess.run([frame_exe, "version"], capture_output=True, text=True, check=True)
    assert int(out.stdout) == _lib.load().cg_abi_version()


@pytest.mark.parametrize("count,seed", [(1, 0), (200, 21), (777, 12345)])
def test_regenerate_billboards_matches_python(frame_exe, tmp_path, count, seed):
    path = tmp_path / "b.bin"
    subprocess.run([frame_exe, "regen", str(path), str(count), str(seed)], check=True)
    data = np.fromfile(path, np.float32)
    pos, sc = data[:3 * count].reshape(count, 3), data[3 * count:]
    # the Python mirror's CloudVolume.regenerateBillboards stream
    rng = scene.SplitMix64(seed)
    u = rng.uniform(3 * count).reshape(count, 3)
    ppos = (-2.5 + 5.0 * u).astype(np.float32)
    psc = rng.uniform_range(count, 1.0, 2.5).astype(np.float32)
    assert np.array_equal(pos, ppos) and np.array_equal(sc, psc)


@pytest.mark.gpu
def test_cpp_frame_equals_python_frame(frame_exe, tmp_path, ctx):
    import cloudgb
    cfg = configs.SMALL_64
    wl = workload.build(cfg, boards=48, width=96, height=64)
    cam = wl.cameras[0]
    kw = wl.shader_kwargs()
    kw.update(numOctaves=3, noiseSeed=5, windVel=(0.2, 0.0, 0.1), runTime=1.5)
    n = len(wl.scales)
    inp = tmp_path / "scene.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<8i", n, cfg["dim"], cfg["mips"], wl.sun_map[0], wl.sun_map[1],
                            cam["width"], cam["height"], kw["numOctaves"]))
        f.write(struct.pack("<13f", *configs.VOLUME_BOUNDS, *configs.VOLUME_POSITION,
                            *wl.sun_direction, *cam["eye"], cam["fov"], 1.0))
        f.write(struct.pack("<3f", *cam["target"]))
        f.write(struct.pack("<3i", kw["viewSteps"], kw["vctSteps"], kw["noiseSeed"]))
        f.write(struct.pack("<12f", kw["vctConeAngle"], kw["vctConeInitialHeight"],
                            kw["vctConeMinRadius"], kw["densityScale"], kw["ambient"],
                            kw["noiseFrequency"], kw["freqStep"], kw["persStep"],
                            kw["runTime"], *kw["windVel"]))
        f.write(np.ascontiguousarray(wl.positions, np.float32).tobytes())
        f.write(np.ascontiguousarray(wl.scales, np.float32).tobytes())
        f.write(np.ascontiguousarray(wl.densities, np.float32).tobytes())
    out = tmp_path / "img.bin"
    r = subprocess.run([frame_exe, "render", str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    img_cpp = np.fromfile(out, np.float32).reshape(cam["height"], cam["width"], 4)
    # the same frame through the Python mirror
    vol = cloudgb.CloudVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION,
                              cfg["mips"], ctx=ctx)
    vol.set_billboards(wl.positions, wl.scales, wl.densities)
    vol.update()
    cloudgb.VoxelizeShader().voxelize(vol, cloudgb.Sun(wl.sun_direction, *wl.sun_map))
    img_py = cloudgb.ConeTraceShader(**kw).coneTrace(vol, workload.make_camera(cam))
    assert np.array_equal(img_cpp, img_py)
    assert img_py[..., 3].max() > 0.3
    assert f"active voxels {vol.activeVoxels()}" in r.stdout
    vol.close()
