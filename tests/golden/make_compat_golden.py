"""Generate tests/golden/reference_compat.npz: the reference's cone-trace pass
(billboard_vert_instanced.glsl + conetrace_frag.glsl compiled as C++ through
oracle/ref_shim/, driven by oracle/ref_shim/ref_driver.inc's
ref_compat_render the way ConeTraceShader::coneTrace drives them) on seeded
scenes at the reference's own scale (cloudgb.configs.COMPAT_REF).

The light channel the shader's traceCone reads comes from the FP64 oracle's
voxelization of the same boards (itself pinned to the reference's voxelize
shaders by reference_shaders.npz); the noise map is
oracle.compat_noise_map(seed).

Cases: name -> (camera index or explicit camera, board count, parameter
overrides).  Per case the file holds the boards, camera, sun, parameter block
(raw bytes of or_compat_params) and the image (row 0 = top).

    python tests/golden/make_compat_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "cloud-renderer_gb300"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

from cloudgb import configs, workload  # noqa: E402
from oracle import build_ref, oracle as O, ref_shaders as R  # noqa: E402

OUT = os.path.join(HERE, "reference_compat.npz")
W, H = 96, 64

CASES = {
    "default": (0, 200, {}),
    "noise_only": (3, 200, dict(do_cone_trace=0)),
    "cone_only": (5, 200, dict(do_noise=0, vct_steps=24, vct_lod_offset=0.5,
                               vct_down_scaling=2.0)),
    "quad": (1, 120, dict(show_quad=1)),
    "wind": (2, 200, dict(num_octaves=3, octave_offsets=(0.3, -0.2, 0.1), min_noise_steps=3,
                          max_noise_steps=6, noise_seed=9, freq_step=2.5, pers_step=0.6)),
    "inside": (dict(eye=(25.0, 0.5, -1.5), target=(25.3, 0.0, 3.0)), 64,
               dict(vct_cone_angle=0.5, noise_opacity=2.0)),
}


def compat_params(**kw):
    """or_compat_params with the reference's defaults (ConeTraceShader.hpp:15-32),
    no early termination."""
    p = O.or_compat_params()
    d = dict(show_quad=0, do_noise=1, do_cone_trace=1, step_size=0.01, noise_opacity=4.0,
             num_octaves=4, freq_step=3.0, pers_step=0.5, adjust_size=40.0, min_noise_steps=2,
             max_noise_steps=8, min_noise_color=0.2, noise_color_scale=0.45, noise_seed=1,
             vct_steps=16, vct_cone_angle=0.9, vct_cone_initial_height=0.1, vct_lod_offset=0.0,
             vct_down_scaling=1.0, near_plane=0.01, transmittance_cutoff=0.0,
             clear_color=(0.2, 0.3, 0.5, 1.0), octave_offsets=(0.0, 0.0, 0.0))
    d.update(kw)
    for k, v in d.items():
        if k in ("clear_color", "octave_offsets"):
            getattr(p, k)[:] = [float(x) for x in v]
        else:
            setattr(p, k, v)
    return p


def case_inputs(cam, n):
    """Scene, camera dict, oracle volume (voxelized) for a case."""
    cfg = configs.COMPAT_REF
    wl = workload.build_compat(cfg, boards=n, width=W, height=H)
    if isinstance(cam, int):
        c = dict(wl.cameras[cam])
    else:
        c = dict(cam, fov=60.0, width=W, height=H)
    ov = O.OracleVolume(cfg["dim"], cfg["bounds"], cfg["position"], cfg["mips"])
    ov.set_boards(wl.positions, wl.scales, np.ones(n, np.float32))
    ov.voxelize(wl.sun_direction, *cfg["sun_map"])
    return wl, c, ov


def main():
    if build_ref.build() is None:
        raise SystemExit("reference shader sources not found: cannot generate fixtures")
    cfg = configs.COMPAT_REF
    data = {}
    for name, (cam, n, kw) in CASES.items():
        wl, c, ov = case_inputs(cam, n)
        P = compat_params(**kw)
        light = [lv[..., 1].astype(np.float32) for lv in ov.pyramid()]
        img, shaded = R.compat_render(wl.positions, wl.scales, cfg["position"], cfg["bounds"],
                                      cfg["dim"], light, O.compat_noise_map(P.noise_seed),
                                      c["eye"], c["target"], (0.0, 1.0, 0.0), c["fov"], W, H,
                                      wl.sun_direction, P)
        data[f"{name}_image"] = img
        data[f"{name}_params"] = np.frombuffer(bytes(P), np.uint8).copy()
        data[f"{name}_camera"] = np.array(list(c["eye"]) + list(c["target"]) + [c["fov"]],
                                          np.float64)
        data[f"{name}_boards"] = np.array([n], np.int32)
        data[f"{name}_shaded"] = np.array([shaded], np.int64)
        print(name, "fragments", shaded, "range", float(img.min()), float(img.max()))
    data["size"] = np.array([W, H], np.int32)
    np.savez_compressed(OUT, **data)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
