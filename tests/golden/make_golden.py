"""Generate tests/golden/reference_shaders.npz from the reference's own shader
code (oracle/_ref/libref_shaders.so, built by oracle/build_ref.py from the
reference's res/*.glsl through oracle/ref_shim/).

Cases (all inputs seeded; the scene generator is cloudgb.scene's SplitMix64):
  sun_<case>   first_voxelize + billboard_vert_instanced over a scene: covered
               texels, their winning board, depth and surface position
  marks_<case> second_voxelize over that position map: marked voxels
  marks_rand   second_voxelize over a seeded random position map whose points
               straddle the volume box (out-of-range stores are dropped)
  cone_<case>  traceCone over the scene's mark volume (level 0 = marks,
               2x2x2 box mips, float storage) at seeded world positions
  cone_rand    traceCone over a seeded random float mip chain

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "cloud-renderer_gb300"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

from cloudgb import configs, scene  # noqa: E402
from oracle import build_ref, ref_shaders as R  # noqa: E402

OUT = os.path.join(HERE, "reference_shaders.npz")
BOUNDS = configs.VOLUME_BOUNDS
VPOS = configs.VOLUME_POSITION

# (name, boards, board seed, radius scale, ball radius, D, map W, map H, sun direction)
SCENES = [
    ("small", 64, 1, 1.0, 0.35, 64, 160, 90, configs.SUN_DIRECTION),
    ("oblique", 200, 3, 0.5, 0.35, 48, 128, 128, (-0.6, 0.5, 0.3)),
    ("edge", 48, 5, 1.0, 0.48, 32, 96, 64, (0.1, -1.0, 0.35)),
]
CONE_PARAMS = [  # (steps, full cone angle, initial height, lod offset, down scaling)
    (16, 0.1, 1.0, 0.0, 1.0),
    (24, 0.6, 2.0, 0.5, 2.0),
]


def unit(v):
    v = np.asarray(v, np.float64)
    return tuple(float(x) for x in v / np.linalg.norm(v))


def box_mips(level0, levels):
    out = [np.asarray(level0, np.float64)]
    for _ in range(1, levels):
        c = out[-1]
        n = c.shape[0]
        m = max(1, n // 2)
        idx = np.minimum(np.arange(2 * m), n - 1)
        c = c[np.ix_(idx, idx, idx)]
        out.append(c.reshape(m, 2, m, 2, m, 2).mean(axis=(1, 3, 5)))
    return [l.astype(np.float32) for l in out]


def main():
    if build_ref.build() is None:
        raise SystemExit("reference shader sources not found: cannot generate fixtures")
    rng = np.random.default_rng(20240611)
    data = {}
    for name, n, seed, rs, ball, D, W, H, sun in SCENES:
        pos, rad, dens = scene.billboards(seed, n, ball_radius=ball, radius_scale=rs,
                                          volume_position=VPOS)
        sun = unit(sun)
        pm, win, dep, _ = R.sun_pass(pos, rad, VPOS, BOUNDS, sun, W, H)
        cov = np.flatnonzero(win.reshape(-1) >= 0).astype(np.int32)
        data[f"sun_{name}_scene"] = np.concatenate([pos.astype(np.float32).reshape(-1),
                                                    rad.astype(np.float32).reshape(-1),
                                                    dens.astype(np.float32).reshape(-1)])
        data[f"sun_{name}_meta"] = np.array([n, D, W, H], np.int32)
        data[f"sun_{name}_dir"] = np.array(sun, np.float32)
        data[f"sun_{name}_texels"] = cov
        data[f"sun_{name}_winner"] = win.reshape(-1)[cov].astype(np.int32)
        data[f"sun_{name}_depth"] = dep.reshape(-1)[cov].astype(np.float32)
        data[f"sun_{name}_pos"] = pm.reshape(-1, 4)[cov, :3].astype(np.float32)
        marks = R.second_pass(pm, D, VPOS, BOUNDS)
        data[f"marks_{name}"] = np.flatnonzero(marks.reshape(-1)).astype(np.int32)
        # cone over the mark volume
        L = int(np.log2(D)) + 1 if (D & (D - 1)) == 0 else int(np.floor(np.log2(D))) + 1
        levels = box_mips(marks.astype(np.float32), L)
        wp = rng.uniform(0.2, 0.8, (96, 3)).astype(np.float32)
        for k, (steps, ang, h0, lodo, ds) in enumerate(CONE_PARAMS):
            vals, vps = [], []
            for p in wp:
                v, vp = R.trace_cone(levels, D, VPOS, BOUNDS, p, sun, steps, ang, h0, lodo, ds)
                vals.append(v)
                vps.append(vp)
            data[f"cone_{name}_{k}_levels"] = np.array([L], np.int32)
            data[f"cone_{name}_{k}_voxpos"] = np.array(vps, np.float32)
            data[f"cone_{name}_{k}_value"] = np.array(vals, np.float32)
    # second pass over a random position map straddling the box
    D, W, H = 40, 64, 48
    lo = np.array(VPOS) + BOUNDS[0] - 0.05
    hi = np.array(VPOS) + BOUNDS[1] + 0.05
    pm = np.zeros((H, W, 4), np.float32)
    pm[..., :3] = rng.uniform(lo, hi, (H, W, 3))
    pm[..., 3] = (rng.uniform(size=(H, W)) < 0.7).astype(np.float32)
    data["marks_rand_posmap"] = pm
    data["marks_rand_meta"] = np.array([D, W, H], np.int32)
    data["marks_rand"] = np.flatnonzero(R.second_pass(pm, D, VPOS, BOUNDS).reshape(-1)).astype(
        np.int32)
    # traceCone over a random float mip chain
    D = 16
    levels = box_mips(rng.uniform(0, 1, (D, D, D)) ** 3, 5)
    data["cone_rand_level0"] = levels[0]
    wp = rng.uniform(0.1, 0.9, (128, 3)).astype(np.float32)
    dirs = rng.normal(size=(128, 3)).astype(np.float32)
    for k, (steps, ang, h0, lodo, ds) in enumerate(CONE_PARAMS):
        vals, vps = [], []
        for p, d in zip(wp, dirs):
            v, vp = R.trace_cone(levels, D, VPOS, BOUNDS, p, d, steps, ang, h0, lodo, ds)
            vals.append(v)
            vps.append(vp)
        data[f"cone_rand_{k}_voxpos"] = np.array(vps, np.float32)
        data[f"cone_rand_{k}_value"] = np.array(vals, np.float32)
    data["cone_rand_dirs"] = dirs
    np.savez_compressed(OUT, **data)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
