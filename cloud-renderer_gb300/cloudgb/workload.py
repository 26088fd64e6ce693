"""Build a benchmark workload (scene, sun, cameras, render parameters) from a
configuration in cloudgb.configs, for the GPU path and its checkers alike."""
from dataclasses import dataclass, field

import numpy as np

from . import configs, scene


@dataclass
class Workload:
    cfg: dict
    positions: np.ndarray
    scales: np.ndarray
    densities: np.ndarray
    sun_direction: tuple
    sun_map: tuple
    cameras: list = field(default_factory=list)

    @property
    def dim(self):
        return self.cfg["dim"]

    def shader_kwargs(self):
        c = self.cfg
        return dict(viewSteps=c["view_steps"], vctSteps=c["sun_steps"],
                    vctConeAngle=2.0 * c["cone_half_angle"], vctConeInitialHeight=c["cone_h0"],
                    vctConeMinRadius=c["cone_min_radius"], densityScale=c["density_scale"],
                    ambient=c["ambient"], numOctaves=c["noise_octaves"],
                    noiseSeed=c["noise_seed"], noiseFrequency=c["noise_frequency"],
                    freqStep=c["noise_lacunarity"], persStep=c["noise_gain"])


def camera_dicts(cfg):
    cam = cfg["camera"]
    if "eye" in cam:
        return [dict(eye=cam["eye"], target=cam["target"], fov=cam["fov"], width=cam["width"],
                     height=cam["height"])]
    eyes = scene.orbit_cameras(cfg["orbit_seed"], cfg["orbits"], radius=cfg["orbit_radius"])
    return [dict(eye=e, target=(0.5, 0.5, 0.5), fov=cam["fov"], width=cam["width"],
                 height=cam["height"]) for e in eyes]


def build(cfg, boards=None, width=None, height=None):
    """Scene for cfg; `boards`, `width`, `height` override the sizes (used by
    tests to shrink a workload while keeping its distributions)."""
    n = boards if boards is not None else cfg["boards"]
    pos, rad, dens = scene.billboards(cfg["board_seed"], n, ball_radius=cfg["ball_radius"],
                                      radius_range=cfg["radius_range"],
                                      radius_scale=cfg["radius_scale"],
                                      density_range=cfg["density_range"],
                                      volume_position=configs.VOLUME_POSITION)
    cams = camera_dicts(cfg)
    for c in cams:
        if width:
            c["width"] = width
        if height:
            c["height"] = height
    d = np.asarray(configs.SUN_DIRECTION, np.float64)
    d = tuple(float(x) for x in d / np.sqrt((d * d).sum()))
    return Workload(cfg=cfg, positions=pos, scales=rad, densities=dens, sun_direction=d,
                    sun_map=cfg["sun_map"], cameras=cams)


def make_camera(c):
    from . import Camera
    return Camera(c["eye"], c["target"], fov_y_degrees=c["fov"], width=c["width"],
                  height=c["height"])


@dataclass
class BatchWorkload:
    """The batching form: independent clouds (sizes, board counts) and views
    (cloud, camera dict with resolution)."""
    cfg: dict
    clouds: list  # dicts: dim, mips, positions, scales, densities
    views: list   # dicts: cloud, eye, target, fov, width, height
    sun_direction: tuple


def build_batch(cfg, clouds=None, views=None, max_pixels=None):
    """Seeded batch scene: cloud sizes uniform from cfg['dims'], board counts
    uniform in cfg['boards_range'], the same board distributions as
    the single-cloud workloads; view resolutions uniform from
    cfg['resolutions'] (optionally capped at max_pixels), cameras on the
    orbit sphere; view v renders cloud v mod clouds.  `clouds` / `views`
    shrink the counts for tests."""
    nc = clouds if clouds is not None else cfg["clouds"]
    nv = views if views is not None else cfg["views"]
    rng = scene.SplitMix64(cfg["seed"])
    cl = []
    for k in range(nc):
        u = rng.uniform(2)
        dim = cfg["dims"][min(int(u[0] * len(cfg["dims"])), len(cfg["dims"]) - 1)]
        lo, hi = cfg["boards_range"]
        n = int(lo + u[1] * (hi - lo))
        pos, rad, dens = scene.billboards(cfg["seed"] * 1000 + k, n,
                                          radius_range=cfg["radius_range"],
                                          radius_scale=cfg["radius_scale"],
                                          volume_position=configs.VOLUME_POSITION)
        mips = int(np.floor(np.log2(dim))) + 1
        cl.append(dict(dim=dim, mips=mips, positions=pos, scales=rad, densities=dens))
    eyes = scene.orbit_cameras(cfg["seed"] + 1, nv, radius=1.5)
    vs = []
    for v in range(nv):
        u = rng.uniform(1)
        res = cfg["resolutions"][min(int(u[0] * len(cfg["resolutions"])),
                                     len(cfg["resolutions"]) - 1)]
        w, h = res
        if max_pixels and w * h > max_pixels:
            s = np.sqrt(max_pixels / (w * h))
            w, h = max(16, int(w * s)), max(16, int(h * s))
        vs.append(dict(cloud=v % nc, eye=eyes[v], target=(0.5, 0.5, 0.5), fov=60.0, width=w,
                       height=h))
    d = np.asarray(configs.SUN_DIRECTION, np.float64)
    d = tuple(float(x) for x in d / np.sqrt((d * d).sum()))
    return BatchWorkload(cfg=cfg, clouds=cl, views=vs, sun_direction=d)


@dataclass
class CompatWorkload:
    """The compat render's scene: boards as offsets from the volume position
    (CloudVolume::regenerateBillboards, CloudVolume.cpp:120-133), the sun as
    the direction from the volume toward the reference's sun position."""
    cfg: dict
    positions: np.ndarray
    scales: np.ndarray
    sun_direction: tuple
    sun_map: tuple
    cameras: list


def build_compat(cfg, boards=None, width=None, height=None):
    n = boards if boards is not None else cfg["boards"]
    rng = scene.SplitMix64(cfg["board_seed"])
    lo, hi = cfg["offset_range"]
    pos = (lo + (hi - lo) * rng.uniform(3 * n).reshape(n, 3)).astype(np.float32)
    sc = rng.uniform_range(n, *cfg["scale_range"]).astype(np.float32)
    c = np.asarray(cfg["position"], np.float64)
    d = np.asarray(cfg["sun_position"], np.float64) - c
    sun = tuple(float(x) for x in d / np.linalg.norm(d))
    cam = cfg["camera"]
    crng = scene.SplitMix64(cfg["orbit_seed"])
    m = cfg["orbits"]
    ang = 2.0 * np.pi * (np.arange(m) + crng.uniform(m)) / m
    hgt = crng.uniform_range(m, *cfg["orbit_height"])
    R = cfg["orbit_radius"]
    cams = [dict(eye=(float(c[0] + R * np.sin(a)), float(c[1] + h), float(c[2] - R * np.cos(a))),
                 target=tuple(float(x) for x in c), fov=cam["fov"],
                 width=width or cam["width"], height=height or cam["height"])
            for a, h in zip(ang, hgt)]
    return CompatWorkload(cfg=cfg, positions=pos, scales=sc, sun_direction=sun,
                          sun_map=cfg["sun_map"], cameras=cams)
