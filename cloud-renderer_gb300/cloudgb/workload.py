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
