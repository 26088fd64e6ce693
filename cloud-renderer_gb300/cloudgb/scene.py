"""Seeded synthetic scenes: billboard lists and orbit cameras.

Replaces the reference's unseeded rand() (Util.hpp:19-45, srand(time(0)) at
main.cpp:70) with SplitMix64 (Steele, Lea & Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014).  Only IEEE basic operations are
used (rejection sampling, no transcendental functions), so a seed produces
the same scene on every host.
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)
_MASK = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.state = int(seed) & _MASK

    def next_u64(self, n):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = np.uint64(self.state) + idx * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _C1
            z = (z ^ (z >> np.uint64(27))) * _C2
            z = z ^ (z >> np.uint64(31))
        self.state = (self.state + n * int(_GOLDEN)) & _MASK
        return z

    def uniform(self, n):
        """n doubles in [0, 1) with 53 random bits each."""
        return (self.next_u64(n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)

    def uniform_range(self, n, lo, hi):
        return lo + (hi - lo) * self.uniform(n)

    def in_unit_ball(self, n):
        """n points uniform in the unit ball (rejection from the cube)."""
        out = np.empty((0, 3))
        while out.shape[0] < n:
            c = self.uniform(3 * 64).reshape(64, 3) * 2.0 - 1.0
            keep = (c * c).sum(axis=1) <= 1.0
            out = np.concatenate([out, c[keep]], axis=0)
        return out[:n]

    def on_unit_sphere(self, n):
        out = np.empty((0, 3))
        while out.shape[0] < n:
            c = self.uniform(3 * 64).reshape(64, 3) * 2.0 - 1.0
            r2 = (c * c).sum(axis=1)
            keep = (r2 <= 1.0) & (r2 > 1e-4)
            c = c[keep] / np.sqrt(r2[keep])[:, None]
            out = np.concatenate([out, c], axis=0)
        return out[:n]


def billboards(seed, count, center=(0.5, 0.5, 0.5), ball_radius=0.35,
               radius_range=(0.05, 0.15), radius_scale=1.0, density_range=(0.5, 1.0),
               volume_position=(0.5, 0.5, 0.5)):
    """Board positions (relative to the volume position), radii and densities.

    Centres uniform in a ball about `center`, radii uniform in radius_range
    times radius_scale, densities uniform in density_range."""
    rng = SplitMix64(seed)
    c = np.asarray(center, np.float64) + ball_radius * rng.in_unit_ball(count)
    r = rng.uniform_range(count, radius_range[0], radius_range[1]) * radius_scale
    d = rng.uniform_range(count, density_range[0], density_range[1])
    pos = (c - np.asarray(volume_position, np.float64)).astype(np.float32)
    return pos, r.astype(np.float32), d.astype(np.float32)


def orbit_cameras(seed, count, radius=1.5, center=(0.5, 0.5, 0.5), max_abs_y=0.95):
    """Eyes on a sphere about `center`, each looking at it with up = +y."""
    rng = SplitMix64(seed)
    eyes = []
    while len(eyes) < count:
        u = rng.on_unit_sphere(1)[0]
        if abs(u[1]) > max_abs_y:
            continue
        eyes.append(np.asarray(center) + radius * u)
    return [tuple(float(x) for x in e) for e in eyes]


def sun_direction(x=0.3, y=1.0, z=0.2):
    v = np.array([x, y, z], np.float64)
    return tuple(float(a) for a in (v / np.sqrt((v * v).sum())).astype(np.float32))
