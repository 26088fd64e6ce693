"""Seeded scene generation: SplitMix64 stream and distributions."""
import numpy as np

from cloudgb import configs, scene, workload


def test_splitmix64_known_values():
    # SplitMix64 from seed 1234567 (Steele, Lea & Flood 2014; the published
    # reference implementation's first outputs)
    r = scene.SplitMix64(1234567)
    got = [int(x) for x in r.next_u64(5)]
    assert got == [6457827717110365317, 3203168211198807973, 9817491932198370423,
                   4593380528125082431, 16408922859458223821]


def test_stream_is_split_invariant():
    a = scene.SplitMix64(99).next_u64(10)
    r = scene.SplitMix64(99)
    b = np.concatenate([r.next_u64(3), r.next_u64(7)])
    assert np.array_equal(a, b)


def test_billboard_distributions():
    pos, rad, dens = scene.billboards(5, 4096, radius_scale=0.5)
    c = pos.astype(np.float64) + 0.5
    d = np.sqrt(((c - 0.5) ** 2).sum(axis=1))
    assert d.max() <= 0.35 + 1e-6
    assert 0.025 - 1e-7 <= rad.min() and rad.max() <= 0.075 + 1e-7
    assert 0.5 - 1e-7 <= dens.min() and dens.max() <= 1.0 + 1e-7
    # uniform in the ball: fraction within half the radius is 1/8
    assert abs((d <= 0.175).mean() - 0.125) < 0.02


def test_scene_is_deterministic():
    a = scene.billboards(3, 100)
    b = scene.billboards(3, 100)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    c = scene.billboards(4, 100)
    assert not np.array_equal(a[0], c[0])


def test_orbit_cameras():
    eyes = scene.orbit_cameras(11, 16)
    assert len(eyes) == 16
    for e in eyes:
        r = np.sqrt(((np.asarray(e) - 0.5) ** 2).sum())
        assert abs(r - 1.5) < 1e-9


def test_workload_sizes():
    wl = workload.build(configs.PLAIN_1080P)
    assert wl.positions.shape == (4096, 3)
    assert len(wl.cameras) == 16 and wl.cameras[0]["width"] == 1920
    wl1 = workload.build(configs.SMALL_64)
    assert wl1.cameras[0]["eye"] == (0.5, 0.5, -1.5)
