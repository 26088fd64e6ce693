"""The benchmark workloads as data: the plain small case (64^3), the plain
1080p case (256^3, noise), the precision form (512^3 BF16/FP16, 4K), the
batching form and the learned form.  Values not fixed by the workload
descriptions (density scale, ambient, cone radius floor, sun-map size,
seeds) are this build's choices and are listed here once."""

SUN_DIRECTION = (0.3, 1.0, 0.2)  # normalized by Sun()
VOLUME_POSITION = (0.5, 0.5, 0.5)  # unit cube: position +- 0.5
VOLUME_BOUNDS = (-0.5, 0.5)

SMALL_64 = dict(
    name="plain_64cube_256px",
    dim=64, mips=7, fmt="rgba32f",
    boards=64, board_seed=1, radius_range=(0.05, 0.15), radius_scale=1.0,
    density_range=(0.5, 1.0), ball_radius=0.35,
    sun_map=(1280, 720),
    camera=dict(eye=(0.5, 0.5, -1.5), target=(0.5, 0.5, 0.0), fov=60.0, width=256, height=256),
    view_steps=32, sun_steps=16, cone_half_angle=0.05, cone_h0=1.0, cone_min_radius=2.0,
    density_scale=8.0, ambient=0.3, noise_octaves=0, noise_seed=7,
    noise_frequency=4.0, noise_lacunarity=2.0, noise_gain=0.5,
)

PLAIN_1080P = dict(
    name="plain_fp32_256cube_1080p",
    dim=256, mips=8, fmt="rgba32f",
    boards=4096, board_seed=2, radius_range=(0.05, 0.15), radius_scale=0.5,
    density_range=(0.5, 1.0), ball_radius=0.35,
    sun_map=(1280, 720),
    orbit_seed=11, orbits=16, orbit_radius=1.5,
    camera=dict(fov=60.0, width=1920, height=1080),
    view_steps=64, sun_steps=24, cone_half_angle=0.03, cone_h0=1.0, cone_min_radius=2.0,
    density_scale=2.0, ambient=0.3, noise_octaves=4, noise_seed=7,
    noise_frequency=4.0, noise_lacunarity=2.0, noise_gain=0.5,
)

PRECISION_4K = dict(
    name="bf16_512cube_4k",
    dim=512, mips=9, fmt="bf16_fp16",
    boards=16384, board_seed=3, radius_range=(0.05, 0.15), radius_scale=0.5,
    density_range=(0.5, 1.0), ball_radius=0.35,
    sun_map=(1280, 720),
    orbit_seed=13, orbits=16, orbit_radius=1.5,
    camera=dict(fov=60.0, width=3840, height=2160),
    view_steps=128, sun_steps=32, cone_half_angle=0.03, cone_h0=1.0, cone_min_radius=2.0,
    density_scale=2.0, ambient=0.3, noise_octaves=5, noise_seed=7,
    noise_frequency=4.0, noise_lacunarity=2.0, noise_gain=0.5,
)

BATCH_48x128 = dict(
    name="batch_48clouds_128views",
    clouds=48, views=128, dims=(64, 96, 128, 192, 256), boards_range=(256, 4096),
    resolutions=((256, 256), (512, 512), (960, 540), (1920, 1080)),
    seed=17, radius_range=(0.05, 0.15), radius_scale=0.5,
    view_steps=64, sun_steps=24, cone_half_angle=0.03,
    autotune=dict(brick=(4, 8, 16), rays_per_warp=(1, 4, 8), unroll=(1, 2, 4)),
)

LEARNED = dict(
    name="mlp_sun_surrogate",
    features=16, hidden=64, layers=3, train_samples=4_000_000, batch=16384, steps=20000,
    lr=1e-3, eval_base="PLAIN_1080P", eval_fmt="bf16_fp16",
)

# The compat render's scene at the reference's own scale (main.cpp:29-37, :82):
# a 32^3 volume of bounds +-5 at (25, 0, 0), 4 mips, 200 boards offset
# uniformly in +-2.5 with radii in [1, 2.5], the sun at (5, 20, -5); the
# views orbit the cloud at 14 world units.
COMPAT_REF = dict(
    name="compat_reference_scene_1080p",
    dim=32, mips=4, bounds=(-5.0, 5.0), position=(25.0, 0.0, 0.0),
    boards=200, board_seed=21, offset_range=(-2.5, 2.5), scale_range=(1.0, 2.5),
    sun_position=(5.0, 20.0, -5.0), sun_map=(256, 256),
    orbit_seed=23, orbits=8, orbit_radius=14.0, orbit_height=(1.0, 6.0),
    camera=dict(fov=60.0, width=1920, height=1080),
)

ALL = dict(SMALL_64=SMALL_64, PLAIN_1080P=PLAIN_1080P, PRECISION_4K=PRECISION_4K,
           BATCH_48x128=BATCH_48x128, LEARNED=LEARNED, COMPAT_REF=COMPAT_REF)
