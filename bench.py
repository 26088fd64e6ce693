"""Benchmark: Mpix/s of the cloud path at 1080p over a 256^3 volume.

One step = one frame = voxelize (clear, sun-view map, highlights, coverage
splat, mips) + render of one 1920x1080 view, cycling through the 16 seeded
orbit cameras.  `value` is device-resident throughput (boards already in
HBM); `e2e` goes through the public C ABI with host buffers (board upload
and image download inside the timed region).  Multi-GPU runs are
independent replicas (the path has no exchange step): value = pixels of all
ranks / max-over-ranks time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cloud-renderer_gb300")
for p in (PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "Mpix/s 1080p @256³ volume: plain FP32 vs BF16+MLP surrogate at RMSE≤1e-2"
UNIT = "Mpix/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fmt", choices=["rgba32f", "bf16_fp16"], default="rgba32f")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget-s", type=float, default=15.0)
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload():
    from cloudgb import configs, workload as W
    return W.build(configs.PLAIN_1080P)


def config_block(wl, fmt, extra=None):
    c = wl.cfg
    d = {"workload": "plain 1080p cloud frame: 256^3 volume, 4096 billboards, 4-octave fBm, "
                     "64 view steps, 24-step sun cone, 16 orbit views",
         "volume": f"{c['dim']}^3 {fmt}, {c['mips']} mips", "boards": c["boards"],
         "image": f"{c['camera']['width']}x{c['camera']['height']}",
         "view_steps": c["view_steps"], "sun_steps": c["sun_steps"],
         "cone_half_angle": c["cone_half_angle"], "noise_octaves": c["noise_octaves"],
         "sun_map": f"{c['sun_map'][0]}x{c['sun_map'][1]}", "views": c["orbits"],
         "l2": "256 MiB buffer written between timed steps (L2 flush)",
         "parallelism": "replicas"}
    if extra:
        d.update(extra)
    return d


# ---------------------------------------------------------------------------
# CPU legs (the oracle's FP32 build: the reference's CPU restatement)
# ---------------------------------------------------------------------------
def cpu_frame_rate(wl, budget_s, threads):
    """FP32 port on `threads` host cores: voxelize the full scene, then render
    whole rows of view 0 (centre outward) until the time budget is spent.
    Returns (Mpix/s, description)."""
    from oracle import oracle as O
    from cloudgb import configs, workload as Wm
    import numpy as np
    c = wl.cfg
    ov = O.OracleVolume(c["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, c["mips"], bits=32)
    ov.set_boards(wl.positions, wl.scales, wl.densities)
    t0 = time.perf_counter()
    ov.voxelize(wl.sun_direction, *wl.sun_map, threads=threads)
    t_vox = time.perf_counter() - t0

    class Cam:
        pass
    cam = Cam()
    cd = wl.cameras[0]
    cam.eye, cam.target, cam.up = cd["eye"], cd["target"], (0.0, 1.0, 0.0)
    cam.fov_y_degrees, cam.width, cam.height = cd["fov"], cd["width"], cd["height"]
    P = O.make_params(view_steps=c["view_steps"], sun_steps=c["sun_steps"],
                      cone_half_angle=c["cone_half_angle"], cone_initial_height=c["cone_h0"],
                      cone_min_radius=c["cone_min_radius"], density_scale=c["density_scale"],
                      ambient=c["ambient"], noise_octaves=c["noise_octaves"],
                      noise_seed=c["noise_seed"], noise_frequency=c["noise_frequency"],
                      noise_lacunarity=c["noise_lacunarity"], noise_gain=c["noise_gain"])
    W, H = cam.width, cam.height
    band = 8
    order = []
    mid = H // 2
    for k in range(0, H // band + 1):
        for y0 in (mid + k * band, mid - (k + 1) * band):
            if 0 <= y0 < H and y0 not in order:
                order.append(y0)
    rows = 0
    t_render = 0.0
    for y0 in order:
        h = min(band, H - y0)
        t0 = time.perf_counter()
        ov.render(cam, P, wl.sun_direction, rect=(0, y0, W, h), threads=threads)
        t_render += time.perf_counter() - t0
        rows += h
        if t_render + t_vox >= budget_s:
            break
    px = rows * W
    frame_s = t_vox + t_render * (W * H) / px
    desc = (f"FP32 port of the path on {threads} host threads: full 256^3 voxelize "
            f"({t_vox:.2f} s) + {rows} of {H} rows of view 0 ({px} px, {t_render:.2f} s), "
            f"frame time extrapolated per pixel")
    return (W * H) / frame_s / 1e6, desc, frame_s


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = workload()
    threads = os.cpu_count() or 1
    budget = max(2.0, args.cpu_budget_s)
    rates = []
    desc = ""
    for _ in range(max(0, args.warmup)):
        pass  # the CPU port has no warm-up state beyond the first call
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        r, desc, _ = cpu_frame_rate(wl, budget / max(1, args.steps) + 1.0, threads)
        rates.append(r)
    wall = time.perf_counter() - t0
    value = sorted(rates)[len(rates) // 2]
    ms = (wl.cfg["camera"]["width"] * wl.cfg["camera"]["height"]) / (value * 1e6) * 1e3
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64 scene)", "impl": "reference",
            "config": config_block(wl, "rgba32f", {"cpu_wall_s": round(wall, 2)}),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads,
                             "kind": "port", "sample": desc},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(key):
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(key)
    except Exception:
        return None


def run_ours(args):
    import numpy as np
    import torch

    import cloudgb
    from cloudgb import _lib, workload as Wm

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = workload()
    c = wl.cfg
    fmt = cloudgb.FORMAT_RGBA32F if args.fmt == "rgba32f" else cloudgb.FORMAT_BF16_FP16
    ctx = cloudgb.Context(local)
    from cloudgb import configs
    vol = cloudgb.CloudVolume(c["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, c["mips"],
                              fmt=fmt, ctx=ctx)
    vol.set_billboards(wl.positions, wl.scales, wl.densities)
    vol.update()
    sun = cloudgb.Sun(wl.sun_direction, *wl.sun_map)
    csun = sun._c()
    shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
    params = shader.params()
    cams = [Wm.make_camera(cd) for cd in wl.cameras]
    ccams = [cm._c() for cm in cams]
    W, H = cams[0].width, cams[0].height
    lib = _lib.load()

    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    img = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def frame(k):
        _lib.check(lib.cg_voxelize(vol.handle, ctypes.byref(csun), sp), "cg_voxelize")
        ev_mid = torch.cuda.Event(enable_timing=True)
        ev_mid.record(stream)
        _lib.check(lib.cg_render(ctx.handle, vol.handle, ctypes.byref(ccams[k % len(ccams)]),
                                 ctypes.byref(params), ctypes.c_void_p(img.data_ptr()), 1, sp),
                   "cg_render")
        return ev_mid

    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            frame(k)
        stream.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        launches0 = ctx.launch_count
        gpu_index = local
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        if vis:
            try:
                gpu_index = int(vis.split(",")[local])
            except ValueError:
                pass
        ev = []
        with ClockSampler(gpu_index) as clocks:
            for k in range(args.steps):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e2 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                e1 = frame(k)
                e2.record(stream)
                ev.append((e0, e1, e2))
            stream.synchronize()
        torch.cuda.synchronize()
        launches = ctx.launch_count - launches0
    step_ms = [a.elapsed_time(b) for a, _, b in ev]
    vox_ms = [a.elapsed_time(m) for a, m, _ in ev]
    trace_ms = [m.elapsed_time(b) for _, m, b in ev]
    total_ms = float(sum(step_ms))
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    pixels = W * H * args.steps * world
    value = pixels / (total_ms / 1e3) / 1e6

    # executed-work counters of the timed views (untimed) -> algorithmic bytes
    bpv = 16 if fmt == cloudgb.FORMAT_RGBA32F else 4
    used = sorted({k % len(cams) for k in range(args.steps)})
    per_view = {}
    for v in used:
        per_view[v] = shader.renderStats(vol, cams[v])
    alg_bytes = [(per_view[k % len(cams)]["view_samples"] + per_view[k % len(cams)]["sun_samples"])
                 * bpv + W * H * 16 for k in range(args.steps)]
    achieved = float(np.sum(alg_bytes)) / (float(np.sum(trace_ms)) / 1e3) / 1e9
    peak, peak_kind = load_peak()
    traffic = load_traffic(f"trace_fused_{args.fmt}")

    # e2e through the public API: host boards in, host image out
    out = cloudgb.HostBuffer((H, W, 4))
    e2e_ms = []
    for k in range(max(2, min(args.steps, 16)) + 1):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vol.update()
        cloudgb.VoxelizeShader().voxelize(vol, sun)
        shader.coneTrace(vol, cams[k % len(cams)], out=out)
        t1 = time.perf_counter()
        if k > 0:
            e2e_ms.append((t1 - t0) * 1e3)
    e2e_val = W * H / (float(np.median(e2e_ms)) / 1e3) / 1e6 * world
    h2d = vol.count * 45
    d2h = W * H * 16

    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if bpv == 16 else "bf16",
            "data": "synthetic (seeded SplitMix64 scene)",
            "config": config_block(wl, args.fmt, {
                "path": "plain FP32 exact sun cone" if bpv == 16 else "BF16/FP16 volume, exact cone",
                "voxelize_ms": round(float(np.mean(vox_ms)), 4),
                "trace_ms": round(float(np.mean(trace_ms)), 4)}),
            "roofline": {"bound": "hbm", "kernel": "k_trace_fused", "achieved": round(achieved, 1),
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "alg_bytes_per_launch": int(np.mean(alg_bytes))},
            "gpu_launches": int(launches),
            "clocks": clocks.summary(),
            "e2e": {"value": round(e2e_val, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h}}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r, desc, _ = cpu_frame_rate(wl, args.cpu_budget_s, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": round(r, 4), "unit": UNIT, "cores": os.cpu_count(),
                                "kind": "port", "sample": desc}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
