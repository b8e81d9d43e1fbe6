"""Benchmark of the render-pass path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One step = one render pass (one frame) of the workload, submitted through the library's queue.

Workloads (seeded synthetic inputs with the configurations' shapes; no dataset exists):
  textured            displaced icosphere subdivided 6 times (81,920 triangles; f32x3 position,
                      f32x3 normal, f32x2 UV), 1024x1024 Rgba8UnormSrgb checker x value-noise
                      texture, texture x Lambert shading, 1920x1080 Rgba8UnormSrgb + Depth32Float
                      (Less).  Parity profile: nearest sampling, sRGB formats read and written as
                      linear, exactly as wgpu-cpu does (its sampler ignores filter modes).
  textured_filtered   the same textured scene as the configuration states it, extension profile:
                      full mip chain, linear min/mag/mip filtering with repeat addressing, sRGB
                      texture decode and sRGB target encode (LOD per primitive from analytic UV
                      derivatives; the reference has no filtering, mips or sRGB conversion).
  blend               10,000 screen-aligned quads (20,000 triangles), sides U[16,1024] px, RGBA f16
                      colours with alpha U[0.1,0.9], painter order, SrcAlpha/OneMinusSrcAlpha into
                      3840x2160 Rgba16Float (extension profile: the reference has neither blending
                      nor f16 targets).  The fill-rate-bound configuration.
  colored             UV sphere 32x16 (992 triangles), per-vertex colours, back-face cull,
                      512x512 Rgba8Unorm (the reference's CPU-runnable configuration).
  batched (default)   256 draws into 64 render targets (sides log-uniform in [128, 2048], triangle
                      counts log-uniform in [100, 200k], random model rotations, half textured x
                      Lambert and half vertex-colour programs), Rgba8Unorm + Depth32Float (Less),
                      one command buffer, replayed from a CUDA graph with the tile shape chosen by
                      the device's autotuner (its trial submissions run before warm-up; `--fixed`
                      or `--tile/--warps` run a fixed shape without graphs).  Besides the batched
                      launch sequence the line reports the same command buffer launched per draw,
                      the plain path it replaces, at the same tile shape.

`value` is shaded fragments per second (fragment-shader invocations, counted as the reference
counts them) with every input resident in HBM, over the device time of the K steps (CUDA events on
the library's stream; a 256 MiB L2 flush is enqueued between steps, so each step starts cold).
`e2e` is the same metric through the C ABI with host buffers: each step uploads the pass's inputs
from pinned host memory, renders, and reads the colour target back.  `roofline` covers the
dominant kernel (k_raster).  `--impl reference` times the CPU restatement of wgpu-cpu's rasteriser
(the oracle; the Rust reference cannot be built here) on all host cores.  One GPU per process;
with N > 1 each rank renders its own replica and `value` sums them.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "wgpu-cpu_gb300"), os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

METRIC = "shaded fragments/s, batched vs per-draw GPU at bit-exact coverage; p99 submit ms"
UNIT = "fragments/s"


class Workload:
    def __init__(self, name, profile, builder, kwargs, bytes_per_fragment, pixel_bytes, description, extra_cfg,
                 cpu_kwargs=None, dtype="f32", tile=(16, 8)):
        self.name, self.profile, self.builder, self.kwargs = name, profile, builder, kwargs
        self.tile = tile  # (side, warps per tile): the fastest shape measured for this workload
        self.bytes_per_fragment, self.pixel_bytes = bytes_per_fragment, pixel_bytes
        self.description, self.extra_cfg = description, extra_cfg
        self.cpu_kwargs = cpu_kwargs if cpu_kwargs is not None else kwargs
        self.dtype = dtype

    def build(self, dev, **over):
        from wgpu_gb300 import workloads as wl

        return getattr(wl, self.builder)(dev, **{**self.kwargs, **over})

    def config(self, flush=True, launch_mode="batched", graphs=False):
        return {"workload": self.description, **self.extra_cfg, "launch_mode": launch_mode, "cuda_graphs": graphs,
                "l2": "flushed between timed steps (256 MiB write)" if flush else "n/a (CPU)"}


def workloads():
    from wgpu_gb300 import api as W

    return {
        "textured": Workload(
            "textured", W.Profile.PARITY, "scene_textured_icosphere",
            dict(width=1920, height=1080, level=6, tex_size=1024),
            4 + 4 + 4 + 4, 1920 * 1080 * (4 + 4),
            "textured icosphere: 81,920 tris, 1920x1080 Rgba8UnormSrgb + Depth32Float Less, 1024^2 texture, "
            "texture x Lambert, parity profile (nearest, sRGB as linear)",
            {"triangles": 81920, "target": "1920x1080", "texture": "1024x1024 rgba8", "profile": "parity", "seed": 2},
            tile=(16, 4)),
        "textured_filtered": Workload(
            "textured_filtered", W.Profile.EXTENSION, "scene_textured_icosphere",
            dict(width=1920, height=1080, level=6, tex_size=1024, filtering=True, srgb=True),
            4 + 4 + 4 + 32, 1920 * 1080 * (4 + 4),
            "textured icosphere: 81,920 tris, 1920x1080 Rgba8UnormSrgb + Depth32Float Less, 1024^2 Rgba8UnormSrgb "
            "texture with full mip chain, linear min/mag/mip filtering, repeat, texture x Lambert, extension profile",
            {"triangles": 81920, "target": "1920x1080 rgba8 srgb", "texture": "1024x1024 rgba8 srgb, 11 mips",
             "filtering": "trilinear", "profile": "extension", "seed": 2},
            tile=(16, 4)),
        "blend": Workload(
            "blend", W.Profile.EXTENSION, "scene_blended_quads", dict(width=3840, height=2160, n_quads=10000),
            8 + 8, 3840 * 2160 * 8,
            "blended quads: 10,000 quads (20,000 tris) sides U[16,1024], painter order, SrcAlpha/OneMinusSrcAlpha "
            "into 3840x2160 Rgba16Float, extension profile",
            {"triangles": 20000, "target": "3840x2160 rgba16float", "profile": "extension", "seed": 4},
            cpu_kwargs=dict(width=3840, height=2160, n_quads=60), dtype="f32 (f16 storage)", tile=(32, 8)),
        "colored": Workload(
            "colored", W.Profile.PARITY, "scene_colored_sphere", dict(width=512, height=512),
            4, 512 * 512 * 4,
            "colored UV sphere: 992 tris, 512x512 Rgba8Unorm, back-face cull, no depth",
            {"triangles": 992, "target": "512x512", "profile": "parity", "seed": 1}),
        "batched": Workload(
            "batched", W.Profile.PARITY, "scene_batched", dict(n_targets=64, n_draws=256, seed=3),
            4 + 4 + 4 + 4, None,
            "batched draws: 256 draws into 64 targets (sides log-uniform [128,2048], tris log-uniform [100,200k]), "
            "Rgba8Unorm + Depth32Float Less, half texture x Lambert / half vertex colour, one command buffer",
            {"draws": 256, "targets": 64, "profile": "parity", "seed": 3},
            cpu_kwargs=dict(n_targets=16, n_draws=64, seed=3), tile=(32, 8)),
    }


def pixel_bytes(wk: Workload, scene) -> int:
    """Target bytes written per step: colour plus depth of every target."""
    from wgpu_gb300 import api as W

    if wk.pixel_bytes is not None:
        return wk.pixel_bytes
    total = 0
    for color, depth, _ in scene.passes:
        total += color.width * color.height * (W.BYTES_PER_TEXEL[color.format] + (4 if depth is not None else 0))
    return total


def color_targets(scene):
    return [p[0] for p in scene.passes] if hasattr(scene, "passes") else [scene.color]


LAUNCH_MODES = {"batched": 0, "per_pass": 2, "per_draw": 1}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_rate(units_per_step: float, steps: int, device_s: float) -> tuple[float, float]:
    """Replicas only: every rank renders its own copy of the workload (no data-path collective);
    the job's time is the slowest rank's and its rate is all ranks' units over that time.
    Returns (max device seconds over ranks, whole-job units per second)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    if world > 1:
        t = torch.tensor([device_s], dtype=torch.float64)
        if dist.get_backend() == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        device_s = float(t.item())
    return device_s, units_per_step * steps * world / device_s


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu, self.proc, self.lines = gpu_index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def raster_profile(name):
    """The committed ncu summary of this workload's raster kernel ({} when there is none)."""
    p = os.path.join(ROOT, "profiles", f"raster_{name}.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except (OSError, ValueError):
            return {}
    return {}


def raster_traffic(name):
    """DRAM bytes per raster launch from the committed ncu summary of this workload, if any."""
    return raster_profile(name).get("dram_bytes_per_launch")


def cpu_baseline(wk: Workload, target_seconds: float = 12.0):
    """The oracle (CPU restatement of wgpu-cpu's rasteriser) on all host cores, bounded sample."""
    import oracle_device

    cores = os.cpu_count() or 1
    dev = oracle_device.device(profile=wk.profile, threads=cores)
    scene = getattr(__import__("wgpu_gb300.workloads", fromlist=["x"]), wk.builder)(dev, **wk.cpu_kwargs)
    frags, frames = 0, 0
    t0 = time.perf_counter()
    while True:
        idx = scene.render()
        frags += dev.submission_stats(idx).fragments_shaded
        frames += 1
        if time.perf_counter() - t0 > target_seconds or frames >= 200:
            break
    dt = time.perf_counter() - t0
    oracle_device.oracle_lib.load().orc_set_threads(1)
    what = "full frames of the workload" if wk.cpu_kwargs == wk.kwargs else f"frames of the workload cut to {wk.cpu_kwargs}"
    return {"value": frags / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{frames} {what} ({frags // frames} fragments each) in {dt:.1f} s, row bands per thread"}


def run_reference(args, wk: Workload):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    base = cpu_baseline(wk, target_seconds=max(5.0, min(60.0, 2.0 * args.steps)))
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": wk.dtype, "data": "synthetic (seeded)", "config": wk.config(False),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, wk: Workload):
    import torch

    from wgpu_gb300 import api as W

    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = W.Device(device_ordinal=local, profile=wk.profile, time_kernels=True, tile_size=args.tile,
                   warps_per_tile=args.warps, launch_mode=LAUNCH_MODES[args.launch_mode], use_graphs=args.graphs)
    over = {"n_quads": args.quads} if args.quads and wk.name == "blend" else {}
    if wk.name == "batched" and (args.draws or args.targets):
        over = {"n_draws": args.draws or wk.kwargs["n_draws"], "n_targets": args.targets or wk.kwargs["n_targets"]}
    scene = wk.build(dev, **over)
    enc = dev.create_command_encoder()
    scene.record(enc)
    cmd = enc.finish()

    if args.autotune:  # the tuner's trial submissions (one per candidate tile shape), before warm-up
        for _ in range(TUNE_TRIALS):
            dev.flush_caches()
            dev.poll(True, dev.queue.submit([cmd]))
    for _ in range(args.warmup):
        dev.flush_caches()
        idx = dev.queue.submit([cmd])
    dev.poll(True, idx)
    frags_per_step = dev.submission_stats(idx).fragments_shaded

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed_steps(d, c, steps):
        subs = []
        for _ in range(steps):
            d.flush_caches()
            subs.append(d.queue.submit([c]))
        d.poll(True, subs[-1])
        return [d.submission_stats(i) for i in subs]

    barrier()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        stats = timed_steps(dev, cmd, args.steps)
        wall = time.perf_counter() - t0
    barrier()

    # the same command buffer on the plain per-draw path (one launch sequence per draw)
    per_draw = None
    if wk.name == "batched" and args.launch_mode != "per_draw" and not args.no_per_draw:
        shape = stats[-1].tile_shape  # the batched arm's tile shape (the tuner's choice when autotuned)
        d2 = W.Device(device_ordinal=local, profile=wk.profile, time_kernels=True,
                      tile_size=(shape >> 8) or dev_tile(args), warps_per_tile=(shape & 0xFF) or dev_warps(args),
                      launch_mode=W.LaunchMode.PER_DRAW)
        scene2 = wk.build(d2, **over)
        enc2 = d2.create_command_encoder()
        scene2.record(enc2)
        cmd2 = enc2.finish()
        timed_steps(d2, cmd2, 3)
        st2 = timed_steps(d2, cmd2, max(3, min(args.steps, 10)))
        ms2 = float(np.mean([s.gpu_ms for s in st2]))
        if st2[-1].fragments_shaded != frags_per_step:
            raise RuntimeError("per-draw launches shaded a different number of fragments")
        per_draw = {"value": st2[-1].fragments_shaded / (ms2 / 1e3), "unit": UNIT, "ms_per_step": ms2,
                    "gpu_launches_per_step": int(st2[-1].kernel_launches)}
        del scene2, cmd2
        d2.close()
    gpu_ms = [s.gpu_ms for s in stats]
    raster_ms = [s.raster_ms for s in stats]
    device_s = sum(gpu_ms) / 1e3
    device_s, value = replica_rate(frags_per_step, args.steps, device_s)
    launches = int(sum(s.kernel_launches for s in stats))

    # roofline of the dominant kernel: algorithmic bytes per launch / its event-timed duration
    alg_bytes = pixel_bytes(wk, scene) + frags_per_step * wk.bytes_per_fragment
    peak, peak_src = measured_peak_hbm()
    r_ms = float(np.mean(raster_ms))
    achieved = alg_bytes / (r_ms / 1e3) / 1e9 if r_ms > 0 else None

    # end to end through the C ABI: inputs from pinned host memory, colour target read back
    pinned = [(obj, torch.from_numpy(np.array(arr).reshape(-1).view(np.uint8)).pin_memory())
              for obj, arr in scene.uploads]
    reads = []
    for t in color_targets(scene):
        n = t.width * t.height * W.BYTES_PER_TEXEL[t.format]
        reads.append((t, torch.empty(n, dtype=torch.uint8).pin_memory()))
    out_bytes = sum(o.numel() for _, o in reads)

    # the buffer uploads as one prepared batch (gbr_queue_write_buffers), textures one by one; the
    # read is queue-ordered after the submission (it waits for it)
    buffer_writes = W.PreparedWrites([(obj, 0, host.numpy()) for obj, host in pinned if not isinstance(obj, W.Texture)])
    texture_writes = [(obj, host.numpy()) for obj, host in pinned if isinstance(obj, W.Texture)]
    read_items = [(t, 0, o.data_ptr(), o.numel()) for t, o in reads]

    def e2e_step():
        dev.queue.write_buffers(buffer_writes)
        for obj, host in texture_writes:
            dev.queue.write_texture(obj, host)
        dev.queue.submit([cmd])
        dev.read_textures_into(read_items)

    for _ in range(max(1, min(args.warmup, 3))):
        e2e_step()
    e_steps = max(3, min(args.steps, 20))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e_steps
    # replicas: the slowest rank's time per step, every rank's fragments
    e2e_s, e2e_rate = replica_rate(frags_per_step, 1, e2e_s)
    h2d = sum(h.numel() for _, h in pinned)

    if rank == 0:
        base = cpu_baseline(wk) if world == 1 and not args.no_cpu_baseline else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(gpu_ms)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wk.dtype, "data": "synthetic (seeded)",
            "config": {**wk.config(launch_mode=args.launch_mode, graphs=args.graphs),
                       "tile": dev_tile(args) if not args.autotune else f"autotuned: {stats[-1].tile_shape >> 8}",
                       "warps_per_tile": dev_warps(args) if not args.autotune else f"autotuned: {stats[-1].tile_shape & 0xFF}",
                       **over},
            "fragments_per_step": frags_per_step, "wall_ms_per_step": wall * 1e3 / args.steps,
            "generic_setup_prims_per_step": int(stats[-1].generic_setup_prims),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None, "traffic": raster_traffic(wk.name) if not over else None,
                         "peak_source": peak_src, "kernel": raster_profile(wk.name).get("kernel", "raster kernel (k_raster_vis or k_raster)"),
                         "algorithmic_bytes_per_launch": alg_bytes, "kernel_ms": r_ms},
            "cpu_baseline": base,
            "e2e": {"value": e2e_rate, "unit": UNIT, "h2d_bytes_per_step": int(h2d) * world,
                    "d2h_bytes_per_step": int(out_bytes) * world, "ms_per_step": e2e_s * 1e3},
            "gpu_launches": launches,
            "clocks": clocks.summary(),
        }
        if per_draw is not None:
            line["per_draw_path"] = per_draw
        print(json.dumps(line), flush=True)
    dev.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def serve_arm(dev, sset, lam, duration, seed, max_submissions):
    """Poisson arrivals at `lam`/s for `duration` s (at most max_submissions), cycling through the
    pre-recorded submissions; waits for the last one.  Returns per-submission stats and the wall
    time from the first submit to the last fence."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / lam, size=max_submissions)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < duration]
    subs = []
    t0 = time.perf_counter()
    for k, ta in enumerate(arrivals):
        while True:
            now = time.perf_counter() - t0
            if now >= ta:
                break
            if ta - now > 0.0005:
                time.sleep(min(ta - now - 0.0003, 0.002))
        subs.append(dev.queue.submit([sset.commands[k % len(sset.commands)]]))
    dev.poll(True, subs[-1])
    wall = time.perf_counter() - t0
    return [dev.submission_stats(i) for i in subs], wall


def serve_summary(stats, wall, lam, duration):
    lat = np.array([s.submit_to_fence_ms for s in stats])
    frags = int(sum(s.fragments_shaded for s in stats))
    return {"lambda_per_s": lam, "arrival_window_s": duration, "submissions": len(stats),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "frames_per_s": len(stats) / wall, "fragments_per_s": frags / wall,
            "fragments": frags, "wall_s": wall, "mean_batched_with": float(np.mean([s.batched_with for s in stats])),
            "kernel_launches": int(sum(s.kernel_launches / max(1, s.batched_with) for s in stats))}


SERVE_TILE = (32, 8)  # tile side, warps per tile of both serving arms (--tile / --warps override)


def run_serve(args):
    """Serving loop: Poisson arrivals of pre-recorded submissions over resident meshes, textures and
    targets; the batched server (continuous batching, HBM-budget admission) and, on the same
    arrival stream, the plain per-draw path."""
    import torch

    from wgpu_gb300 import api as W
    from wgpu_gb300 import workloads as wl

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    lam, duration = args.rate, args.duration
    arms = {}
    for name, kw in (("served", dict(batch_submissions=True, launch_mode=W.LaunchMode.BATCHED)),
                     ("per_draw", dict(batch_submissions=False, launch_mode=W.LaunchMode.PER_DRAW))):
        dev = W.Device(device_ordinal=local, tile_size=args.tile or SERVE_TILE[0], warps_per_tile=args.warps or SERVE_TILE[1],
                       hbm_budget_bytes=80 << 30, **kw)
        sset = wl.serving_set(dev)
        for c in sset.commands[:8]:  # warm-up (allocations, first launches)
            dev.poll(True, dev.queue.submit([c]))
        with ClockSampler(local) as clocks:
            stats, wall = serve_arm(dev, sset, lam, duration, seed=11, max_submissions=int(lam * duration * 2) + 16)
        arms[name] = serve_summary(stats, wall, lam, duration)
        arms[name]["clocks"] = clocks.summary()
        dev.close()
        del sset
    s = arms["served"]
    if rank == 0:
        line = {
            "metric": METRIC, "value": s["fragments_per_s"] * world, "unit": UNIT, "n_gpus": world,
            "steps": s["submissions"], "warmup": 8, "ms_per_step": s["mean_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "serving: Poisson arrivals of submissions with 1-64 draws (log-uniform) of 512 "
                                   "resident meshes (100..200k tris) and 128 textures into 256^2..1920x1080 "
                                   "Rgba8Unorm + Depth32Float targets, textured Lambert / vertex colour",
                       "lambda_per_s": lam, "hbm_budget_gb": 80, "launch_mode": "batched + merged submissions",
                       "tile": args.tile or SERVE_TILE[0], "warps_per_tile": args.warps or SERVE_TILE[1],
                       "l2": "not flushed (inputs resident; a step is one submission)"},
            "serving": s, "per_draw_path": arms["per_draw"],
            "e2e": {"value": s["fragments_per_s"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "wall clock from first submit to last fence through the C ABI; inputs resident"},
            "gpu_launches": s["kernel_launches"], "clocks": s["clocks"],
        }
        print(json.dumps(line), flush=True)


TUNE_TRIALS = 6  # the library times five candidate tile shapes per batch shape, then keeps the fastest


def dev_tile(args):
    return args.tile or 16


def dev_warps(args):
    return args.warps or (2 if dev_tile(args) == 8 else 8)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["textured", "textured_filtered", "blend", "colored", "batched", "serve"])
    ap.add_argument("--rate", type=float, default=1000.0, help="serve workload: submissions per second")
    ap.add_argument("--duration", type=float, default=2.0, help="serve workload: arrival window in seconds")
    ap.add_argument("--launch-mode", default="batched", choices=list(LAUNCH_MODES))
    ap.add_argument("--graphs", action="store_true", help="replay each submission's launches from a CUDA graph")
    ap.add_argument("--autotune", action="store_true", help="let the device time tile shapes (tile/warps ignored)")
    ap.add_argument("--quads", type=int, default=0, help="blend workload: number of quads (profiling runs)")
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--warps", type=int, default=0)
    ap.add_argument("--draws", type=int, default=0, help="batched workload: number of draws (profiling runs)")
    ap.add_argument("--targets", type=int, default=0, help="batched workload: number of targets (profiling runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-per-draw", action="store_true", help="batched workload: skip the per-draw comparison")
    ap.add_argument("--fixed", action="store_true",
                    help="batched workload: no CUDA graph and no autotuner (the workload's fixed tile shape)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.workload == "batched" and not args.fixed and not args.tile and args.impl == "ours":
        # the configuration as specified: one launch sequence captured in a CUDA graph, tile shape
        # and warps per tile chosen by the device's autotuner (its trials run before warm-up)
        args.autotune = args.graphs = True
    if args.autotune:
        args.tile = args.warps = 0
    elif not args.tile and args.workload in workloads():
        args.tile, args.warps = workloads()[args.workload].tile
    elif not args.tile:
        args.tile, args.warps = dev_tile(args), dev_warps(args)
    if args.workload == "serve":
        if args.impl == "reference":
            wk = workloads()["batched"]
            run_reference(args, wk)
        else:
            run_serve(args)
        return
    wk = workloads()[args.workload]
    if args.impl == "reference":
        run_reference(args, wk)
    else:
        run_ours(args, wk)


if __name__ == "__main__":
    main()
