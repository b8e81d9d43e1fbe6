"""Benchmark of the render-pass path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One step = one render pass set (one frame) of the workload, submitted through the library's queue.

Workloads (seeded synthetic inputs with the configurations' shapes; no dataset exists; the scenes
and their arguments are wgpu_gb300.workloads.FULL_SIZE):
  batched (default)   256 draws into 64 render targets (sides log-uniform in [128, 2048], triangle
                      counts log-uniform in [100, 200k], random model rotations, half textured x
                      Lambert with the 1024^2 checker x value-noise texture (nearest, repeat) and
                      half vertex-colour programs), Rgba8Unorm + Depth32Float (Less), one command
                      buffer replayed from a CUDA graph with the tile shape chosen by the device's
                      autotuner (its trial submissions run before warm-up; `--fixed` or
                      `--tile/--warps` run a fixed shape without graphs).  Beside it the line
                      reports the same command buffer on the plain per-draw path (one launch
                      sequence per draw), launched directly and replayed from CUDA graphs; the
                      fill-bound configuration (`fill_bound`); and the serving loop at 2,000
                      submissions/s (`serving`).
  textured            displaced icosphere subdivided 6 times (81,920 triangles), 1024x1024
                      checker x value-noise texture, texture x Lambert, 1920x1080 Rgba8UnormSrgb +
                      Depth32Float (Less); parity profile (nearest, sRGB read and written as
                      linear, exactly as wgpu-cpu does).
  textured_filtered   the same scene as the configuration states it, extension profile: full mip
                      chain, trilinear filtering, sRGB decode and encode.
  blend               10,000 screen-aligned quads (20,000 triangles), sides U[16,1024] px, RGBA f16
                      colours with alpha U[0.1,0.9], painter order, SrcAlpha/OneMinusSrcAlpha into
                      3840x2160 Rgba16Float (extension profile).  The fill-rate-bound configuration.
  colored             UV sphere 32x16 (992 triangles), per-vertex colours, back-face cull,
                      512x512 Rgba8Unorm (the reference's CPU-runnable configuration).
  serve               the serving loop alone (Poisson arrivals, --rate, --duration).

`value` is shaded fragments per second (fragments counted as the reference counts its
fragment_processing calls) with every input resident in HBM, over the device time of the K steps
(CUDA events on the library's stream; a 256 MiB L2 flush is enqueued between steps, so each step
starts cold).  `fs_invocations_per_step` counts fragment-stage runs: the visibility raster runs
the fragment stage once per pixel, for the surviving fragment.  `parity` compares the last timed
frame of every arm with the oracle's frame (SHA-256 digests in tests/golden/frame_digests.json).
`e2e` is the same metric through the C ABI with host buffers: each step uploads the pass's inputs
from pinned host memory, renders, and reads every colour target back.  `roofline` covers the
dominant kernel (the raster kernel).  `--impl reference` times the CPU restatement of wgpu-cpu's
rasteriser (the oracle; the Rust reference cannot be built here) on all host cores, on the same
configuration.  One GPU per process; with N > 1 each rank renders its own replica and `value`
sums them.
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
TEXEL_BYTES_NEAREST = 4  # one Rgba8 texel per nearest sample


class Workload:
    def __init__(self, name, description, extra_cfg, tile, dtype="f32", texel_bytes=TEXEL_BYTES_NEAREST,
                 blend_bytes=0):
        from wgpu_gb300 import workloads as wl

        self.name = name
        self.builder, self.profile, self.kwargs = wl.FULL_SIZE[name]
        self.description, self.extra_cfg = description, extra_cfg
        self.tile = tile  # (side, warps per tile): the fastest fixed shape measured for this workload
        self.dtype = dtype
        self.texel_bytes = texel_bytes  # bytes read per texture sample
        self.blend_bytes = blend_bytes  # colour bytes read back per fragment when blending

    def build(self, dev, **over):
        from wgpu_gb300 import workloads as wl

        return wl.build_config(dev, self.name, **over)

    def config(self):
        """The workload as both arms run it (identical for --impl ours and --impl reference)."""
        return {"workload": self.description, **self.extra_cfg,
                "l2": "GPU: flushed between timed steps (256 MiB write); CPU: n/a"}


def workloads():
    return {
        "batched": Workload(
            "batched",
            "batched draws: 256 draws into 64 targets (sides log-uniform [128,2048], tris log-uniform [100,200k]), "
            "Rgba8Unorm + Depth32Float Less, half texture x Lambert (1024^2 checker x noise, nearest, repeat) / half "
            "vertex colour, one command buffer",
            {"draws": 256, "targets": 64, "texture": "1024x1024 rgba8", "profile": "parity", "seed": 3},
            tile=(32, 8)),
        "textured": Workload(
            "textured",
            "textured icosphere: 81,920 tris, 1920x1080 Rgba8UnormSrgb + Depth32Float Less, 1024^2 texture, "
            "texture x Lambert, parity profile (nearest, sRGB as linear)",
            {"triangles": 81920, "target": "1920x1080", "texture": "1024x1024 rgba8", "profile": "parity", "seed": 2},
            tile=(16, 4)),
        "textured_filtered": Workload(
            "textured_filtered",
            "textured icosphere: 81,920 tris, 1920x1080 Rgba8UnormSrgb + Depth32Float Less, 1024^2 Rgba8UnormSrgb "
            "texture with full mip chain, linear min/mag/mip filtering, repeat, texture x Lambert, extension profile",
            {"triangles": 81920, "target": "1920x1080 rgba8 srgb", "texture": "1024x1024 rgba8 srgb, 11 mips",
             "filtering": "trilinear", "profile": "extension", "seed": 2},
            tile=(16, 4), texel_bytes=32),
        "blend": Workload(
            "blend",
            "blended quads: 10,000 quads (20,000 tris) sides U[16,1024], painter order, SrcAlpha/OneMinusSrcAlpha "
            "into 3840x2160 Rgba16Float, extension profile",
            {"triangles": 20000, "target": "3840x2160 rgba16float", "profile": "extension", "seed": 4},
            tile=(32, 4), dtype="f32 (f16 storage)", texel_bytes=0, blend_bytes=8),
        "colored": Workload(
            "colored", "colored UV sphere: 992 tris, 512x512 Rgba8Unorm, back-face cull, no depth",
            {"triangles": 992, "target": "512x512", "profile": "parity", "seed": 1}, tile=(16, 8)),
    }


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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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


# ------------------------------------------------------------------------------------ byte model
def algorithmic_bytes(wk: Workload, scene, stats) -> dict:
    """Bytes the raster kernel must move at least, per launch:
      every target pixel written once (colour + depth: the clear is fused into the raster),
      per covered fragment the depth read and write (8 B) when the pass has depth,
      per fragment-stage run the colour write (plus the colour read when blending) and the texel
      bytes of a texture-sampling program (4 B nearest, 32 B trilinear Rgba8)."""
    from wgpu_gb300 import api as W
    from wgpu_gb300 import workloads as wl

    pixels, has_depth, bpp = 0, False, 4
    for color, depth in wl.scene_targets(scene):
        bpp = W.BYTES_PER_TEXEL[color.format]
        pixels += color.width * color.height * (bpp + (4 if depth is not None else 0))
        has_depth = has_depth or depth is not None
    covered = int(stats.fragments_shaded)
    fs_runs = int(stats.fs_invocations)
    tex_runs = int(stats.texture_fs_invocations)
    total = pixels + covered * (8 if has_depth else 0) + fs_runs * (bpp + wk.blend_bytes) + tex_runs * wk.texel_bytes
    return {"total": total, "target_pixels": pixels, "covered_fragments": covered, "fs_invocations": fs_runs,
            "texture_fs_invocations": tex_runs}


# ------------------------------------------------------------------------------------ parity
def parity_of(name, dev, scene, stats) -> dict:
    """The rendered frame against the oracle's (tests/golden/frame_digests.json)."""
    import frame_digests as fd

    diffs = fd.compare(name, fd.input_digest(scene), fd.target_digests(dev, scene), int(stats.fragments_shaded))
    return {"status": "ok" if not diffs else "MISMATCH", "checked": "colour + depth bytes of every target and the "
            "fragment count vs the oracle (sha256)", **({"diffs": diffs[:8]} if diffs else {})}


# ------------------------------------------------------------------------------------ CPU (oracle)
def oracle_frames(wk: Workload, threads: int, budget_s: float, max_frames: int, warmup: int = 0, passes=None):
    """Renders the workload's frame with the oracle (the CPU restatement of wgpu-cpu's rasteriser)
    on `threads` host threads: `warmup` untimed frames, then frames until `max_frames` or the time
    budget.  `passes` limits a multi-pass scene to its first passes (a bounded sample).
    Returns (fragments per frame, frames, seconds)."""
    import oracle_device
    from wgpu_gb300 import workloads as wl

    dev = oracle_device.device(profile=wk.profile, threads=threads)
    try:
        scene = wl.build_config(dev, wk.name)
        if passes is not None:
            scene.passes = scene.passes[:passes]
        enc = dev.create_command_encoder()
        scene.record(enc)
        cmd = enc.finish()
        for _ in range(warmup):
            dev.queue.submit([cmd])
        frags, frames = 0, 0
        t0 = time.perf_counter()
        while True:
            idx = dev.queue.submit([cmd])
            frags = dev.submission_stats(idx).fragments_shaded
            frames += 1
            if frames >= max_frames or time.perf_counter() - t0 > budget_s:
                break
        return frags, frames, time.perf_counter() - t0
    finally:
        dev.close()
        oracle_device.oracle_lib.load().orc_set_threads(1)


def cpu_baseline(wk: Workload, budget_s: float = 12.0, single_thread_s: float = 10.0) -> dict:
    """The oracle on the host cores, on the same workload: all cores on whole frames (bounded by
    the time budget), and one thread — the reference's single engine thread (engine.rs:15-22) —
    on a bounded sample (the first passes of the frame, or whole frames of a single-pass one)."""
    cores = os.cpu_count() or 1
    frags, frames, dt = oracle_frames(wk, cores, budget_s, 200)
    out = {"value": frags * frames / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{frames} full frames of the workload ({frags} fragments each) in {dt:.1f} s, "
                     f"{cores} threads (row bands / passes per thread)"}
    passes = 4 if wk.name == "batched" else None
    f1, n1, d1 = oracle_frames(wk, 1, single_thread_s, 50, passes=passes)
    what = f"the first {passes} of the frame's 64 passes" if passes else "full frames"
    out["single_thread"] = {"value": f1 * n1 / d1, "unit": UNIT, "cores": 1,
                            "sample": f"{n1} x {what} ({f1} fragments each) in {d1:.1f} s"}
    return out


def run_reference(args, wk: Workload):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    # whole frames of the same configuration as the GPU arm: W untimed, then K timed (at most 150 s)
    frags, frames, dt = oracle_frames(wk, cores, 150.0, args.steps, warmup=args.warmup)
    value = frags * frames / dt
    base = {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{frames} timed full frames ({frags} fragments each) after {args.warmup} untimed, "
                      f"{dt:.1f} s, {cores} threads"}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / frames, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wk.dtype, "data": "synthetic (seeded)",
            "config": wk.config(), "cpu_baseline": base, "fragments_per_step": frags,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------ GPU arms
def record(dev, scene):
    enc = dev.create_command_encoder()
    scene.record(enc)
    return enc.finish()


def timed_steps(dev, cmd, steps, flush=True):
    subs = []
    for _ in range(steps):
        if flush:
            dev.flush_caches()
        subs.append(dev.queue.submit([cmd]))
    dev.poll(True, subs[-1])
    return [dev.submission_stats(i) for i in subs]


def per_draw_arm(wk, local, shape, graphs, steps):
    """The same command buffer on the plain path: one launch sequence per draw, at `shape`."""
    from wgpu_gb300 import api as W

    dev = W.Device(device_ordinal=local, profile=wk.profile, time_kernels=True, tile_size=shape[0],
                   warps_per_tile=shape[1], launch_mode=W.LaunchMode.PER_DRAW, use_graphs=graphs)
    try:
        scene = wk.build(dev)
        cmd = record(dev, scene)
        timed_steps(dev, cmd, 3)  # warm-up (graph capture on the first)
        st = timed_steps(dev, cmd, steps)
        ms = float(np.mean([s.gpu_ms for s in st]))
        return {"value": st[-1].fragments_shaded / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "cuda_graphs": graphs,
                "gpu_launches_per_step": int(st[-1].kernel_launches), "draws": int(st[-1].draws),
                "kernels_per_draw": round(st[-1].kernel_launches / max(1, st[-1].draws), 2),
                "parity": parity_of(wk.name, dev, scene, st[-1])["status"]}
    finally:
        dev.close()


def fill_bound_arm(local, steps):
    """The fill-bound configuration (10,000 blended quads into 3840x2160 Rgba16Float)."""
    from wgpu_gb300 import api as W

    wk = workloads()["blend"]
    dev = W.Device(device_ordinal=local, profile=wk.profile, time_kernels=True, tile_size=wk.tile[0],
                   warps_per_tile=wk.tile[1])
    try:
        scene = wk.build(dev)
        cmd = record(dev, scene)
        timed_steps(dev, cmd, 3)
        st = timed_steps(dev, cmd, steps)
        ms = float(np.mean([s.gpu_ms for s in st]))
        r_ms = float(np.mean([s.raster_ms for s in st]))
        ab = algorithmic_bytes(wk, scene, st[-1])
        peak, src = measured_peak_hbm()
        achieved = ab["total"] / (r_ms / 1e3) / 1e9
        prof = raster_profile("blend")
        return {"workload": wk.description, "value": st[-1].fragments_shaded / (ms / 1e3), "unit": UNIT,
                "ms_per_step": ms, "steps": steps, "fragments_per_step": int(st[-1].fragments_shaded),
                "fs_invocations_per_step": int(st[-1].fs_invocations), "tile": f"{wk.tile[0]}x{wk.tile[1]}",
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                             "traffic": prof.get("dram_bytes_per_launch"), "peak_source": src,
                             "kernel": prof.get("kernel", "k_raster"), "kernel_ms": r_ms,
                             "algorithmic_bytes_per_launch": ab["total"], "byte_model": ab,
                             "note": "algorithmic bytes: the Rgba16Float read + write of every blended fragment; DRAM "
                                     "traffic is the target once (tiles stay in registers), so the kernel is "
                                     "instruction-bound, not HBM-bound"},
                "parity": parity_of("blend", dev, scene, st[-1])}
    finally:
        dev.close()


SERVE_TILE = (32, 8)  # tile side, warps per tile of both serving arms (--tile / --warps override)


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


def serving_arms(local, lam, duration, tile, warps):
    """The served (continuous batching, HBM-budget admission) and the per-draw arm on the same
    Poisson arrival stream of pre-recorded submissions over resident resources."""
    from wgpu_gb300 import api as W
    from wgpu_gb300 import workloads as wl

    arms = {}
    for name, kw in (("served", dict(batch_submissions=True, launch_mode=W.LaunchMode.BATCHED)),
                     ("per_draw", dict(batch_submissions=False, launch_mode=W.LaunchMode.PER_DRAW))):
        dev = W.Device(device_ordinal=local, tile_size=tile, warps_per_tile=warps, hbm_budget_bytes=80 << 30, **kw)
        try:
            sset = wl.serving_set(dev)
            for c in sset.commands[:8]:  # warm-up (allocations, first launches)
                dev.poll(True, dev.queue.submit([c]))
            with ClockSampler(local) as clocks:
                stats, wall = serve_arm(dev, sset, lam, duration, seed=11, max_submissions=int(lam * duration * 2) + 16)
            arms[name] = serve_summary(stats, wall, lam, duration)
            arms[name]["clocks"] = clocks.summary()
            del sset
        finally:
            dev.close()
    return arms


SERVE_WORKLOAD = ("serving: Poisson arrivals of submissions with 1-64 draws (log-uniform) of 512 resident meshes "
                  "(100..200k tris) and 128 textures into 256^2..1920x1080 Rgba8Unorm + Depth32Float targets, "
                  "textured Lambert / vertex colour, 80 GB HBM admission budget")


def run_ours(args, wk: Workload):
    import torch

    from wgpu_gb300 import api as W

    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = W.Device(device_ordinal=local, profile=wk.profile, time_kernels=True, tile_size=args.tile,
                   warps_per_tile=args.warps, launch_mode=LAUNCH_MODES[args.launch_mode], use_graphs=args.graphs)
    over = {}
    if args.quads and wk.name == "blend":
        over = {"n_quads": args.quads}
    if wk.name == "batched" and (args.draws or args.targets):
        over = {"n_draws": args.draws or wk.kwargs["n_draws"], "n_targets": args.targets or wk.kwargs["n_targets"]}
    scene = wk.build(dev, **over)
    cmd = record(dev, scene)

    if args.autotune:  # the tuner's trial submissions (one per candidate tile shape), before warm-up
        for _ in range(TUNE_TRIALS):
            dev.flush_caches()
            dev.poll(True, dev.queue.submit([cmd]))
    timed_steps(dev, cmd, args.warmup)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    barrier()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        stats = timed_steps(dev, cmd, args.steps)
        wall = time.perf_counter() - t0
    barrier()
    last = stats[-1]
    frags_per_step = int(last.fragments_shaded)
    parity = parity_of(wk.name, dev, scene, last) if not over else {"status": "not checked (cut workload)"}
    shape = (last.tile_shape >> 8, last.tile_shape & 0xFF)

    gpu_ms = [s.gpu_ms for s in stats]
    raster_ms = [s.raster_ms for s in stats]
    device_s, value = replica_rate(frags_per_step, args.steps, sum(gpu_ms) / 1e3)
    launches = int(sum(s.kernel_launches for s in stats))

    # roofline of the dominant kernel: algorithmic bytes per launch / its event-timed duration
    ab = algorithmic_bytes(wk, scene, last)
    peak, peak_src = measured_peak_hbm()
    r_ms = float(np.mean(raster_ms))
    achieved = ab["total"] / (r_ms / 1e3) / 1e9 if r_ms > 0 else None
    prof = raster_profile(wk.name)

    # end to end through the C ABI: inputs from pinned host memory, every colour target read back
    pinned = [(obj, torch.from_numpy(np.array(arr).reshape(-1).view(np.uint8)).pin_memory())
              for obj, arr in scene.uploads]
    from wgpu_gb300 import workloads as wl

    reads = []
    for t, _ in wl.scene_targets(scene):
        n = t.width * t.height * W.BYTES_PER_TEXEL[t.format]
        reads.append((t, torch.empty(n, dtype=torch.uint8).pin_memory()))
    out_bytes = sum(o.numel() for _, o in reads)
    buffer_writes = W.PreparedWrites([(obj, 0, host.numpy()) for obj, host in pinned if not isinstance(obj, W.Texture)])
    texture_writes = [(obj, host.numpy()) for obj, host in pinned if isinstance(obj, W.Texture)]
    # double-buffered targets, as a swapchain: frame k + 1 renders into the other set while frame
    # k's targets come back (the same host destinations, written in frame order)
    scene_b = wl.with_new_targets(scene)
    cmds = [cmd, record(dev, scene_b)]
    read_items = [[(t, 0, o.data_ptr(), o.numel()) for (t, _), (_, o) in zip(wl.scene_targets(sc), reads)]
                  for sc in (scene, scene_b)]

    def e2e_step(k):
        dev.queue.write_buffers(buffer_writes)
        for obj, host in texture_writes:
            dev.queue.write_texture(obj, host)
        dev.queue.submit([cmds[k % 2]])
        # the readback, queue-ordered after the submission, without blocking: the next frame is
        # enqueued while this one's targets come back (copy_texture_to_buffer + map_async)
        return dev.read_textures_into_async(read_items[k % 2])

    for k in range(max(2, min(args.warmup, 4))):
        dev.poll(True, e2e_step(k))
    e_steps = max(4, min(args.steps, 20))
    barrier()
    t0 = time.perf_counter()
    for k in range(e_steps):
        last_read = e2e_step(k)
    dev.poll(True, last_read)  # every frame's targets are back in host memory
    e2e_s = (time.perf_counter() - t0) / e_steps
    e2e_s, e2e_rate = replica_rate(frags_per_step, 1, e2e_s)
    h2d = sum(h.numel() for _, h in pinned)
    dev.close()
    del pinned, reads

    extras = {}
    if wk.name == "batched" and not args.no_extras:
        pd_steps = max(3, min(args.steps, 10))
        extras["per_draw_path"] = per_draw_arm(wk, local, shape, False, pd_steps)
        extras["per_draw_path_graphs"] = per_draw_arm(wk, local, shape, True, pd_steps)
        extras["fill_bound"] = fill_bound_arm(local, max(5, min(args.steps, 20)))
        arms = serving_arms(local, 2000.0, 1.0, *SERVE_TILE)
        extras["serving"] = {"workload": SERVE_WORKLOAD, "tile": f"{SERVE_TILE[0]}x{SERVE_TILE[1]}", **arms}
        extras["p99_submit_ms"] = arms["served"]["p99_ms"]

    if rank == 0:
        base = cpu_baseline(wk) if world == 1 and not args.no_cpu_baseline and not over else None
        cfg = wk.config()
        if over:
            cfg = {**cfg, "cut_for_profiling": over}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(gpu_ms)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wk.dtype, "data": "synthetic (seeded)",
            "config": cfg,
            "launch": {"launch_mode": args.launch_mode, "cuda_graphs": bool(args.graphs),
                       "tile": f"autotuned: {shape[0]}" if args.autotune else shape[0],
                       "warps_per_tile": f"autotuned: {shape[1]}" if args.autotune else shape[1]},
            "parity": parity["status"], "parity_detail": parity,
            "fragments_per_step": frags_per_step, "fs_invocations_per_step": int(last.fs_invocations),
            "texture_fs_invocations_per_step": int(last.texture_fs_invocations),
            "wall_ms_per_step": wall * 1e3 / args.steps,
            "generic_setup_prims_per_step": int(last.generic_setup_prims),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None,
                         "traffic": prof.get("dram_bytes_per_launch") if not over else None,
                         "peak_source": peak_src, "kernel": prof.get("kernel", "raster kernel (k_raster_vis or k_raster)"),
                         "algorithmic_bytes_per_launch": ab["total"], "byte_model": ab, "kernel_ms": r_ms,
                         **({"note": prof["note"]} if prof.get("note") and not over else {})},
            "cpu_baseline": base,
            "e2e": {"value": e2e_rate, "unit": UNIT, "h2d_bytes_per_step": int(h2d) * world,
                    "d2h_bytes_per_step": int(out_bytes) * world, "ms_per_step": e2e_s * 1e3,
                    "note": "per frame: inputs uploaded from pinned host memory, frame submitted, every colour "
                            "target read back to pinned host memory; frames pipelined over two target sets "
                            "(double buffering: frame k+1 renders while frame k's targets are read back), the "
                            "clock stopped when the last readback landed"},
            "gpu_launches": launches,
            "clocks": clocks.summary(),
            **extras,
        }
        if "per_draw_path" in extras:
            line["batched_vs_per_draw"] = value / extras["per_draw_path"]["value"]
            line["batched_vs_per_draw_graphs"] = value / extras["per_draw_path_graphs"]["value"]
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_serve(args):
    """The serving loop alone at --rate for --duration seconds."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    arms = serving_arms(local, args.rate, args.duration, args.tile or SERVE_TILE[0], args.warps or SERVE_TILE[1])
    s = arms["served"]
    if rank == 0:
        line = {
            "metric": METRIC, "value": s["fragments_per_s"] * world, "unit": UNIT, "n_gpus": world,
            "steps": s["submissions"], "warmup": 8, "ms_per_step": s["mean_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": SERVE_WORKLOAD, "lambda_per_s": args.rate, "hbm_budget_gb": 80,
                       "l2": "not flushed (inputs resident; a step is one submission)"},
            "launch": {"launch_mode": "batched + merged submissions", "tile": args.tile or SERVE_TILE[0],
                       "warps_per_tile": args.warps or SERVE_TILE[1]},
            "serving": s, "per_draw_path": arms["per_draw"], "p99_submit_ms": s["p99_ms"],
            "e2e": {"value": s["fragments_per_s"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "wall clock from first submit to last fence through the C ABI; inputs resident"},
            "gpu_launches": s["kernel_launches"], "clocks": s["clocks"],
        }
        print(json.dumps(line), flush=True)


LAUNCH_MODES = {"batched": 0, "per_pass": 2, "per_draw": 1}
TUNE_TRIALS = 6  # the library times five candidate tile shapes per batch shape, then keeps the fastest


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200, help="timed steps (the batched step is ~2.6 ms: 200 steps keep the clock sampler busy for ~0.5 s)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["textured", "textured_filtered", "blend", "colored", "batched", "serve"])
    ap.add_argument("--rate", type=float, default=2000.0, help="serve workload: submissions per second")
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
    ap.add_argument("--no-extras", action="store_true",
                    help="batched workload: skip the per-draw, fill-bound and serving arms (profiling runs)")
    ap.add_argument("--fixed", action="store_true",
                    help="no CUDA graph (and for the batched workload no autotuner: its fixed tile shape)")
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
        # the other workloads at their fixed tile shape, their launch sequence replayed from a
        # CUDA graph as a frame loop would (--fixed: launched directly)
        args.graphs = args.graphs or (args.impl == "ours" and not args.fixed)
    if args.workload == "serve":
        if args.impl == "reference":
            run_reference(args, workloads()["batched"])
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
