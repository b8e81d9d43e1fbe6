"""Benchmark of the render-pass path on the textured-mesh workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step = one render pass = one frame): displaced icosphere subdivided 6 times
(81,920 triangles, f32x3 position + f32x3 normal + f32x2 UV), a 1024x1024 Rgba8UnormSrgb
checker x value-noise texture, texture x Lambert fragment shader, 1920x1080 Rgba8UnormSrgb +
Depth32Float (Less), cleared every frame.  Parity profile: nearest sampling with sRGB formats
read and written as linear, exactly as wgpu-cpu does (its sampler ignores filter modes and it
stores mip 0 only).  Inputs are seeded synthetic data.

`value` is shaded fragments per second with every input resident in HBM, timed with CUDA events
on the library's stream (each step's device time; an L2 flush between steps keeps every step
cold because the working set is smaller than the 129 MB L2).  `e2e` is the same metric through the
C ABI with host buffers: each step uploads vertices, indices, uniforms and the texture from pinned
host memory, renders, and reads the colour target back.  `--impl reference` times the CPU
restatement of wgpu-cpu's rasteriser (the oracle; the Rust reference cannot be built here) on all
host cores.  One GPU per process: with N > 1 every rank renders its own replica.
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
WORKLOAD = dict(width=1920, height=1080, level=6, tex_size=1024)


def config_block(flush: bool = True) -> dict:
    return {"workload": "textured icosphere: 81,920 tris, 1920x1080 Rgba8UnormSrgb + Depth32Float Less, "
                        "1024^2 texture, texture x Lambert, parity profile (nearest, sRGB as linear)",
            "triangles": 81920, "target": "1920x1080", "texture": "1024x1024 rgba8", "profile": "parity",
            "launch_mode": "per_pass", "tile": 16, "warps_per_tile": 8,
            "l2": "flushed between timed steps (256 MiB write)" if flush else "inputs resident",
            "seed": 2}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
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


def raster_traffic():
    """DRAM bytes per raster launch from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "raster_textured_icosphere_1080p.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            return None
    return None


def cpu_baseline(target_seconds: float = 12.0):
    """The oracle (CPU restatement of wgpu-cpu's rasteriser) on all host cores."""
    import oracle_device
    from wgpu_gb300 import workloads as wl

    cores = os.cpu_count() or 1
    dev = oracle_device.device(threads=cores)
    scene = wl.scene_textured_icosphere(dev, **WORKLOAD)
    frags, t0, frames = 0, time.perf_counter(), 0
    while True:
        idx = scene.render()
        frags += dev.submission_stats(idx).fragments_shaded
        frames += 1
        if time.perf_counter() - t0 > target_seconds or frames >= 200:
            break
    dt = time.perf_counter() - t0
    oracle_device.oracle_lib.load().orc_set_threads(1)
    return {"value": frags / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{frames} full frames of the workload ({frags // frames} fragments each) in {dt:.1f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    base = cpu_baseline(target_seconds=max(5.0, 2.0 * args.steps))
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": config_block(False),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    from wgpu_gb300 import api as W
    from wgpu_gb300 import workloads as wl

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = W.Device(device_ordinal=local, time_kernels=True)
    scene = wl.scene_textured_icosphere(dev, **WORKLOAD)
    enc = dev.create_command_encoder()
    scene.record(enc)
    cmd = enc.finish()

    for _ in range(args.warmup):
        dev.flush_caches()
        idx = dev.queue.submit([cmd])
    dev.poll(True, idx)
    frags_per_step = dev.submission_stats(idx).fragments_shaded

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    barrier()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        first = None
        subs = []
        for _ in range(args.steps):
            dev.flush_caches()
            i = dev.queue.submit([cmd])
            subs.append(i)
        dev.poll(True, subs[-1])
        wall = time.perf_counter() - t0
    barrier()
    stats = [dev.submission_stats(i) for i in subs]
    gpu_ms = [s.gpu_ms for s in stats]
    raster_ms = [getattr(s, "raster_ms", 0.0) for s in stats]
    device_s = sum(gpu_ms) / 1e3
    if world > 1:
        t = torch.tensor([device_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        device_s = float(t.item())
    total_frags = frags_per_step * args.steps * world
    value = total_frags / device_s
    launches = int(sum(s.kernel_launches for s in stats))

    # roofline of the dominant kernel (raster/shade/ROP): algorithmic bytes per launch
    w, h = WORKLOAD["width"], WORKLOAD["height"]
    pix_bytes = w * h * (4 + 4)                       # colour + depth written once per pixel
    frag_bytes = frags_per_step * (4 + 4 + 4 + 4)     # depth read + depth write + colour write + texel
    alg_bytes = pix_bytes + frag_bytes
    peak, peak_src = measured_peak_hbm()
    r_ms = float(np.mean(raster_ms)) if any(raster_ms) else float(np.mean(gpu_ms))
    achieved = alg_bytes / (r_ms / 1e3) / 1e9
    traffic = raster_traffic()

    # end to end through the C ABI with host buffers (pinned), host<->device copies timed
    pos, nrm, uv, faces = wl.displaced_icosphere(WORKLOAD["level"], 2)
    vdata = torch.from_numpy(np.concatenate([pos, nrm, uv], 1).astype(np.float32).ravel().view(np.uint8)).pin_memory()
    idata = torch.from_numpy(faces.ravel().view(np.uint8)).pin_memory()
    tdata = torch.from_numpy(wl.checker_noise_texture(WORKLOAD["tex_size"], 102).ravel()).pin_memory()
    udata = torch.from_numpy(np.frombuffer(
        wl.mvp_bytes(wl.camera_mvp(w, h)) + np.array([0.3, 0.5, 0.8, 0.0], np.float32).tobytes(), np.uint8).copy()
    ).pin_memory()
    out = torch.empty(w * h * 4, dtype=torch.uint8).pin_memory()
    vb, ib = scene.draws[0][2][0], scene.draws[0][3]
    ub, tex = scene._keep[2], scene._keep[3]

    def e2e_step():
        dev.queue.write_buffer(vb, 0, vdata.numpy())
        dev.queue.write_buffer(ib, 0, idata.numpy())
        dev.queue.write_buffer(ub, 0, udata.numpy())
        dev.queue.write_texture(tex, tdata.numpy())
        i = dev.queue.submit([cmd])
        dev.poll(True, i)
        dev.lib.texture_read(dev.handle, scene.color.handle, 0, out.data_ptr(), out.numel())
        return i

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e_steps = max(3, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e_steps
    h2d = vdata.numel() + idata.numel() + udata.numel() + tdata.numel()

    if rank == 0:
        base = cpu_baseline() if world == 1 and not args.no_cpu_baseline else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sum(gpu_ms) / len(gpu_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": config_block(), "fragments_per_step": frags_per_step,
            "wall_ms_per_step": wall * 1e3 / args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "kernel": "k_raster (tile sort + raster + shade + depth + ROP)",
                         "algorithmic_bytes_per_launch": alg_bytes, "kernel_ms": r_ms},
            "cpu_baseline": base,
            "e2e": {"value": frags_per_step / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(out.numel()), "ms_per_step": e2e_s * 1e3},
            "gpu_launches": launches,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    dev.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
