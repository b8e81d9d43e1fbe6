"""Renders the benchmark configurations at full size through the oracle (the CPU restatement of
wgpu-cpu's rasteriser) and writes tests/golden/frame_digests.json: per configuration the SHA-256
of the scene's inputs, the shaded-fragment count and the SHA-256 of every target's colour and
depth bytes.  The full-size GPU tests and bench.py compare libgbr's frames with these digests.

    python tests/golden/make_frame_digests.py [--threads N] [name ...]

Names are the keys of wgpu_gb300.workloads.FULL_SIZE (default: all of them).  Entries already in
the file are kept unless named again.  The blend configuration (3840x2160, 10,000 alpha-blended
quads, about 3.1e9 fragments) takes the longest: several minutes on a few cores.
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "wgpu-cpu_gb300"), os.path.join(ROOT, "tests")]

import frame_digests as fd  # noqa: E402
import oracle_device  # noqa: E402
from wgpu_gb300 import workloads as wl  # noqa: E402


def render(name: str, threads: int) -> dict:
    _, profile, _ = wl.FULL_SIZE[name]
    dev = oracle_device.device(profile=profile, threads=threads)
    try:
        scene = wl.build_config(dev, name)
        t0 = time.perf_counter()
        idx = scene.render()
        dt = time.perf_counter() - t0
        return {"inputs": fd.input_digest(scene), "fragments": int(dev.submission_stats(idx).fragments_shaded),
                "targets": fd.target_digests(dev, scene), "oracle_seconds": round(dt, 1), "oracle_threads": threads,
                "arguments": {k: v for k, v in wl.FULL_SIZE[name][2].items()}}
    finally:
        dev.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("names", nargs="*", default=list(wl.FULL_SIZE))
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    data = {"about": "full-size frames of the benchmark configurations rendered by the oracle "
                     "(tests/golden/make_frame_digests.py); sha256 of inputs and of each target's bytes",
            "configs": {}}
    if os.path.exists(fd.FIXTURE):
        data = json.load(open(fd.FIXTURE))
    for name in args.names:
        t0 = time.perf_counter()
        data["configs"][name] = render(name, args.threads)
        print(f"{name}: {data['configs'][name]['fragments']} fragments, "
              f"{len(data['configs'][name]['targets'])} targets, {time.perf_counter() - t0:.1f} s", flush=True)
        with open(fd.FIXTURE, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main()
