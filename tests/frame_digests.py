"""Digests of full-size frames: what the parity fixture (tests/golden/frame_digests.json) stores
and what the full-size GPU tests and bench.py compare with it.

A frame is checked through SHA-256 digests instead of pixels, so a 3840x2160 Rgba16Float target
or 64 targets of up to 2048x2048 need a few hundred bytes of fixture each.  Every digest covers
the exact bytes read back (colour texels, and Depth32Float depth as f32 bits), so equal digests
mean bit-exact frames.  The scene's inputs get a digest too: the vertex, index, uniform and
texture bytes the workload generator produced.  The fixture is generated on one machine and
checked on another, so a test first compares the input digest — a mismatch there means the
generator produced other inputs (a different platform's libm, say), not that the renderer
differs — and only then the frame.
"""

from __future__ import annotations

import hashlib
import json
import os

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "frame_digests.json")


def _sha(arr) -> str:
    a = np.ascontiguousarray(arr)
    return hashlib.sha256(a.reshape(-1).view(np.uint8).tobytes()).hexdigest()


def input_digest(scene) -> str:
    """SHA-256 over every upload of the scene (buffers and texture level 0), in upload order."""
    h = hashlib.sha256()
    for _, arr in scene.uploads:
        a = np.ascontiguousarray(arr)
        h.update(str(a.nbytes).encode())
        h.update(a.reshape(-1).view(np.uint8).tobytes())
    return h.hexdigest()


def target_digests(dev, scene) -> list:
    """[[colour sha256, depth sha256 or None], ...] of every target of the scene, pass order."""
    from wgpu_gb300 import workloads as wl

    pairs = wl.scene_targets(scene)
    colors = dev.read_textures([c for c, _ in pairs])
    depths_t = [d for _, d in pairs if d is not None]
    depths = iter(dev.read_textures(depths_t)) if depths_t else iter(())
    out = []
    for (c, d), img in zip(pairs, colors):
        out.append([_sha(img), _sha(next(depths)) if d is not None else None])
    return out


def load_fixture() -> dict:
    with open(FIXTURE) as f:
        return json.load(f)


def compare(name: str, inputs: str, targets: list, fragments: int, fixture: dict | None = None) -> list:
    """Differences between a rendered frame and the fixture entry `name` (empty when equal)."""
    fx = (fixture or load_fixture())["configs"][name]
    if inputs != fx["inputs"]:
        return [f"{name}: the scene generator produced other inputs than the fixture's ({inputs[:12]} vs "
                f"{fx['inputs'][:12]}): the frames cannot be compared"]
    diffs = []
    if fragments != fx["fragments"]:
        diffs.append(f"{name}: {fragments} fragments shaded, fixture {fx['fragments']}")
    if len(targets) != len(fx["targets"]):
        return diffs + [f"{name}: {len(targets)} targets, fixture {len(fx['targets'])}"]
    for k, (got, want) in enumerate(zip(targets, fx["targets"])):
        if got[0] != want[0]:
            diffs.append(f"{name}: target {k} colour differs")
        if got[1] != want[1]:
            diffs.append(f"{name}: target {k} depth differs")
    return diffs
