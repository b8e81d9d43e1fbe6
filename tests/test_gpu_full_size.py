"""The benchmark configurations at their full sizes, rendered by libgbr, against the oracle's
frames (tests/golden/frame_digests.json, made by tests/golden/make_frame_digests.py).

These are the frames bench.py times: 256 draws into 64 targets (6.3 M primitives, 45.9 M
fragments), 10,000 alpha-blended quads into 3840x2160 Rgba16Float (3.1 G fragments), the
textured icosphere in both profiles and the coloured sphere.  Each must match the oracle bit for
bit — colour bytes, Depth32Float bits and the shaded-fragment count — through every launch path
the benchmark reports: graph-captured with the autotuner choosing the tile shape (every trial
shape included), the plain per-draw path, and fixed shapes with both raster orders.
"""

import numpy as np
import pytest

import frame_digests as fd
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FIXTURE = fd.load_fixture()


def render_and_compare(name, dev, submissions=1):
    """Builds configuration `name` on `dev`, submits it `submissions` times and compares every
    submission's frame with the fixture."""
    scene = wl.build_config(dev, name)
    inputs = fd.input_digest(scene)
    enc = dev.create_command_encoder()
    scene.record(enc)
    cmd = enc.finish()
    diffs = []
    for k in range(submissions):
        idx = dev.queue.submit([cmd])
        dev.poll(True, idx)
        frags = dev.submission_stats(idx).fragments_shaded
        diffs += [f"submission {k}: {d}" for d in fd.compare(name, inputs, fd.target_digests(dev, scene), frags, FIXTURE)]
    return diffs


def test_batched_graph_autotuned():
    """As the benchmark runs it: one command buffer replayed from a CUDA graph, the autotuner
    timing its candidate tile shapes on the first submissions (each of them checked)."""
    dev = W.Device(use_graphs=True, time_kernels=True)
    try:
        diffs = render_and_compare("batched", dev, submissions=7)
    finally:
        dev.close()
    assert not diffs, diffs


def test_batched_per_draw():
    """The plain drop-in path: one launch sequence per draw."""
    dev = W.Device(launch_mode=W.LaunchMode.PER_DRAW, tile_size=32, warps_per_tile=8)
    try:
        diffs = render_and_compare("batched", dev)
    finally:
        dev.close()
    assert not diffs, diffs


@pytest.mark.parametrize("tile,warps,order", [(16, 4, W.RasterOrder.AUTO), (32, 8, W.RasterOrder.ORDERED),
                                              (8, 2, W.RasterOrder.AUTO)])
def test_batched_fixed_shapes(tile, warps, order):
    dev = W.Device(tile_size=tile, warps_per_tile=warps, raster_order=order)
    try:
        diffs = render_and_compare("batched", dev)
    finally:
        dev.close()
    assert not diffs, diffs


@pytest.mark.parametrize("tile,warps", [(32, 8), (16, 8)])
def test_blend_full(tile, warps):
    """10,000 quads alpha-blended in painter order into 3840x2160 Rgba16Float: bit-exact."""
    dev = W.Device(profile=W.Profile.EXTENSION, tile_size=tile, warps_per_tile=warps)
    try:
        diffs = render_and_compare("blend", dev, submissions=2)
    finally:
        dev.close()
    assert not diffs, diffs


@pytest.mark.parametrize("name", ["colored", "textured", "textured_filtered"])
def test_single_pass_configs(name):
    _, profile, _ = wl.FULL_SIZE[name]
    dev = W.Device(profile=profile, use_graphs=True)
    try:
        diffs = render_and_compare(name, dev, submissions=2)
    finally:
        dev.close()
    assert not diffs, diffs
