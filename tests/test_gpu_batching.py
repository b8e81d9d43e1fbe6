"""GPU parity of the batched launch modes: a submission of many render passes into many
targets renders the same bits whether it is merged into one launch sequence (BATCHED), split
per pass (PER_PASS) or per draw (PER_DRAW), replayed from a CUDA graph, or tile-autotuned — and
the same as the oracle."""

import numpy as np
import pytest

import oracle_device
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SMALL = dict(n_targets=12, n_draws=40, tri_lo=50, tri_hi=20000, side_lo=48, side_hi=400, seed=5)


def render_all(dev, **kw):
    s = wl.scene_batched(dev, **kw)
    idx = s.render()
    out = [(dev.read_texture(c), dev.read_texture(d)) for c, d, _ in s.passes]
    st = dev.submission_stats(idx)
    return out, st.fragments_shaded, st, s


def assert_targets_same(a, b, what):
    (ta, na), (tb, nb) = a, b
    assert len(ta) == len(tb)
    for t, ((ca, da), (cb, db)) in enumerate(zip(ta, tb)):
        diff = (ca != cb).any(-1)
        assert not diff.any(), f"{what}: target {t}: {int(diff.sum())} colour pixels differ"
        dd = da.view(np.uint32) != db.view(np.uint32)
        assert not dd.any(), f"{what}: target {t}: {int(dd.sum())} depth values differ"
    assert na == nb, f"{what}: fragments {na} vs {nb}"


@pytest.fixture(scope="module")
def oracle_result():
    orc = oracle_device.device(threads=8)
    out, n, _, _ = render_all(orc, **SMALL)
    return out, n


@pytest.mark.parametrize("order", [W.RasterOrder.AUTO, W.RasterOrder.ORDERED])
@pytest.mark.parametrize("mode", [W.LaunchMode.BATCHED, W.LaunchMode.PER_PASS, W.LaunchMode.PER_DRAW])
def test_launch_modes_match_oracle(oracle_result, mode, order):
    dev = W.Device(launch_mode=mode, tile_size=16, warps_per_tile=8, raster_order=order)
    try:
        out, n, st, _ = render_all(dev, **SMALL)
        assert_targets_same((out, n), oracle_result, f"mode {mode}")
        if mode == W.LaunchMode.BATCHED:
            # one launch sequence for all draws: the setup stage is one launch per vertex-shader
            # shape present in the batch, every other stage one launch
            assert st.kernel_launches <= 8, st.kernel_launches
        if mode == W.LaunchMode.PER_DRAW:
            assert st.kernel_launches >= 4 * SMALL["n_draws"]
    finally:
        dev.close()


def test_graph_replay_matches_oracle(oracle_result):
    """The first submission captures the batch's launches into a CUDA graph; resubmitting the same
    command buffer replays it."""
    dev = W.Device(use_graphs=True, tile_size=16, warps_per_tile=8)
    try:
        s = wl.scene_batched(dev, **SMALL)
        for rep in range(3):
            idx = s.render()
            out = [(dev.read_texture(c), dev.read_texture(d)) for c, d, _ in s.passes]
            assert_targets_same((out, dev.submission_stats(idx).fragments_shaded), oracle_result, f"graph rep {rep}")
    finally:
        dev.close()


def test_autotuned_tiles_match_oracle(oracle_result):
    """tile_size = warps_per_tile = 0 lets the device time candidate tile shapes on the first
    submissions of a batch shape and keep the fastest; every candidate renders the same bits."""
    dev = W.Device()
    try:
        s = wl.scene_batched(dev, **SMALL)
        for rep in range(7):  # the five candidate shapes, then the chosen one
            idx = s.render()
            out = [(dev.read_texture(c), dev.read_texture(d)) for c, d, _ in s.passes]
            assert_targets_same((out, dev.submission_stats(idx).fragments_shaded), oracle_result, f"autotune rep {rep}")
    finally:
        dev.close()
