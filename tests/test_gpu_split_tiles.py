"""GPU parity of the visibility raster's split tiles: dense meshes drawn into small targets bin
thousands of records into single tiles, which the raster cuts into chunks of 2048 records (or
the chunk size GBR_VIS_SPLIT_CHUNK gives) run by different CTAs and merged by the last one to
finish.  Colour, depth and the
fragment count must equal the oracle's bit for bit, at every tile shape, under both raster
rules, and when the split buffers hold only some of the heavy tiles (the rest are rasterised
whole)."""

import numpy as np
import pytest

import oracle_device
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

DENSE = dict(n_targets=2, n_draws=6, tri_lo=30000, tri_hi=60000, side_lo=64, side_hi=80, seed=7)


def render_all(dev, **kw):
    s = wl.scene_batched(dev, **kw)
    idx = s.render()
    out = [(dev.read_texture(c), dev.read_texture(d)) for c, d, _ in s.passes]
    return out, dev.submission_stats(idx)


def assert_targets_same(a, b, what):
    assert len(a) == len(b)
    for t, ((ca, da), (cb, db)) in enumerate(zip(a, b)):
        diff = (ca != cb).any(-1)
        assert not diff.any(), f"{what}: target {t}: {int(diff.sum())} colour pixels differ"
        dd = da.view(np.uint32) != db.view(np.uint32)
        assert not dd.any(), f"{what}: target {t}: {int(dd.sum())} depth values differ"


@pytest.fixture(scope="module")
def oracle_dense():
    out, st = render_all(oracle_device.device(threads=8), **DENSE)
    return out, st.fragments_shaded


@pytest.fixture(scope="module")
def oracle_dense_edge():
    orc = oracle_device.device(profile=W.Profile.EXTENSION, threads=8, raster_rule=W.RasterRule.EDGE)
    out, st = render_all(orc, **DENSE)
    return out, st.fragments_shaded


@pytest.mark.parametrize("tile,warps", [(8, 1), (16, 4), (32, 8)])
def test_split_tiles_match_oracle(oracle_dense, tile, warps):
    dev = W.Device(tile_size=tile, warps_per_tile=warps)
    try:
        out, st = render_all(dev, **DENSE)
        assert st.split_tile_chunks >= 2, "no tile was split: the scene no longer exercises the split path"
        assert_targets_same(out, oracle_dense[0], f"tile {tile} warps {warps}")
        assert st.fragments_shaded == oracle_dense[1]
    finally:
        dev.close()


def test_split_tiles_edge_rule(oracle_dense_edge):
    dev = W.Device(profile=W.Profile.EXTENSION, raster_rule=W.RasterRule.EDGE, tile_size=16, warps_per_tile=4)
    try:
        out, st = render_all(dev, **DENSE)
        assert st.split_tile_chunks >= 2
        assert_targets_same(out, oracle_dense_edge[0], "edge rule")
        assert st.fragments_shaded == oracle_dense_edge[1]
    finally:
        dev.close()


def test_split_capacity_leaves_the_rest_whole(oracle_dense, monkeypatch):
    """With room for fewer chunk work items than the heavy tiles need, the heavy tiles that fit
    (a prefix of k_scan's list) are split and the others rasterised by one CTA each; with room
    for one item none is split.  The same image every time."""
    dev = W.Device(tile_size=16, warps_per_tile=4)
    try:
        _, st = render_all(dev, **DENSE)
        full = st.split_tile_chunks
    finally:
        dev.close()
    assert full >= 4
    for cap, lo, hi in [(full - 1, 2, full - 1), (1, 0, 0)]:
        monkeypatch.setenv("GBR_VIS_SPLIT_ITEMS", str(cap))
        dev = W.Device(tile_size=16, warps_per_tile=4)
        try:
            out, st = render_all(dev, **DENSE)
            assert lo <= st.split_tile_chunks <= hi, (cap, st.split_tile_chunks)
            assert_targets_same(out, oracle_dense[0], f"cap {cap}")
            assert st.fragments_shaded == oracle_dense[1]
        finally:
            dev.close()


@pytest.mark.parametrize("chunk", [100, 700])
def test_split_chunk_sizes(oracle_dense, chunk, monkeypatch):
    """Chunks smaller than a CTA's width and of sizes that are no multiple of it."""
    monkeypatch.setenv("GBR_VIS_SPLIT_CHUNK", str(chunk))
    dev = W.Device(tile_size=16, warps_per_tile=4)
    try:
        out, st = render_all(dev, **DENSE)
        assert st.split_tile_chunks >= 20
        assert_targets_same(out, oracle_dense[0], f"chunk {chunk}")
        assert st.fragments_shaded == oracle_dense[1]
    finally:
        dev.close()
