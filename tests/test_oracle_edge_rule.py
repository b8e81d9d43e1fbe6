"""The extension profile's edge-function raster rule in the oracle (no GPU): 1/256-pixel
snapping, pixel-centre coverage, top-left rule.  Checked against a brute-force restatement in
Python integers (every pixel centre against the three edges), on hand-placed triangles whose
edges run exactly through pixel centres, on random triangles of both windings, and on meshes
that tile a rectangle, where every centre inside must be covered exactly once."""

import numpy as np
import pytest

import oracle_device
import scenes
from wgpu_gb300 import api as W

WIDTH, HEIGHT = 128, 64  # powers of two: pixel coordinates on a 1/256 grid map to clip space exactly


def model_mask(tri, width, height):
    """Covered pixels of one triangle by the rule, in exact integers."""
    X = [int(round(x * 256)) for x, _ in tri]
    Y = [int(round(y * 256)) for _, y in tri]
    a2 = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0])
    if a2 == 0:
        return np.zeros((height, width), bool)
    if a2 < 0:
        X[1], X[2], Y[1], Y[2] = X[2], X[1], Y[2], Y[1]
    yy, xx = np.mgrid[0:height, 0:width]
    px, py = xx * 256 + 128, yy * 256 + 128
    inside = np.ones((height, width), bool)
    for i in range(3):
        j = (i + 1) % 3
        dx, dy = X[j] - X[i], Y[j] - Y[i]
        e = dx * (py - Y[i]) - dy * (px - X[i])
        owns = dy < 0 or (dy == 0 and dx > 0)
        inside &= (e > 0) | ((e == 0) & owns)
    return inside


def model_counts(tris, width, height):
    return sum(model_mask(t, width, height).astype(np.int64) for t in tris)


@pytest.fixture(scope="module")
def orc_edge():
    return oracle_device.device(profile=W.Profile.EXTENSION, threads=4, raster_rule=W.RasterRule.EDGE)


def test_top_left_rule_on_centre_edges(orc_edge):
    """Right triangle with its three edges through pixel centres: the top edge (row 10) and the
    left edge (column 10) own their centres, the hypotenuse x + y = 30 does not."""
    tri = [(10.5, 10.5), (20.5, 10.5), (10.5, 20.5)]
    counts, n = scenes.coverage_counts(orc_edge, WIDTH, HEIGHT, [tri])
    want = np.zeros((HEIGHT, WIDTH), np.int64)
    for y in range(HEIGHT):
        for x in range(WIDTH):
            if x >= 10 and y >= 10 and x + y < 30:
                want[y, x] = 1
    assert np.array_equal(counts, want)
    assert n == want.sum() == 55
    # the same triangle wound the other way covers the same pixels
    counts2, _ = scenes.coverage_counts(orc_edge, WIDTH, HEIGHT, [[tri[0], tri[2], tri[1]]])
    assert np.array_equal(counts2, want)
    # the complementary triangle across the hypotenuse owns it: together exactly the square once
    other = [(20.5, 10.5), (20.5, 20.5), (10.5, 20.5)]
    both, _ = scenes.coverage_counts(orc_edge, WIDTH, HEIGHT, [tri, other])
    square = np.zeros((HEIGHT, WIDTH), np.int64)
    square[10:20, 10:20] = 1
    assert np.array_equal(both, square)


def test_random_triangles_match_model(orc_edge):
    rng = np.random.default_rng(21)
    tris = []
    for k in range(60):
        pts = rng.uniform([-4, -4], [WIDTH + 4, HEIGHT + 4], (3, 2))
        if k % 3 == 0:
            pts = np.round(pts * 2) / 2  # corners and edges through centres
        else:
            pts = np.round(pts * 256) / 256
        tris.append([tuple(p) for p in pts])
    for t in tris:
        t = [(min(max(x, 0.0), WIDTH), min(max(y, 0.0), HEIGHT)) for x, y in t]  # inside the clip volume
        counts, n = scenes.coverage_counts(orc_edge, WIDTH, HEIGHT, [t])
        want = model_mask(t, WIDTH, HEIGHT).astype(np.int64)
        assert np.array_equal(counts, want), t
        assert n == want.sum()


@pytest.mark.parametrize("seed,flip", [(1, False), (2, True), (3, False)])
def test_mesh_covers_each_centre_once(orc_edge, seed, flip):
    """A jittered grid mesh over [x0, x1] x [y0, y1] (1/256-pixel vertices, both diagonal
    directions): every pixel centre strictly inside is covered exactly once, and the rectangle's
    own top and left edges own the centres on them."""
    rng = np.random.default_rng(seed)
    x0, x1, y0, y1 = 7.5, 101.25, 4.0, 58.5
    nx, ny = 9, 6
    gx = np.linspace(x0, x1, nx + 1)
    gy = np.linspace(y0, y1, ny + 1)
    P = np.zeros((ny + 1, nx + 1, 2))
    for j in range(ny + 1):
        for i in range(nx + 1):
            p = np.array([gx[i], gy[j]])
            if 0 < i < nx and 0 < j < ny:
                p += rng.uniform(-2.5, 2.5, 2)
            P[j, i] = np.round(p * 256) / 256
    tris = []
    for j in range(ny):
        for i in range(nx):
            a, b, c, d = P[j, i], P[j, i + 1], P[j + 1, i + 1], P[j + 1, i]
            if (i + j + flip) % 2:
                tris += [[a, b, c], [a, c, d]]
            else:
                tris += [[a, b, d], [b, c, d]]
    counts, n = scenes.coverage_counts(orc_edge, WIDTH, HEIGHT, [[tuple(p) for p in t] for t in tris])
    want = model_counts([[tuple(p) for p in t] for t in tris], WIDTH, HEIGHT)
    assert np.array_equal(counts, want)
    xs = np.arange(WIDTH) + 0.5
    ys = np.arange(HEIGHT) + 0.5
    inside = ((ys[:, None] >= y0) & (ys[:, None] < y1)) & ((xs[None, :] >= x0) & (xs[None, :] < x1))
    assert np.array_equal(counts, inside.astype(np.int64))
    assert n == inside.sum()


def test_edge_rule_needs_the_extension_profile():
    with pytest.raises(Exception):
        oracle_device.device(profile=W.Profile.PARITY, raster_rule=W.RasterRule.EDGE)
