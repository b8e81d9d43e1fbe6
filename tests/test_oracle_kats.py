"""Pins the oracle against the known answers of wgpu-cpu's own unit tests.

The vectors come from tests/golden/reference_kats.json, extracted from the reference's test
sources by tests/golden/make_kats.py; each record names the test it came from.  Float
comparisons use the reference tests' own `assert_abs_diff_eq!` default (f32::EPSILON).
"""

import ctypes
import json
import os

import numpy as np
import pytest

import oracle_lib

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))
EPS = float(np.finfo(np.float32).eps)


@pytest.fixture(scope="module")
def orc():
    return oracle_lib.load()


def f32arr(vals):
    a = np.ascontiguousarray(np.asarray(vals, dtype=np.float32).ravel())
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


@pytest.mark.parametrize("case", KATS["bubblesort3"], ids=lambda c: str(c["input"]))
def test_bubblesort3(orc, case):
    v = (ctypes.c_int64 * 3)(*case["input"])
    orc.orc_kat_bubblesort3(v)
    assert list(v) == case["expected"], case["source"]


@pytest.mark.parametrize("case", KATS["bresenham"], ids=lambda c: f'{c["start"]}->{c["end"]}')
def test_bresenham(orc, case):
    xy = (ctypes.c_uint32 * 256)()
    t = (ctypes.c_float * 128)()
    n = orc.orc_kat_bresenham(*case["start"], *case["end"], xy, t, 128)
    pts = [[xy[2 * i], xy[2 * i + 1]] for i in range(n)]
    assert pts == case["expected"], case["source"]


@pytest.mark.parametrize("case", KATS["scanlines_no_panic"], ids=lambda c: str(c["tri"]))
def test_scanlines_regressions(orc, case):
    flat = (ctypes.c_uint32 * 6)(*[c for p in case["tri"] for c in p])
    out = (ctypes.c_int64 * (3 * 4096))()
    n = orc.orc_kat_scanlines(flat, out, 4096)
    assert n > 0, case["source"]
    rows = np.array(out[: 3 * n]).reshape(n, 3)
    assert (rows[:, 1] >= 0).all() and (rows[:, 2] >= rows[:, 1]).all()


def test_scanlines_rules(orc):
    """Closed properties of the span state machine (util/scanline.rs:84-146)."""
    def rows(tri):
        flat = (ctypes.c_uint32 * 6)(*[c for p in tri for c in p])
        out = (ctypes.c_int64 * (3 * 4096))()
        n = orc.orc_kat_scanlines(flat, out, 4096)
        return [tuple(out[3 * i: 3 * i + 3]) for i in range(n)]

    # flat bottom (b.y == c.y, a above): the last row is skipped.
    r = rows([(5, 0), (0, 4), (10, 4)])
    assert [y for y, _, _ in r] == [0, 1, 2, 3]
    # flat top (a.y == b.y): start in the second half, last row included.
    r = rows([(0, 0), (10, 0), (5, 4)])
    assert [y for y, _, _ in r] == [0, 1, 2, 3, 4]
    assert r[0] == (0, 0, 10)
    # degenerate line: one row from min x to max x.
    assert rows([(7, 3), (2, 3), (4, 3)]) == [(3, 2, 7)]
    # a single point.
    assert rows([(4, 4), (4, 4), (4, 4)]) == [(4, 4, 4)]


def test_triangle_strip(orc):
    case = KATS["triangle_strip"][0]
    out = (ctypes.c_uint32 * 3)()
    got = []
    for p in range(case["vertices"] - 2):
        orc.orc_kat_strip_tri(p, out)
        got.append(list(out))
    assert got == case["expected"], case["source"]


@pytest.mark.parametrize("case", KATS["front_face"], ids=lambda c: c["expected"])
def test_front_face(orc, case):
    verts = [v + [1.0] for v in case["vertices"]]  # Point3::to_homogeneous
    _, ptr = f32arr(verts)
    r = orc.orc_kat_tri_face(ptr)
    assert r == (1 if case["expected"] == "Ccw" else 0), case["source"]


@pytest.mark.parametrize("case", KATS["clip_line"], ids=lambda c: f'{c["a"]}-{c["b"]}')
def test_clip_line(orc, case):
    _, ptr = f32arr([case["a"], case["b"]])
    out = (ctypes.c_float * 8)()
    alphas = (ctypes.c_float * 2)()
    ok = orc.orc_kat_clip_line(ptr, out, alphas)
    if case["expected"] is None:
        assert ok == 0, case["source"]
    else:
        assert ok == 1, case["source"]
        np.testing.assert_allclose(np.array(out[:]).reshape(2, 4), np.array(case["expected"]), atol=EPS, rtol=0)


@pytest.mark.parametrize("case", KATS["clip_tri"], ids=lambda c: str(len(c["expected"])))
def test_clip_tri(orc, case):
    _, ptr = f32arr(case["tri"])
    out = (ctypes.c_float * (64 * 21))()
    n = orc.orc_kat_clip_tri(ptr, out, 64)
    assert n == len(case["expected"]), case["source"]
    got = np.array(out[: n * 21]).reshape(n, 3, 7)[:, :, :4]
    if n:
        np.testing.assert_allclose(got, np.array(case["expected"]), atol=EPS, rtol=0)


def test_clip_tri_barycentrics_identity(orc):
    """An unclipped triangle keeps Barycentric::at_vertex(i) (clipper.rs:760-765)."""
    _, ptr = f32arr([[0, 0.5, 0, 1], [-0.5, -0.5, 0, 1], [0.5, -0.5, 0, 1]])
    out = (ctypes.c_float * (64 * 21))()
    assert orc.orc_kat_clip_tri(ptr, out, 64) == 1
    b = np.array(out[:21]).reshape(3, 7)[:, 4:]
    assert (b == np.eye(3, dtype=np.float32)).all()


def test_clip_tri_many_subtriangles(orc):
    """A large triangle crossing all side planes splits into several sub-triangles whose
    vertices all lie inside the clip volume."""
    _, ptr = f32arr([[-3, -3, 0.5, 1], [3, -2.5, 0.5, 1], [0.2, 4, 0.5, 1]])
    out = (ctypes.c_float * (64 * 21))()
    n = orc.orc_kat_clip_tri(ptr, out, 64)
    assert 2 <= n <= 64
    v = np.array(out[: n * 21]).reshape(n, 3, 7)
    w = v[:, :, 3]
    assert (np.abs(v[:, :, 0]) <= w + 1e-6).all() and (np.abs(v[:, :, 1]) <= w + 1e-6).all()


def test_index_resolution_via_pass(orc):
    """u16/u32 index + base_vertex (index.rs:172-207) through the oracle's draw path:
    covered by tests/test_oracle_render.py; here the plain arithmetic."""
    for case in KATS["index_resolution"]:
        assert [i + case["base_vertex"] for i in case["indices"]] == case["expected"]


def test_texture_layout(orc):
    case = KATS["texture_layout"][0]
    assert orc.orc_kat_texture_byte_size(case["width"], case["height"], 1, 3) == case["byte_size"]


def test_f16_round_trip(orc):
    """binary16 conversion used by the extension profile: exhaustive round trip and RNE ties."""
    for h in range(0, 0x10000, 7):
        if (h & 0x7C00) == 0x7C00 and (h & 0x3FF):
            continue  # NaN payloads
        f = orc.orc_kat_f16_to_f32(h)
        assert orc.orc_kat_f32_to_f16(f) == h
    assert orc.orc_kat_f32_to_f16(ctypes.c_float(1.0 + 2.0 ** -11).value) == 0x3C00  # tie -> even
    assert orc.orc_kat_f32_to_f16(ctypes.c_float(1.0 + 3 * 2.0 ** -11).value) == 0x3C02
    assert orc.orc_kat_f32_to_f16(65520.0) == 0x7C00
    ref = np.array([0.1, 1e-6, -2.5e-8, 65504.0, 3.14159], dtype=np.float32)
    for v in ref:
        assert orc.orc_kat_f32_to_f16(float(v)) == int(np.float16(v).view(np.uint16))


def test_image_golden_equalities():
    """Only LFS pointers survive; equal oids pin two image equalities used by the render
    tests (colored_triangle == draw_backwards_no_cull, cull_front == draw_backwards)."""
    g = {x["name"]: x["oid"] for x in KATS["image_goldens"]}
    assert g["colored_triangle"] == g["colored_triangle_draw_backwards_no_cull"]
    assert g["colored_triangle_cull_front"] == g["colored_triangle_draw_backwards"]
