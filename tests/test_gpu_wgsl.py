"""WGSL programs on the GPU: the reference's shader-arithmetic known answers (naga-cranelift
tests, evaluated through the translated vertex stage), and frames rendered with WGSL pipelines
that equal, bit for bit, the frames of the native programs they restate (which are themselves
checked against the oracle in test_gpu_parity.py)."""

import numpy as np
import pytest

import scenes
import wgsl_programs as P
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

ERR_SHADER_TRAP = 9


@pytest.fixture(scope="module")
def gpu():
    d = W.Device(tile_size=16, warps_per_tile=8)
    yield d
    d.close()


def vertex_only(dev, src):
    sm = dev.create_shader_module(wgsl=src)
    return dev.create_render_pipeline(sm, [], W.PrimitiveState(), None, None, [], vertex_entry_point="main")


def test_operator_known_answers(gpu):
    src, kats = P.ops_program()
    pl = vertex_only(gpu, src)
    _, var, errs = pl.eval_vertices(0, len(kats))
    bad = [(k["source"], k, int(var[i, 0]), int(errs[i])) for i, k in enumerate(kats) if var[i, 0] != 1 or errs[i]]
    assert not bad, bad[:5]


def test_structural_known_answers(gpu):
    src, recs = P.structural_program()
    pl = vertex_only(gpu, src)
    _, var, errs = pl.eval_vertices(0, len(recs))
    bad = []
    for i, r in enumerate(recs):
        if r["expected"][0] == "DivisionByZero":
            if errs[i] != ERR_SHADER_TRAP:
                bad.append((r["test"], "expected a trap", int(errs[i])))
        elif var[i, 0] != 1 or errs[i]:
            bad.append((r["test"], r["source"], int(var[i, 0]), int(errs[i])))
    assert not bad, bad


def test_vertex_index_program_matches_native(gpu):
    """A WGSL restatement of the colored-triangle program evaluates to the same positions and
    colours as the built-in one for every vertex index."""
    pl = vertex_only(gpu, P.TRIANGLE.replace("vmain", "main"))
    pos, var, errs = pl.eval_vertices(0, 9)
    assert not errs.any()
    for v in range(9):
        k = v % 3
        assert pos[v].tolist() == [float(k - 1), float((k & 1) * 2 - 1), 0.0, 1.0]
        assert var[v, :4].view(np.float32).tolist() == [float(k == 0), float(k == 1), float(k == 2), 1.0]


def frame(dev, s):
    idx = s.render()
    c = dev.read_texture(s.color)
    d = dev.read_texture(s.depth) if s.depth is not None else None
    return c, d, dev.submission_stats(idx).fragments_shaded


def assert_frames_equal(a, b, what):
    (ca, da, na), (cb, db, nb) = a, b
    diff = (ca != cb).any(-1)
    assert not diff.any(), f"{what}: {int(diff.sum())} pixels differ"
    if da is not None:
        assert (da.view(np.uint32) == db.view(np.uint32)).all(), f"{what}: depth differs"
    assert na == nb, f"{what}: fragments {na} vs {nb}"


def with_wgsl(s, dev, src, layouts, prim, depth, fmt, blend=None):
    sm = dev.create_shader_module(wgsl=src)
    pl = dev.create_render_pipeline(sm, layouts, prim, depth, sm, [W.ColorTargetState(fmt, blend)],
                                    vertex_entry_point="vmain", fragment_entry_point="fmain")
    s.draws = [(pl,) + tuple(d[1:]) for d in s.draws]
    return s


@pytest.mark.parametrize("ff,cull", [(W.FrontFace.CCW, W.Face.NONE), (W.FrontFace.CW, W.Face.BACK)])
def test_triangle_frame(gpu, ff, cull):
    nat = frame(gpu, wl.scene_reference_triangle(gpu, front_face=ff, cull_mode=cull))
    s = wl.scene_reference_triangle(gpu, front_face=ff, cull_mode=cull)
    s = with_wgsl(s, gpu, P.TRIANGLE, [], W.PrimitiveState(front_face=ff, cull_mode=cull),
                  W.DepthStencilState(True, W.CompareFunction.LESS), W.TextureFormat.RGBA8_UNORM_SRGB)
    assert_frames_equal(frame(gpu, s), nat, "colored triangle")


MESH_LAYOUT = [W.VertexBufferLayout(24, [W.VertexAttribute(W.VertexFormat.FLOAT32X3, 0, 0),
                                         W.VertexAttribute(W.VertexFormat.FLOAT32X3, 12, 1)])]


def test_mesh_color_frame(gpu):
    nat = frame(gpu, wl.scene_colored_sphere(gpu, 300, 200))
    s = wl.scene_colored_sphere(gpu, 300, 200)
    s = with_wgsl(s, gpu, P.MESH_COLOR, MESH_LAYOUT, W.PrimitiveState(cull_mode=W.Face.BACK), None,
                  W.TextureFormat.RGBA8_UNORM)
    assert_frames_equal(frame(gpu, s), nat, "mesh colour")


def test_mesh_color_discard_frame(gpu):
    def native(dev):
        s = wl.scene_colored_sphere(dev, 200, 160)
        sm = dev.create_shader_module(native="mesh_color_discard")
        pl = dev.create_render_pipeline(sm, MESH_LAYOUT, W.PrimitiveState(cull_mode=W.Face.BACK), None, sm,
                                        [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
        s.draws[0] = (pl,) + s.draws[0][1:]
        return s
    nat = frame(gpu, native(gpu))
    s = with_wgsl(wl.scene_colored_sphere(gpu, 200, 160), gpu, P.MESH_COLOR_DISCARD, MESH_LAYOUT,
                  W.PrimitiveState(cull_mode=W.Face.BACK), None, W.TextureFormat.RGBA8_UNORM)
    assert_frames_equal(frame(gpu, s), nat, "discard")


TEX_LAYOUT = [W.VertexBufferLayout(32, [W.VertexAttribute(W.VertexFormat.FLOAT32X3, 0, 0),
                                        W.VertexAttribute(W.VertexFormat.FLOAT32X3, 12, 1),
                                        W.VertexAttribute(W.VertexFormat.FLOAT32X2, 24, 2)])]


@pytest.mark.parametrize("order", [W.RasterOrder.AUTO, W.RasterOrder.ORDERED])
def test_textured_lambert_frame(order):
    dev = W.Device(tile_size=16, warps_per_tile=8, raster_order=order)
    try:
        kw = dict(width=480, height=270, level=4, tex_size=256)
        nat = frame(dev, wl.scene_textured_icosphere(dev, **kw))
        s = wl.scene_textured_icosphere(dev, **kw)
        s = with_wgsl(s, dev, P.TEX_LAMBERT, TEX_LAYOUT, W.PrimitiveState(cull_mode=W.Face.NONE),
                      W.DepthStencilState(True, W.CompareFunction.LESS), W.TextureFormat.RGBA8_UNORM_SRGB)
        assert_frames_equal(frame(dev, s), nat, f"textured Lambert ({order})")
    finally:
        dev.close()


def test_trap_fails_the_draw(gpu):
    src = P.MESH_COLOR.replace("o.col = c;", "var z: i32 = 0; var q: i32 = 7 / z; o.col = c;")
    s = with_wgsl(wl.scene_colored_sphere(gpu, 64, 64), gpu, src, MESH_LAYOUT, W.PrimitiveState(cull_mode=W.Face.BACK),
                  None, W.TextureFormat.RGBA8_UNORM)
    with pytest.raises(W.GbrError) as e:
        s.render()
    assert e.value.status == -4
    frame(gpu, wl.scene_colored_sphere(gpu, 64, 64))  # the device stays usable


@pytest.mark.parametrize("order", [W.RasterOrder.AUTO, W.RasterOrder.ORDERED])
def test_edge_rule_frames(order):
    """WGSL modules are compiled with the edge-function instantiations of the kernels when the
    device uses that rule: their frames equal the native programs' under the same rule."""
    dev = W.Device(profile=W.Profile.EXTENSION, raster_rule=W.RasterRule.EDGE, raster_order=order)
    try:
        nat = frame(dev, wl.scene_colored_sphere(dev, 300, 200))
        s = with_wgsl(wl.scene_colored_sphere(dev, 300, 200), dev, P.MESH_COLOR, MESH_LAYOUT,
                      W.PrimitiveState(cull_mode=W.Face.BACK), None, W.TextureFormat.RGBA8_UNORM)
        assert_frames_equal(frame(dev, s), nat, f"edge rule mesh colour ({order})")
        ff, cull = W.FrontFace.CCW, W.Face.NONE
        nat = frame(dev, wl.scene_reference_triangle(dev, front_face=ff, cull_mode=cull))
        s = with_wgsl(wl.scene_reference_triangle(dev, front_face=ff, cull_mode=cull), dev, P.TRIANGLE, [],
                      W.PrimitiveState(front_face=ff, cull_mode=cull), W.DepthStencilState(True, W.CompareFunction.LESS),
                      W.TextureFormat.RGBA8_UNORM_SRGB)
        assert_frames_equal(frame(dev, s), nat, f"edge rule triangle ({order})")
    finally:
        dev.close()
