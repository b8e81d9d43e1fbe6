"""The oracle's whole render path on the reference's own integration scenes and on
properties that need no GPU (CPU-only)."""

import numpy as np
import pytest

import oracle_device
import scenes
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl


@pytest.fixture(scope="module")
def orc():
    return oracle_device.device()


def triangle(dev, ff, cull, topology=W.PrimitiveTopology.TRIANGLE_LIST, vertices=range(0, 3)):
    s = wl.scene_reference_triangle(dev, ff, cull, topology, vertices)
    idx = s.render()
    return dev.read_texture(s.color), dev.submission_stats(idx).fragments_shaded


def test_reference_triangle_golden_equalities(orc):
    """wgpu-cpu-tests/src/tests/colored_triangle.rs:140-198 with the LFS-oid equalities:
    colored_triangle == draw_backwards_no_cull, cull_front == draw_backwards == all black."""
    tri, n_tri = triangle(orc, W.FrontFace.CW, W.Face.BACK)
    cull_front, n_cf = triangle(orc, W.FrontFace.CW, W.Face.FRONT)
    backwards, n_b = triangle(orc, W.FrontFace.CCW, W.Face.BACK)
    backwards_nc, n_bnc = triangle(orc, W.FrontFace.CCW, W.Face.NONE)
    assert np.array_equal(tri, backwards_nc) and n_tri == n_bnc
    assert np.array_equal(cull_front, backwards) and n_cf == n_b == 0
    assert (cull_front[..., :3] == 0).all() and (cull_front[..., 3] == 255).all()
    # the lit triangle covers half of the 512x512 target (row 512 / column 512 fall outside)
    assert n_tri == 512 * 512 // 2
    assert tri[..., :3].any(axis=-1).sum() > 0.45 * 512 * 512


def test_reference_triangle_lines(orc):
    img, n = triangle(orc, W.FrontFace.CW, W.Face.NONE, W.PrimitiveTopology.LINE_STRIP, range(0, 4))
    assert n > 0 and img[..., :3].any(axis=-1).sum() == n


def test_threads_do_not_change_bits():
    a = oracle_device.device(threads=1)
    b = oracle_device.device(threads=5)
    ca, da, na = scenes.render_scene(a, wl.scene_textured_icosphere, width=320, height=200, level=3, tex_size=64)
    cb, db, nb = scenes.render_scene(b, wl.scene_textured_icosphere, width=320, height=200, level=3, tex_size=64)
    oracle_device.oracle_lib.load().orc_set_threads(1)
    assert na == nb and np.array_equal(ca, cb) and np.array_equal(da, db)


def test_parity_profile_rejects_what_the_reference_cannot_do(orc):
    with pytest.raises(W.GbrError) as e:
        wl.scene_blended_quads(orc, 64, 64, n_quads=4).render()
    assert e.value.status == -3  # UNSUPPORTED: Rgba16Float colour writes panic in the reference
    s = wl.scene_colored_sphere(orc, 64, 64)
    sm = orc.create_shader_module(native="mesh_color_perspective")
    pl = orc.create_render_pipeline(sm, [W.VertexBufferLayout(24, [W.VertexAttribute(3, 0, 0),
                                                                   W.VertexAttribute(3, 12, 1)])],
                                    W.PrimitiveState(), None, sm, [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
    s.draws[0] = (pl,) + s.draws[0][1:]
    with pytest.raises(W.GbrError) as e:
        s.render()
    assert e.value.status == -3  # perspective interpolation is todo!() in the reference


def test_validation_errors(orc):
    # index beyond the index buffer -> the reference panics (slice index out of range)
    s = wl.scene_colored_sphere(orc, 64, 64)
    pl, groups, vbs, ib, rng, bv = s.draws[0]
    s.draws[0] = (pl, groups, vbs, ib, range(0, rng.stop + 3), bv)
    with pytest.raises(W.GbrError) as e:
        s.render()
    assert e.value.status == -4


def test_random_clip_scene_runs(orc):
    img, _, n = scenes.random_clip_triangles(orc, 200, 96, 64, seed=3)
    assert n > 0 and img.shape == (64, 96, 4)


def test_second_target_set_renders_the_same_frame(orc):
    """with_new_targets (the second buffer of a double-buffered frame loop) draws the same draws
    into fresh targets of the same sizes and formats: both sets hold the same bytes."""
    s = wl.scene_batched(orc, n_targets=3, n_draws=5, tri_lo=20, tri_hi=400, side_lo=32, side_hi=96, seed=9)
    sb = wl.with_new_targets(s)
    pairs = list(zip(wl.scene_targets(s), wl.scene_targets(sb)))
    assert all(a[0] is not b[0] and a[1] is not b[1] for a, b in pairs)
    for sc in (s, sb):
        sc.render()
    for (ca, da), (cb, db) in pairs:
        assert (ca.width, ca.height, ca.format) == (cb.width, cb.height, cb.format)
        assert np.array_equal(orc.read_texture(ca), orc.read_texture(cb))
        assert np.array_equal(orc.read_texture(da), orc.read_texture(db))
