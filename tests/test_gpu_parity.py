"""GPU parity: the CUDA path (libgbr.so through the C ABI) against the oracle on the same seeded
inputs.  Colour and depth must be bit-exact and the fragment-shader invocation count equal; the
f16 blend target (extension profile) is compared to within 1 f16 ULP, though it is expected to
match exactly as well."""

import numpy as np
import pytest

import oracle_device
import scenes
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    d = W.Device()
    yield d
    d.close()


@pytest.fixture(scope="module")
def gpu_ordered():
    """Every batch walks its fragments in primitive order (no visibility raster)."""
    d = W.Device(raster_order=W.RasterOrder.ORDERED)
    yield d
    d.close()


@pytest.fixture(scope="module")
def gpu_ext():
    d = W.Device(profile=W.Profile.EXTENSION)
    yield d
    d.close()


@pytest.fixture(scope="module")
def orc():
    return oracle_device.device(threads=8)


@pytest.fixture(scope="module")
def orc_ext():
    return oracle_device.device(profile=W.Profile.EXTENSION, threads=8)


def assert_same(a, b, what=""):
    (ca, da, na), (cb, db, nb) = a, b
    diff = (ca != cb).any(-1)
    assert not diff.any(), f"{what}: {int(diff.sum())} colour pixels differ, first at {np.argwhere(diff)[:3].tolist()}"
    if da is not None or db is not None:
        dd = da.view(np.uint32) != db.view(np.uint32)
        assert not dd.any(), f"{what}: {int(dd.sum())} depth values differ"
    assert na == nb, f"{what}: fragments {na} vs {nb}"


@pytest.mark.parametrize("ff,cull", [(W.FrontFace.CW, W.Face.BACK), (W.FrontFace.CW, W.Face.FRONT),
                                     (W.FrontFace.CCW, W.Face.BACK), (W.FrontFace.CCW, W.Face.NONE)])
def test_reference_triangle(gpu, orc, ff, cull):
    res = [scenes.render_scene(d, wl.scene_reference_triangle, front_face=ff, cull_mode=cull) for d in (gpu, orc)]
    assert_same(*res, "colored_triangle")


def test_colored_sphere_512(gpu, orc):
    res = [scenes.render_scene(d, wl.scene_colored_sphere) for d in (gpu, orc)]
    assert_same(*res, "colored sphere 512x512")
    assert res[0][2] > 50000


@pytest.mark.parametrize("cull", [W.Face.NONE, W.Face.FRONT])
def test_colored_sphere_cull_modes(gpu, orc, cull):
    res = [scenes.render_scene(d, wl.scene_colored_sphere, width=300, height=200, cull=cull) for d in (gpu, orc)]
    assert_same(*res, f"cull {cull}")


def test_textured_icosphere_small(gpu, orc):
    kw = dict(width=480, height=270, level=4, tex_size=256)
    res = [scenes.render_scene(d, wl.scene_textured_icosphere, **kw) for d in (gpu, orc)]
    assert_same(*res, "textured icosphere level 4")


def test_textured_icosphere_full(gpu, gpu_ordered, orc):
    """The textured-mesh workload at full size: 81,920 triangles, 1920x1080 + Depth32Float."""
    res = [scenes.render_scene(d, wl.scene_textured_icosphere) for d in (gpu, gpu_ordered, orc)]
    assert_same(res[0], res[2], "textured icosphere level 6 1080p")
    assert_same(res[1], res[2], "textured icosphere level 6 1080p (ordered)")
    assert res[0][2] > 500000


@pytest.mark.parametrize("address", [W.AddressMode.CLAMP_TO_EDGE, W.AddressMode.MIRROR_REPEAT])
def test_textured_address_modes(gpu, orc, address):
    kw = dict(width=256, height=160, level=3, tex_size=64, address=address)
    res = [scenes.render_scene(d, wl.scene_textured_icosphere, **kw) for d in (gpu, orc)]
    assert_same(*res, f"address mode {address}")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_clip_triangles(gpu, orc, seed):
    """Triangles crossing every clip plane: sub-triangle order, the clipped-depth composition and
    degenerate spans."""
    kw = dict(n_tris=400, width=160, height=120, seed=seed)
    res = [scenes.random_clip_triangles(d, **kw) for d in (gpu, orc)]
    assert_same(*res, f"random clip seed {seed}")


@pytest.mark.parametrize("compare", [W.CompareFunction.LESS, W.CompareFunction.LESS_EQUAL, W.CompareFunction.GREATER,
                                     W.CompareFunction.GREATER_EQUAL, W.CompareFunction.EQUAL,
                                     W.CompareFunction.NOT_EQUAL, W.CompareFunction.ALWAYS, W.CompareFunction.NEVER])
def test_depth_compare_functions(gpu, gpu_ordered, orc, compare):
    kw = dict(n_tris=300, width=128, height=96, seed=11, depth=compare, z_range=(0.0, 1.0), spread=0.9)
    res = [scenes.random_clip_triangles(d, **kw) for d in (gpu, gpu_ordered, orc)]
    assert_same(res[0], res[2], f"depth compare {compare}")
    assert_same(res[1], res[2], f"depth compare {compare} (ordered)")


@pytest.mark.parametrize("compare", [W.CompareFunction.LESS, W.CompareFunction.LESS_EQUAL, W.CompareFunction.GREATER,
                                     W.CompareFunction.GREATER_EQUAL])
@pytest.mark.parametrize("z", [0.5, 0.0])
def test_depth_ties(gpu, gpu_ordered, orc, compare, z):
    """Triangles at one constant depth, so most fragments tie: Less / Greater keep the first of
    equal depths, LessEqual / GreaterEqual the last.  z = 0 also mixes -0.0 and +0.0 depths,
    which compare equal."""
    for clear_depth in (1.0, z, -0.0):
        kw = dict(n_tris=250, width=120, height=90, seed=17, depth=compare, z_range=(z, z), spread=0.9,
                  w_range=(1.0, 1.0))
        res = [scenes.random_clip_triangles(d, depth_clear=clear_depth, **kw) for d in (gpu, gpu_ordered, orc)]
        assert_same(res[0], res[2], f"ties {compare} z={z} clear={clear_depth}")
        assert_same(res[1], res[2], f"ties {compare} z={z} clear={clear_depth} (ordered)")


def test_depth_write_disabled(gpu, orc):
    kw = dict(n_tris=300, width=128, height=96, seed=12, depth=W.CompareFunction.LESS, depth_write=False,
              z_range=(0.0, 1.0), spread=0.9)
    res = [scenes.random_clip_triangles(d, **kw) for d in (gpu, orc)]
    assert_same(*res, "depth write disabled")


def test_strip_u16_instances_base_vertex(gpu, orc):
    kw = dict(n_tris=120, width=128, height=96, seed=5, topology=W.PrimitiveTopology.TRIANGLE_STRIP,
              index_format=W.IndexFormat.UINT16, instances=3, base_vertex=7, cull=W.Face.BACK,
              depth=W.CompareFunction.LESS_EQUAL, z_range=(0.0, 1.0))
    res = [scenes.random_clip_triangles(d, **kw) for d in (gpu, orc)]
    assert_same(*res, "strip/u16/instances/base_vertex")


def test_direct_draw_scissor_viewport(gpu, orc):
    kw = dict(n_tris=200, width=200, height=150, seed=8, scissor=(17, 9, 150, 101),
              viewport=(-30.0, 12.5, 260.0, 120.0, 0.0, 1.0))
    res = [scenes.random_clip_triangles(d, **kw) for d in (gpu, orc)]
    assert_same(*res, "scissor + viewport")


def test_bgra_target(gpu, orc):
    kw = dict(n_tris=100, width=96, height=64, seed=9, color_format=W.TextureFormat.BGRA8_UNORM)
    res = [scenes.random_clip_triangles(d, **kw) for d in (gpu, orc)]
    assert_same(*res, "bgra8")


@pytest.mark.parametrize("tile,warps", [(8, 1), (8, 2), (16, 2), (16, 4), (32, 4), (32, 8)])
def test_tile_configurations(orc, tile, warps):
    dev = W.Device(tile_size=tile, warps_per_tile=warps)
    try:
        kw = dict(n_tris=300, width=150, height=110, seed=21, depth=W.CompareFunction.LESS, z_range=(0.0, 1.0))
        res = [scenes.random_clip_triangles(d, **kw) for d in (dev, orc)]
        assert_same(*res, f"tile {tile} warps {warps}")
    finally:
        dev.close()


def test_per_draw_launch_mode_matches(orc):
    dev = W.Device(launch_mode=W.LaunchMode.PER_DRAW)
    try:
        res = [scenes.render_scene(d, wl.scene_textured_icosphere, width=320, height=180, level=3, tex_size=64)
               for d in (dev, orc)]
        assert_same(*res, "per-draw mode")
    finally:
        dev.close()


def test_tiny_bins_force_retry(orc):
    """A bin capacity far too small makes the first launch run out of scratch; the worker
    grows it and re-runs, with the same result."""
    dev = W.Device(bin_capacity=64)
    try:
        res = [scenes.render_scene(d, wl.scene_colored_sphere, width=200, height=200) for d in (dev, orc)]
        assert_same(*res, "bin retry")
    finally:
        dev.close()


def test_blended_quads_f16(gpu_ext, orc_ext):
    """Extension profile: Rgba16Float + ALPHA_BLENDING in painter order."""
    kw = dict(width=320, height=192, n_quads=300, size_lo=8, size_hi=160)
    (cg, _, ng), (co, _, no) = [scenes.render_scene(d, wl.scene_blended_quads, **kw) for d in (gpu_ext, orc_ext)]
    assert ng == no
    # bit-exact: every blend step rounds like the oracle's scalar f32 arithmetic and f16 encode
    assert np.array_equal(cg.view(np.uint16), co.view(np.uint16))


def test_blend_kernel_equals_generic_path(gpu_ext):
    """The specialised Rgba16Float blend raster (packed f32x2 arithmetic) must give the bits of
    the generic fragment path: the same scene with an Always, never-written depth target takes
    the generic path and must not change a single colour bit."""
    kw = dict(width=640, height=360, n_quads=600, size_lo=4, size_hi=300)
    cs, _, ns = scenes.render_scene(gpu_ext, wl.scene_blended_quads, **kw)
    cg, _, ng = scenes.render_scene(gpu_ext, wl.scene_blended_quads, depth_always=True, **kw)
    assert ns == ng
    assert np.array_equal(cs.view(np.uint16), cg.view(np.uint16))


@pytest.mark.parametrize("side,uv_scale,srgb,mode,mag,min_,mip,fmt", [
    (64, 1.0, False, W.AddressMode.REPEAT, 1, 1, 1, W.TextureFormat.RGBA8_UNORM),
    (48, 1.0, True, W.AddressMode.REPEAT, 1, 1, 1, W.TextureFormat.RGBA8_UNORM_SRGB),
    (32, 2.0, False, W.AddressMode.MIRROR_REPEAT, 1, 1, 1, W.TextureFormat.RGBA8_UNORM),
    (100, 1.5, True, W.AddressMode.CLAMP_TO_EDGE, 1, 0, 1, W.TextureFormat.RGBA8_UNORM_SRGB),
    (90, 1.3, False, W.AddressMode.REPEAT, 0, 0, 0, W.TextureFormat.BGRA8_UNORM_SRGB),
    (512, 1.0, True, W.AddressMode.REPEAT, 1, 1, 1, W.TextureFormat.RGBA8_UNORM_SRGB),
    (7, 9.0, True, W.AddressMode.MIRROR_REPEAT, 1, 1, 1, W.TextureFormat.RGBA8_UNORM),  # LOD past the last mip
])
def test_textured_quad_sampling_ext(gpu_ext, orc_ext, side, uv_scale, srgb, mode, mag, min_, mip, fmt):
    """Extension-profile sampling (sRGB decode, LOD from the record's derivatives, nearest /
    bilinear / trilinear, address modes) and sRGB target encoding, bit for bit with the oracle."""
    levels = wl.mip_chain(wl.checker_noise_texture(256, 7))
    kw = dict(srgb_texture=srgb, address=mode, mag=mag, min_=min_, mip=mip, color_format=fmt, uv_scale=uv_scale,
              clear=(0.2, 0.1, 0.05, 1.0))
    (cg, ng), (co, no) = [scenes.textured_quad(d, 600, 560, 17, 9, side, levels, **kw) for d in (gpu_ext, orc_ext)]
    assert ng == no
    assert np.array_equal(cg, co), f"{(cg != co).any(-1).sum()} pixels differ"


@pytest.mark.parametrize("order", [W.RasterOrder.AUTO, W.RasterOrder.ORDERED])
def test_textured_icosphere_filtered_ext(orc_ext, order):
    """The textured configuration as the extension profile renders it: Rgba8UnormSrgb texture with
    a full mip chain, linear min/mag/mip filtering, repeat, into an Rgba8UnormSrgb target with
    Depth32Float Less — through the visibility raster and through the ordered raster."""
    dev = W.Device(profile=W.Profile.EXTENSION, raster_order=order)
    try:
        kw = dict(width=480, height=272, level=4, tex_size=256, filtering=True, srgb=True)
        res = [scenes.render_scene(d, wl.scene_textured_icosphere, **kw) for d in (dev, orc_ext)]
        assert_same(*res, "filtered textured icosphere")
    finally:
        dev.close()


def test_srgb_target_blending_ext(gpu_ext, orc_ext):
    """Alpha blending into an Rgba8UnormSrgb target in the extension profile: the destination is
    decoded to linear, blended, and encoded back."""
    kw = dict(n_tris=300, width=200, height=150, seed=11, color_format=W.TextureFormat.RGBA8_UNORM_SRGB,
              blend=W.BlendState.alpha_blending())
    assert_same(scenes.random_clip_triangles(gpu_ext, **kw), scenes.random_clip_triangles(orc_ext, **kw), "srgb blend")


@pytest.fixture(scope="module", params=[W.RasterOrder.AUTO, W.RasterOrder.ORDERED], ids=["auto", "ordered"])
def gpu_edge(request):
    d = W.Device(profile=W.Profile.EXTENSION, raster_rule=W.RasterRule.EDGE, raster_order=request.param)
    yield d
    d.close()


@pytest.fixture(scope="module")
def orc_edge():
    return oracle_device.device(profile=W.Profile.EXTENSION, threads=8, raster_rule=W.RasterRule.EDGE)


def test_edge_rule_coverage(gpu_edge, orc_edge):
    """Edge-function rule: hand-placed triangles with edges through pixel centres, random
    triangles, and a mesh tiling a rectangle (each centre once), counted by additive blending."""
    rng = np.random.default_rng(5)
    tris = [[(10.5, 10.5), (20.5, 10.5), (10.5, 20.5)], [(20.5, 10.5), (20.5, 20.5), (10.5, 20.5)]]
    for _ in range(200):
        pts = rng.uniform([0, 0], [128, 64], (3, 2))
        grid = 2 if rng.random() < 0.3 else 256  # half-pixel corners put edges through centres
        pts = np.round(pts * grid) / grid
        tris.append([tuple(p) for p in pts])
    res = [scenes.coverage_counts(d, 128, 64, tris) for d in (gpu_edge, orc_edge)]
    assert res[0][1] == res[1][1]
    assert np.array_equal(res[0][0], res[1][0])


@pytest.mark.parametrize("depth,blend", [(W.CompareFunction.LESS, None), (None, "alpha"),
                                         (W.CompareFunction.GREATER_EQUAL, None)])
def test_edge_rule_clipped_triangles(gpu_edge, orc_edge, depth, blend):
    """Random clip-space triangles crossing every plane (sub-triangles, composed barycentrics) under
    the edge rule: colour, depth and fragment counts bit for bit."""
    kw = dict(n_tris=400, width=256, height=192, seed=17, depth=depth,
              blend=W.BlendState.alpha_blending() if blend else None)
    assert_same(scenes.random_clip_triangles(gpu_edge, **kw), scenes.random_clip_triangles(orc_edge, **kw), "edge")


def test_edge_rule_textured_and_blended(gpu_edge, orc_edge):
    kw = dict(width=480, height=272, level=4, tex_size=256, filtering=True, srgb=True)
    res = [scenes.render_scene(d, wl.scene_textured_icosphere, **kw) for d in (gpu_edge, orc_edge)]
    assert_same(*res, "edge textured")
    kw = dict(width=320, height=192, n_quads=300, size_lo=8, size_hi=160)
    (cg, _, ng), (co, _, no) = [scenes.render_scene(d, wl.scene_blended_quads, **kw) for d in (gpu_edge, orc_edge)]
    assert ng == no
    assert np.array_equal(cg.view(np.uint16), co.view(np.uint16))


def test_discard_program(gpu, orc):
    def build(dev):
        s = wl.scene_colored_sphere(dev, 200, 160)
        sm = dev.create_shader_module(native="mesh_color_discard")
        pl = dev.create_render_pipeline(
            sm, [W.VertexBufferLayout(24, [W.VertexAttribute(3, 0, 0), W.VertexAttribute(3, 12, 1)])],
            W.PrimitiveState(cull_mode=W.Face.BACK), None, sm, [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
        s.draws[0] = (pl,) + s.draws[0][1:]
        return s
    res = [scenes.render_scene(d, build) for d in (gpu, orc)]
    assert_same(*res, "discard")


def test_division_by_reciprocal_matches_cuda(gpu):
    """The raster kernels divide by a per-record reciprocal with Markstein's correction steps;
    every quotient must carry exactly the bits of CUDA's correctly rounded __fdiv_rn.  The same
    samples check the packed f32x2 helpers and the span rule's binary32 integer division
    (div_trunc_span) against exact integer division."""
    import ctypes

    fn = gpu.lib.cdll.gbr_selftest_division
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_float)]
    mism = ctypes.c_uint64()
    first = (ctypes.c_float * 2)()
    for seed in (1, 2):
        assert fn(1 << 32, seed, ctypes.byref(mism), first) == 0, gpu.lib.error_text()
        assert mism.value == 0, f"{mism.value} mismatches, first a={first[0]!r} b={first[1]!r}"


def test_errors_are_reported(gpu):
    s = wl.scene_colored_sphere(gpu, 64, 64)
    pl, groups, vbs, ib, rng, bv = s.draws[0]
    s.draws[0] = (pl, groups, vbs, ib, range(0, rng.stop + 3), bv)
    with pytest.raises(W.GbrError) as e:
        s.render()
    assert e.value.status == -4
    # the device stays usable after a failed submission
    s2 = wl.scene_colored_sphere(gpu, 64, 64)
    s2.render()


@pytest.mark.parametrize("fmt,n,instances,order", [
    (W.IndexFormat.UINT32, 600, 1, W.RasterOrder.AUTO), (W.IndexFormat.UINT16, 600, 2, W.RasterOrder.AUTO),
    (W.IndexFormat.UINT32, 3000, 1, W.RasterOrder.ORDERED), (W.IndexFormat.UINT16, 2500, 3, W.RasterOrder.ORDERED)])
def test_strip_primitive_restart(orc, fmt, n, instances, order):
    """Triangle strips with separator indices (primitive.rs:428-487): every run restarts its own
    strip (winding parity included), runs shorter than three yield nothing."""
    dev = W.Device(raster_order=order)
    try:
        kw = dict(n_indices=n, width=160, height=120, seed=n + instances, index_format=fmt, instances=instances)
        res = [scenes.restart_strips(d, **kw) for d in (dev, orc)]
        assert_same(*res, f"restart {fmt} n={n}")
        assert res[0][2] > 0
    finally:
        dev.close()


@pytest.mark.parametrize("topology,fmt,restart,instances,scissor", [
    (W.PrimitiveTopology.LINE_LIST, None, False, 1, None),
    (W.PrimitiveTopology.LINE_LIST, W.IndexFormat.UINT32, False, 2, (13, 7, 150, 100)),
    (W.PrimitiveTopology.LINE_STRIP, None, False, 1, None),
    (W.PrimitiveTopology.LINE_STRIP, W.IndexFormat.UINT16, True, 2, None),
    (W.PrimitiveTopology.LINE_STRIP, W.IndexFormat.UINT32, True, 1, (0, 20, 120, 80)),
    (W.PrimitiveTopology.POINT_LIST, None, False, 3, None),
    (W.PrimitiveTopology.POINT_LIST, W.IndexFormat.UINT16, False, 1, (5, 5, 100, 90)),
])
def test_lines_and_points(gpu, orc, topology, fmt, restart, instances, scissor):
    """LineRasterizer (Cohen–Sutherland clip, Bresenham without the end point, t accumulated by
    1/dx) and PointRasterizer, fragments in primitive order (raster.rs:197-265)."""
    kw = dict(n=400, width=180, height=130, seed=31 + topology, index_format=fmt, restart=restart,
              instances=instances, scissor=scissor)
    res = [scenes.lines_points(d, topology, **kw) for d in (gpu, orc)]
    assert_same(*res, f"topology {topology} fmt {fmt} restart {restart}")
    assert res[0][2] > 0


def test_mixed_topologies_in_one_pass(gpu, orc):
    res = [scenes.mixed_pass(d, 200, 150, 5) for d in (gpu, orc)]
    assert_same(*res, "triangles, lines, points, triangles")
