"""Fragment-stage features of the reference, on the GPU against the oracle, bit for bit:

* flat interpolation (render_pass/fragment.rs:286-302, 395-405): the first vertex of the
  unclipped primitive, for float values and for integer values carried bit for bit (the integer
  program's id is a NaN pattern as an f32, so any arithmetic on it would show);
* @early_depth_test (fragment.rs:83-86, 166-194): Force tests (and writes) depth before the
  fragment stage and skips the late test; Allow tests before and again at the colour output;
  a discard after the early test keeps the depth it wrote;
* perspective-correct interpolation (extension profile; the reference has todo!() there,
  fragment.rs:343-345) on triangles the near plane clips;
* the same features written in WGSL (flat u32 varyings, @early_depth_test, pipeline-overridable
  constants), compared with the native programs.

Both raster paths run: the visibility raster (depth-tested opaque batches) and the ordered walk.
"""

import numpy as np
import pytest

import oracle_device
import scenes
from wgpu_gb300 import api as W

pytestmark = pytest.mark.gpu

T = W.PrimitiveTopology
CF = W.CompareFunction


@pytest.fixture(scope="module")
def gpu():
    d = W.Device()
    yield d
    d.close()


@pytest.fixture(scope="module")
def gpu_ordered():
    d = W.Device(raster_order=W.RasterOrder.ORDERED)
    yield d
    d.close()


@pytest.fixture(scope="module")
def orc():
    return oracle_device.device(threads=8)


def assert_same(a, b, what=""):
    (ca, da, na), (cb, db, nb) = a, b
    diff = (ca != cb).any(-1)
    assert not diff.any(), f"{what}: {int(diff.sum())} colour pixels differ, first at {np.argwhere(diff)[:3].tolist()}"
    if da is not None or db is not None:
        dd = da.view(np.uint32) != db.view(np.uint32)
        assert not dd.any(), f"{what}: {int(dd.sum())} depth values differ"
    assert na == nb, f"{what}: fragments {na} vs {nb}"


@pytest.mark.parametrize("program", ["clip_flat", "clip_flat_id"])
@pytest.mark.parametrize("depth", [None, CF.LESS])
@pytest.mark.parametrize("topology", [T.TRIANGLE_LIST, T.TRIANGLE_STRIP])
def test_flat_interpolation(gpu, gpu_ordered, orc, program, depth, topology):
    kw = dict(n_tris=300, width=160, height=120, seed=11, program=program, depth=depth, topology=topology)
    ref = scenes.random_clip_triangles(orc, **kw)
    assert ref[2] > 1000
    for dev, what in ((gpu, "auto"), (gpu_ordered, "ordered")):
        assert_same(scenes.random_clip_triangles(dev, **kw), ref, f"{program} {what}")


@pytest.mark.parametrize("program", ["clip_flat", "clip_flat_id", "clip_flat_id@early_allow"])
@pytest.mark.parametrize("topology", [T.LINE_LIST, T.LINE_STRIP, T.POINT_LIST])
def test_flat_lines_and_points(gpu, orc, program, topology):
    kw = dict(topology=topology, n=120, width=96, height=80, seed=5, program=program)
    assert_same(scenes.lines_points(gpu, **kw), scenes.lines_points(orc, **kw), f"{program} topology {topology}")


EARLY = ["clip_passthrough@early_force", "clip_passthrough@early_allow", "clip_discard@early_force",
         "clip_discard@early_allow", "clip_discard", "clip_flat_id@early_force"]


@pytest.mark.parametrize("program", EARLY)
@pytest.mark.parametrize("compare,write", [(CF.LESS, True), (CF.LESS_EQUAL, True), (CF.GREATER, True),
                                           (CF.LESS, False), (CF.ALWAYS, True)])
def test_early_depth_test(gpu, orc, program, compare, write):
    """Colour, depth and the fragment count as the oracle; and the fragment-stage runs (the early
    test skips the stage for rejected fragments) as the oracle counts them."""
    kw = dict(n_tris=300, width=160, height=120, seed=21, program=program, depth=compare, depth_write=write)
    sg, so = [], []
    got = scenes.random_clip_triangles(gpu, **kw, stats=sg)
    ref = scenes.random_clip_triangles(orc, **kw, stats=so)
    assert_same(got, ref, f"{program} compare {compare} write {write}")
    assert sg[0].fs_invocations == so[0].fs_invocations, (sg[0].fs_invocations, so[0].fs_invocations)
    if compare != CF.ALWAYS and "@early" in program:
        assert so[0].fs_invocations < so[0].fragments_shaded  # the early test rejected some


def test_early_allow_with_less_writes_depth_but_no_colour(orc):
    """Allow + Less + depth writes: the early test stores z, the late test compares z < z and
    fails, so no colour lands — exactly what the reference does (fragment.rs:176-181, 470-479)."""
    kw = dict(n_tris=60, width=64, height=48, seed=3, depth=CF.LESS, clear=(0.1, 0.2, 0.3, 1.0))
    col, dep, n = scenes.random_clip_triangles(orc, program="clip_passthrough@early_allow", **kw)
    col0, dep0, _ = scenes.random_clip_triangles(orc, program="clip_passthrough", **kw)
    assert n > 0
    assert (col == col[0, 0]).all()  # the clear colour everywhere
    assert np.array_equal(dep.view(np.uint32), dep0.view(np.uint32))


@pytest.mark.parametrize("program", ["clip_passthrough@early_force", "clip_discard@early_allow"])
@pytest.mark.parametrize("topology", [T.LINE_STRIP, T.POINT_LIST])
def test_early_depth_lines_and_points(gpu, orc, program, topology):
    kw = dict(topology=topology, n=150, width=96, height=80, seed=8, program=program, depth=CF.LESS)
    assert_same(scenes.lines_points(gpu, **kw), scenes.lines_points(orc, **kw), f"{program} topology {topology}")


@pytest.mark.parametrize("depth", [CF.LESS, None])
@pytest.mark.parametrize("order", [W.RasterOrder.AUTO, W.RasterOrder.ORDERED])
def test_perspective_interpolation_clipped(depth, order):
    """Perspective-correct interpolation (extension profile) on a sphere the near plane cuts."""
    gpu = W.Device(profile=W.Profile.EXTENSION, raster_order=order)
    orc = oracle_device.device(profile=W.Profile.EXTENSION, threads=8)
    try:
        got, st = scenes.perspective_sphere(gpu, 240, 180, depth=depth)
        ref, _ = scenes.perspective_sphere(orc, 240, 180, depth=depth)
    finally:
        gpu.close()
        orc.close()
    assert st.generic_setup_prims > 0  # clipped triangles took the generic (clipping) setup
    assert_same(got, ref, f"perspective depth={depth} order={order}")
    assert ref[2] > 10000


# ------------------------------------------------------------------------------------ WGSL
FLAT_ID_WGSL = """
struct VOut {
    @builtin(position) pos: vec4f,
    @location(0) @interpolate(flat) id: u32,
    @location(1) @interpolate(linear) col: vec3f,
};

@vertex
fn vmain(@builtin(vertex_index) vi: u32, @location(0) p: vec4f, @location(1) c: vec4f) -> VOut {
    var o: VOut;
    o.pos = p;
    o.id = 0x7fc00000u | (vi & 0xffffu);
    o.col = c.xyz;
    return o;
}

@early_depth_test(force)
@fragment
fn fmain(@location(0) @interpolate(flat) id: u32, @location(1) @interpolate(linear) col: vec3f) -> @location(0) vec4f {
    return vec4f(f32(id & 0xffu) / 255.0, col.x, col.y, 1.0);
}
"""

CLIP_LAYOUT = [W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 0)]),
               W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 1)])]


def wgsl_clip_triangles(dev, src, n_tris, width, height, seed, depth, constants=None):
    """random_clip_triangles' geometry drawn with a WGSL program (vmain / fmain)."""
    rng = np.random.default_rng(seed)
    nv = n_tris * 3
    w = rng.uniform(0.3, 2.0, nv)
    pos = np.stack([rng.uniform(-1.6, 1.6, nv) * w, rng.uniform(-1.6, 1.6, nv) * w,
                    rng.uniform(-0.3, 1.3, nv) * w, w], 1).astype(np.float32)
    col = rng.uniform(0, 1, (nv, 4)).astype(np.float32)
    sm = dev.create_shader_module(wgsl=src)
    pl = dev.create_render_pipeline(sm, CLIP_LAYOUT, W.PrimitiveState(), W.DepthStencilState(True, depth), sm,
                                    [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)], vertex_entry_point="vmain",
                                    fragment_entry_point="fmain", vertex_constants=constants,
                                    fragment_constants=constants)
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM)
    dtex = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT)
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, (0.1, 0.2, 0.3, 1.0))],
                               W.RenderPassDepthStencilAttachment(dtex, 0.75))
    rp.set_pipeline(pl)
    rp.set_vertex_buffer(0, dev.create_buffer_init(pos))
    rp.set_vertex_buffer(1, dev.create_buffer_init(col))
    rp.draw(range(0, nv))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    return dev.read_texture(color), dev.read_texture(dtex), dev.submission_stats(sub).fragments_shaded


def test_wgsl_flat_integer_and_early_depth(gpu, orc):
    """The WGSL program equals the native clip_flat_id with @early_depth_test(force), which
    equals the oracle."""
    got = wgsl_clip_triangles(gpu, FLAT_ID_WGSL, 300, 160, 120, 21, CF.LESS)
    kw = dict(n_tris=300, width=160, height=120, seed=21, program="clip_flat_id@early_force", depth=CF.LESS)
    assert_same(got, scenes.random_clip_triangles(orc, **kw), "WGSL flat id + early depth vs oracle")


OVERRIDE_WGSL = """
@id(7) override red_scale: f32 = 1.0;
override keep_green: bool = true;
override blue_shift: u32;
override bias = 0.0;

struct VOut {
    @builtin(position) pos: vec4f,
    @location(0) @interpolate(linear) col: vec4f,
};

@vertex
fn vmain(@location(0) p: vec4f, @location(1) c: vec4f) -> VOut {
    var o: VOut;
    o.pos = p;
    o.col = c;
    return o;
}

@fragment
fn fmain(@location(0) @interpolate(linear) col: vec4f) -> @location(0) vec4f {
    let g = select(0.0, col.y, keep_green);
    let b = f32((u32(col.z * 255.0) >> blue_shift)) / 255.0;
    return vec4f(col.x * red_scale + bias, g, b, 1.0);
}
"""

LITERAL_WGSL = OVERRIDE_WGSL.replace("@id(7) override red_scale: f32 = 1.0;", "const red_scale: f32 = 0.3;") \
    .replace("override keep_green: bool = true;", "const keep_green: bool = false;") \
    .replace("override blue_shift: u32;", "const blue_shift: u32 = 2u;") \
    .replace("override bias = 0.0;", "const bias = 0.0;")


def test_wgsl_pipeline_overridable_constants(gpu):
    """Overrides take the pipeline's constants (by @id and by name; 2.7 truncates to 2u for the
    u32, 0.3 rounds to the nearest f32) and the initializers otherwise: the frame equals the
    same program with those values written as constants."""
    consts = {"7": 0.3, "keep_green": 0.0, "blue_shift": 2.7}
    got = wgsl_clip_triangles(gpu, OVERRIDE_WGSL, 200, 128, 96, 4, CF.LESS, constants=consts)
    want = wgsl_clip_triangles(gpu, LITERAL_WGSL, 200, 128, 96, 4, CF.LESS)
    assert_same(got, want, "overrides vs literals")
    assert got[2] > 1000


@pytest.mark.parametrize("consts,status", [({"7": 0.3}, -7),                       # blue_shift has no value
                                           ({"blue_shift": -1.0}, -7),             # out of range for u32
                                           ({"blue_shift": 1.0, "7": float("inf")}, -7)])  # not finite
def test_wgsl_override_errors(gpu, consts, status):
    sm = gpu.create_shader_module(wgsl=OVERRIDE_WGSL)
    with pytest.raises(W.GbrError) as e:
        gpu.create_render_pipeline(sm, CLIP_LAYOUT, W.PrimitiveState(), None, sm,
                                   [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)], vertex_entry_point="vmain",
                                   fragment_entry_point="fmain", vertex_constants=consts, fragment_constants=consts)
    assert e.value.status == status, str(e.value)
