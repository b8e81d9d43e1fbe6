"""WGSL translator on the host (no GPU): every test program translates; the operator, structural
and render programs compile with NVRTC for sm_103a; unsupported features and malformed sources
come back as status codes, never as crashes."""

import pytest

import wgsl_programs as P
from wgpu_gb300 import _abi as A
from wgpu_gb300 import api as W


@pytest.fixture(scope="module")
def lib():
    return W.gpu_lib()


RENDER = [(P.TRIANGLE, "vmain", "fmain"), (P.MESH_COLOR, "vmain", "fmain"), (P.MESH_COLOR_DISCARD, "vmain", "fmain"),
          (P.TEX_LAMBERT, "vmain", "fmain")]


def test_operator_program_translates(lib):
    src, kats = P.ops_program()
    assert len(kats) >= 40
    code = W.wgsl_translate(lib, src, "main")
    assert "jit_vs" in code and "return 0; }" in code  # a stub fragment stage
    assert code.count("case ") >= len(kats)


def test_structural_program_translates(lib):
    src, recs = P.structural_program()
    assert len(recs) >= 29
    code = W.wgsl_translate(lib, src, "main")
    assert "fn_v_t_loop" in code


@pytest.mark.parametrize("src,vs,fs", RENDER)
def test_render_programs_translate(lib, src, vs, fs):
    code = W.wgsl_translate(lib, src, vs, fs)
    assert "jit_vs" in code and "jit_fs" in code


def test_matrix_product_is_the_column_sum(lib):
    code = W.wgsl_translate(lib, P.MESH_COLOR, "vmain", "fmain")
    assert "w_mulmv(" in code  # ((v0*c0 + v1*c1) + v2*c2) + v3*c3, wgsl_rt.cuh


@pytest.mark.parametrize("which", ["ops", "structural", "tex_lambert"])
def test_programs_compile_with_nvrtc(lib, which):
    why = None
    if which == "ops":
        src, vs, fs = P.ops_program()[0], "main", None
    elif which == "structural":
        src, vs, fs = P.structural_program()[0], "main", None
    else:
        src, vs, fs = P.TEX_LAMBERT, "vmain", "fmain"
    try:
        W.wgsl_compile_check(lib, src, vs, fs)
    except W.GbrError as e:
        why = str(e)
    assert why is None, why


@pytest.mark.parametrize("body,status", [
    ("let d = dot(vec3f(1.0, 0.0, 0.0), vec3f(0.0, 1.0, 0.0));", A.ERR_UNSUPPORTED),   # math builtins
    ("var m = mat4x4f(); let q = m * m;", A.ERR_UNSUPPORTED),                          # matrix * matrix
    ("let q = undefined_name + 1;", -7),                                                # unknown identifier
    ("let q: f32 = true;", -7),                                                         # type mismatch
])
def test_errors_are_status_codes(lib, body, status):
    src = ("@vertex fn main(@builtin(vertex_index) vi: u32) -> @builtin(position) vec4f {\n  " + body +
           "\n  return vec4f(0.0, 0.0, 0.0, 1.0);\n}\n")
    with pytest.raises(W.GbrError) as e:
        W.wgsl_translate(lib, src, "main")
    assert e.value.status == status, str(e.value)


def test_parse_error(lib):
    with pytest.raises(W.GbrError) as e:
        W.wgsl_translate(lib, "@vertex fn main( -> { }", "main")
    assert e.value.status == -7


# Attributes, interpolation and overrides: what the front end cannot honour fails the module
# instead of being dropped.
VS_HEAD = "struct V { @builtin(position) p: vec4f, %s };\n"
VS_FN = ("@vertex fn vmain(@builtin(vertex_index) vi: u32) -> V {\n  var o: V;\n  o.p = vec4f(0.0, 0.0, 0.0, 1.0);\n"
         "  %s\n  return o;\n}\n")
FS_FN = "%s@fragment fn fmain(%s) -> @location(0) vec4f {\n  return vec4f(%s);\n}\n"


def program(member, assign, fs_attr, fs_param, fs_value):
    return VS_HEAD % member + VS_FN % assign + FS_FN % (fs_attr, fs_param, fs_value)


@pytest.mark.parametrize("src,status", [
    # an attribute nobody knows
    (program("@location(0) c: f32", "o.c = 1.0;", "@foo ", "@location(0) c: f32", "c, 0.0, 0.0, 1.0"), -7),
    # layout attributes the uniform loader would not honour
    ("struct U { @align(16) a: f32 };\n" + program("@location(0) c: f32", "o.c = 1.0;", "", "@location(0) c: f32",
                                                   "c, 0.0, 0.0, 1.0"), A.ERR_UNSUPPORTED),
    # integer inter-stage values must be flat (naga validation; the reference panics otherwise)
    (program("@location(0) @interpolate(linear) i: u32", "o.i = vi;", "",
             "@location(0) @interpolate(linear) i: u32", "f32(i), 0.0, 0.0, 1.0"), -7),
    # a sampling that does not fit the interpolation type
    (program("@location(0) @interpolate(flat, center) c: f32", "o.c = 1.0;", "",
             "@location(0) @interpolate(flat, center) c: f32", "c, 0.0, 0.0, 1.0"), -7),
    # @early_depth_test on a vertex entry point, and with an unknown argument
    (program("@location(0) c: f32", "o.c = 1.0;", "", "@location(0) c: f32",
             "c, 0.0, 0.0, 1.0").replace("@vertex fn", "@early_depth_test(force) @vertex fn"), -7),
    # attributes on declarations that take none
    ("@group(0) " + program("@location(0) c: f32", "o.c = 1.0;", "", "@location(0) c: f32", "c, 0.0, 0.0, 1.0"), -7),
    ("@location(1) const q = 1.0;\n" + program("@location(0) c: f32", "o.c = q;", "", "@location(0) c: f32",
                                                 "c, 0.0, 0.0, 1.0"), -7),
    (program("@location(0) c: f32", "o.c = 1.0;", "@early_depth_test(sometimes) ", "@location(0) c: f32",
             "c, 0.0, 0.0, 1.0"), -7),
    # an override with neither a pipeline value nor an initializer
    ("@id(3) override k: f32;\n" + program("@location(0) c: f32", "o.c = k;", "", "@location(0) c: f32",
                                           "c, 0.0, 0.0, 1.0"), -7),
])
def test_unhonoured_attributes_fail(lib, src, status):
    with pytest.raises(W.GbrError) as e:
        W.wgsl_translate(lib, src, "vmain", "fmain")
    assert e.value.status == status, str(e.value)


def test_flat_and_early_depth_translate(lib):
    """Integer flat values travel as bits (no arithmetic); integers default to flat, floats to
    perspective; @early_depth_test(force) is accepted on the fragment entry point."""
    src = program("@location(0) i: u32, @location(1) @interpolate(flat, either) c: vec2f",
                  "o.i = vi;\n  o.c = vec2f(1.0, 2.0);", "@early_depth_test(force) ",
                  "@location(0) i: u32, @location(1) @interpolate(flat) c: vec2f", "f32(i), c.x, c.y, 1.0")
    code = W.wgsl_translate(lib, src, "vmain", "fmain")
    assert "__uint_as_float" in code and "__float_as_uint" in code


def test_override_initializer_is_used_without_a_pipeline_value(lib):
    src = ("override k: f32 = 0.25;\n" +
           program("@location(0) @interpolate(linear) c: f32", "o.c = k;", "",
                   "@location(0) @interpolate(linear) c: f32", "c, 0.0, 0.0, 1.0"))
    code = W.wgsl_translate(lib, src, "vmain", "fmain")
    assert "g_v_k" in code
