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
