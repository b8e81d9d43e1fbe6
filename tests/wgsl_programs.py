"""WGSL programs of the shader tests, written for this project.

* `ops_program(kats)`: one vertex program whose vertex `i` evaluates operator vector `i` of the
  reference's naga-cranelift tests (casts, scalar binops, comparisons, unops; the vectors come
  from tests/golden/reference_kats.json with their file:line) and writes 1 when the result
  equals the expected value exactly.
* `STRUCTURAL`: programs exercising what naga-cranelift's structural tests exercise (control
  flow, calls, constants, private globals, composite access, matrices), each a function
  returning a value compared with the expected output recorded from those tests;
  `structural_program()` joins them into one vertex program switched on the vertex index.
* Render programs equal, operation for operation, to the library's native programs, for
  frame-level parity of the translator.
"""

from __future__ import annotations

import json
import os

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def _lit(value: str, ty: str) -> str:
    if ty == "bool":
        return value
    if ty == "f32":
        return value if ("." in value or "e" in value) else value + ".0"
    return value


def ops_program(kats=None) -> tuple[str, list]:
    kats = kats if kats is not None else KATS["shader_ops"]
    cases = []
    for i, k in enumerate(kats):
        if k["kind"] == "cast":
            body = (f"var a: {k['from']} = {_lit(k['value'], k['from'])};\n"
                    f"      let c: {k['to']} = {k['to']}(a);\n"
                    f"      ok = u32(c == {_lit(k['expected'], k['to'])});")
        elif k["kind"] == "binop":
            t = k["type"]
            exp = k["expected"]
            e = repr(float(exp)) if t == "f32" else str(int(exp))
            body = (f"var a: {t} = {_lit(k['left'], t)};\n      var b: {t} = {_lit(k['right'], t)};\n"
                    f"      let c: {t} = a {k['op']} b;\n      ok = u32(c == {e});")
        elif k["kind"] == "compare":
            t = k["type"]
            body = (f"var a: {t} = {_lit(k['left'], t)};\n      var b: {t} = {_lit(k['right'], t)};\n"
                    f"      ok = u32((a {k['op']} b) == {'true' if k['expected'] else 'false'});")
        else:  # unop
            t = k["type"]
            if t == "bool":
                body = (f"var a: bool = {k['input']};\n"
                        f"      ok = u32(({k['op']} a) == {'true' if k['expected'] else 'false'});")
            else:
                exp = k["expected"]
                e = repr(float(exp)) if t == "f32" else (f"{int(exp)}u" if t == "u32" else str(int(exp)))
                body = f"var a: {t} = {_lit(k['input'], t)};\n      let c: {t} = {k['op']} a;\n      ok = u32(c == {e});"
        cases.append(f"    case {i}u: {{\n      {body}\n    }}")
    src = (
        "struct Probe {\n  @builtin(position) pos: vec4f,\n  @location(0) ok: u32,\n}\n\n"
        "@vertex\nfn main(@builtin(vertex_index) vi: u32) -> Probe {\n  var ok: u32 = 7u;\n  switch vi {\n"
        + "\n".join(cases) + "\n    default: {\n      ok = 9u;\n    }\n  }\n"
        "  return Probe(vec4f(0.0, 0.0, 0.0, 1.0), ok);\n}\n")
    return src, kats


# name -> (helper declarations, expression of the case, result type)
STRUCTURAL = {
    "init_variable": ("", "t_init()", "fn t_init() -> u32 { var a: u32 = 123; return a; }"),
    "store_variable": ("", "t_store()", "fn t_store() -> u32 { var a: u32; a = 123u; return a; }"),
    "early_return": ("", "t_early()", "fn t_early() -> u32 { return 456u; }"),
    "if_early_return": ("", "t_if_early()",
                        "fn t_if_early() -> u32 { var c: bool = true; if c { return 456u; } return 123u; }"),
    "function_call": ("", "t_call()",
                      "fn add2(x: i32, y: i32) -> i32 { return x + y; }\nfn t_call() -> i32 { let r = add2(13, 12); return r; }"),
    "scalar_constant": ("const twice: i32 = 1234 * 2;", "t_const()", "fn t_const() -> i32 { var v: i32 = twice; return v; }"),
    "vector_constant": ("const four: vec4i = vec4i(1, 2, 3, 4);", "t_vconst()",
                        "fn t_vconst() -> vec4i { var v: vec4i = four; return v; }"),
    "loops": ("", "t_loop()",
              "fn t_loop() -> i32 { var f: i32 = 1; for (var i = 2; i <= 6; i += 1) { f *= i; } return f; }"),
    "switch_case_single": ("", "t_sw(4)", ""),
    "switch_case_multiple": ("", "t_sw(5)", ""),
    "switch_default": ("", "t_sw2(42)", ""),
    "switch_break": ("", "t_sw3(3)", ""),
    "global_variable": ("var<private> pv: vec4i = vec4i(1, 2, 3, 4);", "PRIVATE", ""),
    "access_index_vector_variable_read": ("", "t_vread()",
                                          "fn t_vread() -> i32 { var v = vec4i(1, 2, 3, 4); return v.y; }"),
    "access_index_vector_variable_assign": ("", "t_vassign()",
                                            "fn t_vassign() -> vec4i { var v: vec4i = vec4i(1, 2, 3, 4); v.y = 123; return v; }"),
    "access_index_struct_variable_read": ("struct Pair { a: i32, b: i32, }", "t_sread()",
                                          "fn t_sread() -> i32 { var p = Pair(1, 2); return p.b; }"),
    "access_index_struct_variable_assign": ("", "t_sassign()",
                                            "fn t_sassign() -> vec4i { var p = Pair(1, 2); p.b = 123; return vec4i(p.a, p.b, 0, 0); }"),
    "trap_divide_by_zero": ("", "t_div0()", "fn t_div0() -> i32 { var a: i32 = 123; var b: i32 = 0; var c: i32 = a / b; return c; }"),
    "access_global_variable_array_in_bounds_static": ("var<private> arr: array<i32, 4> = array<i32, 4>(4, 5, 6, 7);",
                                                      "PRIVATE_ARR_STATIC", ""),
    "access_global_variable_array_in_bounds_dynamic": ("", "PRIVATE_ARR_DYNAMIC", ""),
    "select": ("", "t_select(true)", "fn t_select(c: bool) -> i32 { var a = 123; var b = 456; return select(a, b, c); }"),
    "vector_access_dynamic": ("", "t_vdyn()",
                              "fn t_vdyn() -> i32 { var v: vec4i = vec4i(12, 23, 34, 45); var s: i32 = 0;\n"
                              "  for (var i = 0; i < 4; i += 1) { s += (i + 1) * v[i]; } return s; }"),
    "vector_access_static": ("", "t_vstat()",
                             "fn t_vstat() -> i32 { var v: vec4i = vec4i(12, 23, 34, 45); return v.x + 2 * v.y + 3 * v.z + 4 * v.w; }"),
    "vectorized_function_argument": ("", "t_vecarg(vec4i(1, 2, 3, 4))", "fn t_vecarg(q: vec4i) -> i32 { return q.y; }"),
    "return_if_else_diverging": ("", "t_diverge(1234)",
                                 "fn t_diverge(x: i32) -> i32 { if x > 100 { return 45; } else { return 67; } }"),
    "return_from_loop_body_diverging": ("", "t_loopret()", "fn t_loopret() -> i32 { loop { return 45; } return 123; }"),
    "matrix_vector_product": ("", "t_mv()", "MATRIX"),
    "matrix_scalar_product": ("", "t_ms()", "MATRIX_SCALAR"),
    "vector_scalar_product": ("", "t_vs()", "fn t_vs() -> vec4f { var v = vec4f(3, 2, 1, 0); var s: f32 = 2; return v * s; }"),
    "global_matrix_init": ("", "t_gm()", "GLOBAL_MATRIX"),
}
SWITCH_HELPERS = """fn t_sw(a: i32) -> i32 {
  var b: i32;
  switch a {
    case 1: { b = 2; }
    case 2, 3: { b = 3; }
    case 4, 5, 6: { b = 4; }
    default: { b = -1; }
  }
  return b;
}
fn t_sw2(a: i32) -> i32 {
  var b: i32;
  switch a {
    case 1: { b = 2; }
    case 4, 5, 6: { b = 4; }
    default: { b = 3; }
  }
  return b;
}
fn t_sw3(a: i32) -> i32 {
  var b: i32;
  switch a {
    case 1: { b = 2; }
    case 2, 3: { b = 3; break; }
    default: { b = 12; }
  }
  return b;
}
"""
SKIPPED = {"array_length": "runtime-sized arrays in storage buffers (no storage bindings on the render path)"}


def structural_program() -> tuple[str, list]:
    records = [r for r in KATS["shader_programs"] if r["test"] in STRUCTURAL]
    decls, fns, cases = [SWITCH_HELPERS], [], []
    for i, r in enumerate(records):
        d, expr, fn = STRUCTURAL[r["test"]]
        if fn in ("MATRIX", "GLOBAL_MATRIX", "MATRIX_SCALAR"):
            # the recorded input columns and vector of the test
            lits = r["vec4_literals"]
            cols = ", ".join("vec4f(" + ", ".join(repr(x) for x in c) + ")" for c in lits[:4])
            vec = "vec4f(" + ", ".join(repr(x) for x in lits[4]) + ")" if len(lits) > 4 else ""
            if fn == "MATRIX_SCALAR":  # the last column of the matrix times 2
                fn = f"fn t_ms() -> vec4f {{ var m = mat4x4f({cols});\n  var s: f32 = 2; let r = m * s; return r[3]; }}"
            elif fn == "MATRIX":
                fn = f"fn t_mv() -> vec4f {{ var m = mat4x4f({cols});\n  var v = {vec}; return m * v; }}"
            else:
                d = f"const gm: mat4x4f = mat4x4f({cols});"
                fn = f"fn t_gm() -> vec4f {{ var v = {vec}; return gm * v; }}"
        if d:
            decls.append(d)
        if fn:
            fns.append(fn)
        exp = r["expected"][0]
        if expr == "PRIVATE":
            stmt = "pv.y = 123;\n      ok = u32(all4(pv == vec4i(1, 123, 3, 4)));"
        elif expr == "PRIVATE_ARR_STATIC":
            stmt = "var o = arr[2];\n      ok = u32(o == 6);"
        elif expr == "PRIVATE_ARR_DYNAMIC":
            stmt = "var o = 0;\n      for (var i = 0; i < 4; i += 1) { o += arr[i]; }\n      ok = u32(o == 22);"
        elif exp == "DivisionByZero":
            stmt = f"let r = {expr};\n      ok = 5u;"
        elif isinstance(exp, list):
            is_f = any(x != int(x) for x in exp) or "f" in expr or r["test"].startswith(("matrix", "vector_scalar", "global_matrix"))
            vec = ("vec4f(" + ", ".join(repr(float(x)) for x in exp) + ")") if is_f else \
                  ("vec4i(" + ", ".join(str(int(x)) for x in exp) + ")")
            stmt = f"let r = {expr};\n      ok = u32(all4(r == {vec}));"
        else:
            stmt = f"let r = {expr};\n      ok = u32(r == {int(exp)});"
        cases.append(f"    case {i}u: {{\n      {stmt}\n    }}")
    # the second select vector (condition false)
    records.append({"test": "select(false)", "expected": [123.0], "source": "select"})
    cases.append(f"    case {len(records) - 1}u: {{\n      let r = t_select(false);\n      ok = u32(r == 123);\n    }}")
    helpers = ("fn all4(b: vec4<bool>) -> bool { return b.x && b.y && b.z && b.w; }\n")
    src = ("struct Probe {\n  @builtin(position) pos: vec4f,\n  @location(0) ok: u32,\n}\n\n" + "\n".join(decls) + "\n"
           + helpers + "\n".join(fns) + "\n\n@vertex\nfn main(@builtin(vertex_index) vi: u32) -> Probe {\n"
           "  var ok: u32 = 7u;\n  switch vi {\n" + "\n".join(cases) +
           "\n    default: {\n      ok = 9u;\n    }\n  }\n  return Probe(vec4f(0.0, 0.0, 0.0, 1.0), ok);\n}\n")
    return src, records


# ---------------------------------------------------------------- render programs
# Same operations, in the same order, as the native programs of csrc/programs.cuh.
TRIANGLE = """
struct VsIn { @builtin(vertex_index) index: u32, }
struct Varyings {
  @builtin(position) clip: vec4f,
  @location(0) @interpolate(linear) rgba: vec4f,
}
@vertex
fn vmain(inp: VsIn) -> Varyings {
  let k = inp.index % 3;
  let px = f32(i32(k) - 1);
  let py = f32(i32(k & 1u) * 2 - 1);
  return Varyings(vec4f(px, py, 0.0, 1.0), vec4f(f32(k == 0), f32(k == 1), f32(k == 2), 1.0));
}
@fragment
fn fmain(v: Varyings) -> @location(0) vec4f {
  return v.rgba;
}
"""

MESH_COLOR = """
struct Camera { mvp: mat4x4f, }
@group(0) @binding(0) var<uniform> cam: Camera;
struct VsOut {
  @builtin(position) clip: vec4f,
  @location(0) @interpolate(linear) col: vec3f,
}
@vertex
fn vmain(@location(0) p: vec3f, @location(1) c: vec3f) -> VsOut {
  var o: VsOut;
  o.clip = cam.mvp * vec4f(p.x, p.y, p.z, 1.0);
  o.col = c;
  return o;
}
@fragment
fn fmain(@location(0) @interpolate(linear) col: vec3f) -> @location(0) vec4f {
  return vec4f(col.x, col.y, col.z, 1.0);
}
"""

MESH_COLOR_DISCARD = MESH_COLOR.replace(
    "fn fmain(@location(0) @interpolate(linear) col: vec3f) -> @location(0) vec4f {\n",
    "fn fmain(@location(0) @interpolate(linear) col: vec3f) -> @location(0) vec4f {\n  if col.x < 0.5 { discard; }\n")

TEX_LAMBERT = """
struct Globals { mvp: mat4x4f, light: vec4f, }
@group(0) @binding(0) var<uniform> g: Globals;
@group(1) @binding(0) var albedo: texture_2d<f32>;
@group(1) @binding(1) var albedo_sampler: sampler;
struct VsOut {
  @builtin(position) clip: vec4f,
  @location(0) @interpolate(linear) n: vec3f,
  @location(1) @interpolate(linear) uv: vec2f,
}
@vertex
fn vmain(@location(0) p: vec3f, @location(1) n: vec3f, @location(2) uv: vec2f) -> VsOut {
  return VsOut(g.mvp * vec4f(p.x, p.y, p.z, 1.0), n, uv);
}
@fragment
fn fmain(inp: VsOut) -> @location(0) vec4f {
  let t = textureSample(albedo, albedo_sampler, inp.uv);
  let d = inp.n.x * g.light.x + inp.n.y * g.light.y + inp.n.z * g.light.z;
  let k = select(0.0, d, d > 0.0);
  return t * k;
}
"""
