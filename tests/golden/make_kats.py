"""Extract the known-answer vectors of wgpu-cpu's hot-path unit tests into reference_kats.json.

The reference is Rust and cannot be built here, so its unit tests are read as text: each
`#[test]` function of the files below is located by name, its body is cut out by brace
matching, and the literal inputs / expected outputs are parsed with small regular expressions.
Every record keeps the `file:line` of the test it came from.

Run from the repository root:  python tests/golden/make_kats.py /path/to/wgpu-cpu
(or set WGPU_CPU_REPO to the checkout of the reference repository).
"""

from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import os

if len(sys.argv) > 1:
    REF = Path(sys.argv[1])
elif os.environ.get("WGPU_CPU_REPO"):
    REF = Path(os.environ["WGPU_CPU_REPO"])
else:
    raise SystemExit("usage: make_kats.py /path/to/wgpu-cpu  (or set WGPU_CPU_REPO)")
SRC = REF / "wgpu-cpu" / "src"
OUT = Path(__file__).with_name("reference_kats.json")

FLOAT = r"-?\d+(?:\.\d*)?(?:[eE]-?\d+)?"


def fn_body(path: Path, name: str) -> tuple[str, int]:
    text = path.read_text()
    m = re.search(r"fn\s+" + re.escape(name) + r"\s*\(", text)
    if not m:
        raise SystemExit(f"{path}: test {name} not found")
    start = text.index("{", m.end())
    depth = 0
    for i in range(start, len(text)):
        if text[i] == "{":
            depth += 1
        elif text[i] == "}":
            depth -= 1
            if depth == 0:
                line = text.count("\n", 0, m.start()) + 1
                return text[start : i + 1], line
    raise SystemExit(f"{path}: unbalanced braces in {name}")


def vec4s(s: str) -> list[list[float]]:
    return [[float(x) for x in v] for v in re.findall(
        r"Vector4::new\(\s*(" + FLOAT + r")\s*,\s*(" + FLOAT + r")\s*,\s*(" + FLOAT + r")\s*,\s*(" + FLOAT + r")\s*\)", s)]


def rel(p: Path) -> str:
    return str(p.relative_to(REF))


def main() -> None:
    kats: dict[str, list] = {}

    # util/sort.rs: bubblesort3
    p = SRC / "util" / "sort.rs"
    body, line = fn_body(p, "random_bubblesorts")
    pairs = re.findall(r"\[\[(\d+), (\d+), (\d+)\], \[(\d+), (\d+), (\d+)\]\]", body)
    kats["bubblesort3"] = [{"input": [int(a), int(b), int(c)], "expected": [int(d), int(e), int(f)],
                            "source": f"{rel(p)}:{line}"} for a, b, c, d, e, f in pairs]
    body, line = fn_body(p, "bubblesort3_bug")
    vals = [int(x) for x in re.search(r"let mut values = \[(\d+), (\d+), (\d+)\]", body).groups()]
    exp = [int(x) for x in re.findall(r"assert_eq!\(values\[\d\], (\d+)\)", body)]
    kats["bubblesort3"].append({"input": vals, "expected": exp, "source": f"{rel(p)}:{line}"})

    # util/bresenham.rs
    p = SRC / "util" / "bresenham.rs"
    kats["bresenham"] = []
    for name in ["test_wp_example", "test_inverse_wp", "test_straight_hline", "test_straight_vline"]:
        body, line = fn_body(p, name)
        pts = [[int(a), int(b)] for a, b in re.findall(r"Point2::new\((\d+), (\d+)\)", body)]
        kats["bresenham"].append({"start": pts[0], "end": pts[1], "expected": pts[2:],
                                  "source": f"{rel(p)}:{line}"})

    # util/scanline.rs: regression triangles (must not panic / emit negative x)
    p = SRC / "util" / "scanline.rs"
    kats["scanlines_no_panic"] = []
    for name in ["bug_negative_coordinates_generated", "bug_switch_to_second_half_assertion_failed"]:
        body, line = fn_body(p, name)
        code = body.split("/*")[0] + body.split("*/")[-1] if "/*" in body else body
        pts = [[int(a), int(b)] for a, b in re.findall(r"Point2::new\(\s*(\d+),\s*(\d+)\s*\)", code)]
        kats["scanlines_no_panic"].append({"tri": pts[:3], "source": f"{rel(p)}:{line}"})

    # render_pass/primitive.rs: strip order and face winding
    p = SRC / "render_pass" / "primitive.rs"
    body, line = fn_body(p, "triangle_strip")
    exp = [[int(a), int(b), int(c)] for a, b, c in re.findall(r"\[(\d+), (\d+), (\d+)\]", body)]
    n = int(re.search(r"TriStripIter::new\(0\.\.(\d+)\)", body).group(1))
    kats["triangle_strip"] = [{"vertices": n, "expected": exp, "source": f"{rel(p)}:{line}"}]
    body, line = fn_body(p, "triangle_front_face")
    blocks = re.findall(r"let (tri_c\w+) = \[(.*?)\];", body, re.S)
    kats["front_face"] = []
    for name, blk in blocks:
        verts = [[float(a), float(b), float(c)] for a, b, c in re.findall(
            r"\[\s*(" + FLOAT + r"),\s*(" + FLOAT + r"),\s*(" + FLOAT + r")\s*\]", blk)]
        if len(verts) == 3:
            kats["front_face"].append({"vertices": verts, "expected": "Ccw" if name == "tri_ccw" else "Cw",
                                       "source": f"{rel(p)}:{line}"})

    # render_pass/clipper.rs: Cohen–Sutherland line clipper
    p = SRC / "render_pass" / "clipper.rs"
    kats["clip_line"] = []
    body, line = fn_body(p, "line_trivially_inside")
    a, b = vec4s(body)[:2]
    kats["clip_line"].append({"a": a, "b": b, "expected": [a, b], "source": f"{rel(p)}:{line}"})
    for name in ["line_trivially_outside", "line_non_trivially_outside"]:
        body, line = fn_body(p, name)
        v = vec4s(body)
        for i in range(0, len(v), 2):
            kats["clip_line"].append({"a": v[i], "b": v[i + 1], "expected": None, "source": f"{rel(p)}:{line}"})
    for plane in ["left", "right", "bottom", "top", "back", "front"]:
        body, line = fn_body(p, f"clip_line_against_{plane}")
        a, b, c = vec4s(body)[:3]
        kats["clip_line"].append({"a": a, "b": b, "expected": [c, b], "source": f"{rel(p)}:{line}"})
        kats["clip_line"].append({"a": b, "b": a, "expected": [b, c], "source": f"{rel(p)}:{line}"})

    # render_pass/clipper.rs: triangle clipper
    kats["clip_tri"] = []
    for name in ["it_passes_through_tris_that_are_full_inside", "it_rejects_tris_that_are_fully_outside",
                 "it_clips_if_one_vertex_is_outside", "it_clips_if_one_vertex_is_inside"]:
        body, line = fn_body(p, name)
        v = vec4s(body)
        tri = v[:3]
        if "is_empty" in body:
            expected = []
        elif name == "it_passes_through_tris_that_are_full_inside":
            expected = [tri]
        else:
            rest = v[3:]
            expected = [rest[i:i + 3] for i in range(0, len(rest), 3)]
        kats["clip_tri"].append({"tri": tri, "expected": expected, "source": f"{rel(p)}:{line}"})

    # render_pass/index.rs: index resolution with base_vertex
    p = SRC / "render_pass" / "index.rs"
    kats["index_resolution"] = []
    for name, fmt in [("indirect_u16_without_stops", "u16"), ("indirect_u32_without_stops", "u32")]:
        body, line = fn_body(p, name)
        idx = [int(x) for x in re.search(r"vec!\[([\d, ]+)\]", body).group(1).split(",")]
        base = int(re.search(r"\.begin\((-?\d+)\)", body).group(1))
        kats["index_resolution"].append({"format": fmt, "indices": idx, "base_vertex": base,
                                         "expected": [i + base for i in idx], "source": f"{rel(p)}:{line}"})

    # texture.rs: data layout
    p = SRC / "texture.rs"
    body, line = fn_body(p, "data_layout_size")
    w = int(re.search(r"width: (\d+)", body).group(1))
    h = int(re.search(r"height: (\d+)", body).group(1))
    size = int(re.search(r"byte_size\(\), (\d+)", body).group(1))
    kats["texture_layout"] = [{"format": "Rgba8Unorm", "width": w, "height": h, "byte_size": size,
                               "source": f"{rel(p)}:{line}"}]

    # Image goldens: only Git-LFS pointers survive; record their oids (equal oids = equal images).
    kats["image_goldens"] = []
    for png in sorted((REF / "tests" / "reference").glob("*.png")):
        text = png.read_text()
        oid = re.search(r"oid sha256:([0-9a-f]+)", text).group(1)
        size = int(re.search(r"size (\d+)", text).group(1))
        kats["image_goldens"].append({"name": png.stem, "oid": oid, "size": size, "source": rel(png)})

    # naga-cranelift/src/tests.rs: the operator vectors of the shader arithmetic (casts, scalar
    # binops, comparisons, unops), and the expected outputs of its structural tests (control
    # flow, calls, constants, globals, composite access, matrices) by test name
    p = REF / "naga-cranelift" / "src" / "tests.rs"
    text = p.read_text()

    def line_of(pos: int) -> int:
        return text.count("\n", 0, pos) + 1

    ops = []
    for m in re.finditer(r'test_cast\("([^"]*)", "(\w+)", "(\w+)", "([^"]*)"\)', text):
        ops.append({"kind": "cast", "value": m.group(1), "from": m.group(2), "to": m.group(3), "expected": m.group(4),
                    "source": f"{rel(p)}:{line_of(m.start())}"})
    for m in re.finditer(r'test_binop::<(\w+)>\("(\w+)", "([^"]*)", "([^"]+)", "([^"]*)", (-?[\d.]+)\)', text):
        ops.append({"kind": "binop", "type": m.group(2), "left": m.group(3), "op": m.group(4), "right": m.group(5),
                    "expected": float(m.group(6)), "source": f"{rel(p)}:{line_of(m.start())}"})
    for m in re.finditer(r'test_compare\("(\w+)", "([^"]*)", "([^"]+)", "([^"]*)", (true|false)\)', text):
        ops.append({"kind": "compare", "type": m.group(1), "left": m.group(2), "op": m.group(3), "right": m.group(4),
                    "expected": m.group(5) == "true", "source": f"{rel(p)}:{line_of(m.start())}"})
    for m in re.finditer(r'test_unop(?:::<\w+>)?\("(\w+)", "([^"]+)", "([^"]*)", (!?-?[\d.]+)\)', text):
        exp = m.group(4)
        val = (~int(exp[1:])) & 0xFFFFFFFF if exp.startswith("!") else float(exp)
        ops.append({"kind": "unop", "type": m.group(1), "op": m.group(2), "input": m.group(3), "expected": val,
                    "source": f"{rel(p)}:{line_of(m.start())}"})
    for m in re.finditer(r'test_bool_unop\("([^"]+)", "(\w+)", (true|false)\)', text):
        ops.append({"kind": "unop", "type": "bool", "op": m.group(1), "input": m.group(2),
                    "expected": m.group(3) == "true", "source": f"{rel(p)}:{line_of(m.start())}"})
    kats["shader_ops"] = ops

    structural = []
    for m in re.finditer(r"#\[test\]\s*(?:#\[[^\]]*\]\s*)*(?:pub )?fn (\w+)\(\)", text):
        name = m.group(1)
        body, line = fn_body(p, name)
        if re.search(r"#\[ignore", text[m.start():m.end()]):
            continue
        vals = []
        for a in re.finditer(r"assert_(?:abs_diff_)?eq!\(\s*(?:output|out|a)\s*,\s*(\[[^\]]*\]|-?[\d.]+)", body):
            v = a.group(1)
            if v.startswith("["):
                vals.append([float(x) for x in v.strip("[]").split(",") if x.strip()])
            else:
                vals.append(float(v))
        if "DivisionByZero" in body:
            vals.append("DivisionByZero")
        if vals:
            rec = {"test": name, "expected": vals, "source": f"{rel(p)}:{line}"}
            if "mat4x4f" in body:  # the input columns and vector of the matrix tests
                rec["vec4_literals"] = [[float(x) for x in v.split(",")]
                                        for v in re.findall(r"vec4f\(([^()]+,[^()]+,[^()]+,[^()]+)\)", body)]
            structural.append(rec)
    kats["shader_programs"] = structural

    OUT.write_text(json.dumps(kats, indent=1) + "\n")
    print(f"wrote {OUT} ({sum(len(v) for v in kats.values())} records)")


if __name__ == "__main__":
    main()
