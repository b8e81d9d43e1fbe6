"""CPU-only checks of the drop-in boundary: libgbr.so loads, exports every entry point that
include/gbr.h declares, and the ctypes mirror has the C header's struct layouts."""

import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbr.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GBR_API\s+[\w\s\*]+?\b(gbr_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def libgbr():
    import build_lib

    path = build_lib.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gbr_device_create" in syms and "gbr_queue_submit" in syms and len(syms) >= 25


def test_library_exports_every_declared_symbol(libgbr):
    missing = [s for s in declared_symbols() if not hasattr(libgbr, s)]
    assert not missing, missing


def test_rust_bindings_declare_every_entry_point():
    """The shim crate's extern block (wgpu-cpu_gb300/rust/src/sys.rs, source only: no Rust
    toolchain here) names every entry point the header declares, and nothing else."""
    sys_rs = open(os.path.join(ROOT, "wgpu-cpu_gb300", "rust", "src", "sys.rs")).read()
    bound = set(re.findall(r"pub fn (gbr_\w+)\s*\(", sys_rs))
    declared = set(declared_symbols())
    assert bound == declared, (sorted(declared - bound), sorted(bound - declared))


_C_SCALARS = {"char": "c_char", "void": "c_void", "uint8_t": "u8", "uint16_t": "u16", "uint32_t": "u32",
              "uint64_t": "u64", "int32_t": "i32", "int64_t": "i64", "float": "f32", "double": "f64"}


def _header_structs():
    """{struct: [(field, Rust spelling of its C type)]} of every typedef struct in gbr.h."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (gbr_\w+)\s*\{(.*?)\}\s*\1\s*;", text, flags=re.S):
        fields = []
        for decl in (" ".join(d.split()) for d in m.group(2).split(";")):
            if not decl:
                continue
            tm = re.match(r"^(const\s+)?(u?int\d+_t|float|double|char|void|gbr_\w+)\s*(.+)$", decl)
            const, base, rest = tm.group(1), tm.group(2), tm.group(3)
            for d in rest.split(","):
                d = d.strip()
                stars = len(d) - len(d.lstrip("*"))
                dm = re.match(r"(\w+)\s*((?:\[[^\]]+\])*)$", d.lstrip("*").strip())
                t = _C_SCALARS.get(base, base)
                if stars:
                    t = ("*const " if const else "*mut ") + t
                for n in reversed(re.findall(r"\[([^\]]+)\]", dm.group(2))):
                    t = f"[{t}; {n}]"
                fields.append((dm.group(1), t.replace(" ", "")))
        out[m.group(1)] = fields
    return out


def test_rust_structs_match_header():
    """Every #[repr(C)] struct of the shim crate's sys.rs has the header struct's fields, in order,
    with the same types (the crate cannot be compiled here, so its layout is checked as text)."""
    text = re.sub(r"//[^\n]*", "", open(os.path.join(ROOT, "wgpu-cpu_gb300", "rust", "src", "sys.rs")).read())
    rust = {}
    for m in re.finditer(r"pub struct (gbr_\w+)\s*\{(.*?)\n\}", text, flags=re.S):
        rust[m.group(1)] = [(f, t.replace(" ", "")) for f, t in re.findall(r"pub (\w+):\s*([^,\n]+),", m.group(2))]
    header = _header_structs()
    assert len(header) >= 30 and set(rust) == set(header), (sorted(set(header) ^ set(rust)))
    bad = {k: (header[k], rust[k]) for k in header if header[k] != rust[k]}
    assert not bad, bad


def test_rust_enum_conversions_match_header():
    """The shim crate's wgpu -> gbr enum conversions (literal codes in lib.rs) give each wgpu
    variant the value of the header enumerator of the same name."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    values = {k: int(v) for k, v in re.findall(r"\b(GBR_\w+)\s*=\s*(-?\d+)\b", text)}
    lib = open(os.path.join(ROOT, "wgpu-cpu_gb300", "rust", "src", "lib.rs")).read()
    prefixes = {"texture_format": "GBR_TEXTURE_FORMAT_", "vertex_format": "GBR_VERTEX_FORMAT_",
                "index_format": "GBR_INDEX_", "topology": "GBR_TOPOLOGY_", "compare": "GBR_COMPARE_",
                "blend_factor": "GBR_BLEND_", "blend_component": "GBR_BLEND_OP_", "address_mode": "GBR_ADDRESS_",
                "filter": "GBR_FILTER_", "mipmap_filter": "GBR_FILTER_"}
    none_names = {"index_format": "GBR_INDEX_NONE", "compare": "GBR_COMPARE_UNDEFINED"}
    snake = lambda v: re.sub(r"(?<=[a-z0-9])(?=[A-Z])", "_", v).upper()
    checked, bad = 0, []
    for fn, prefix in prefixes.items():
        body = re.search(r"\nfn " + fn + r"\(.*?\n\}\n", lib, flags=re.S)
        assert body, fn
        arms = re.findall(r"(?:Some\()?(?:[\w:]*::)?(\w+)\)?\s*=>\s*(\d+),", body.group(0))
        assert arms, fn
        for variant, code in arms:
            name = none_names[fn] if variant == "None" else prefix + snake(variant)
            checked += 1
            if values.get(name) != int(code):
                bad.append((fn, variant, name, values.get(name), int(code)))
    assert checked >= 60 and not bad, (checked, bad)


def test_python_enums_match_header():
    """The ctypes mirror's enum classes (wgpu_gb300.api) hold the header enumerators' values."""
    from wgpu_gb300 import api as W

    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    values = {k: int(v) for k, v in re.findall(r"\b(GBR_\w+)\s*=\s*(-?\d+)\b", text)}
    prefixes = {W.TextureFormat: "GBR_TEXTURE_FORMAT_", W.VertexFormat: "GBR_VERTEX_FORMAT_",
                W.VertexStepMode: "GBR_STEP_", W.IndexFormat: "GBR_INDEX_", W.PrimitiveTopology: "GBR_TOPOLOGY_",
                W.FrontFace: "GBR_FRONT_FACE_", W.Face: "GBR_CULL_", W.CompareFunction: "GBR_COMPARE_",
                W.BlendFactor: "GBR_BLEND_", W.BlendOperation: "GBR_BLEND_OP_", W.AddressMode: "GBR_ADDRESS_",
                W.FilterMode: "GBR_FILTER_", W.LoadOp: "GBR_LOAD_OP_", W.Profile: "GBR_PROFILE_",
                W.LaunchMode: "GBR_LAUNCH_", W.RasterOrder: "GBR_RASTER_", W.RasterRule: "GBR_RASTER_RULE_"}
    checked, bad = 0, []
    for cls, prefix in prefixes.items():
        for name, v in vars(cls).items():
            if name.startswith("_") or not isinstance(v, int):
                continue
            checked += 1
            if values.get(prefix + name) != v:
                bad.append((cls.__name__, name, prefix + name, values.get(prefix + name), v))
    assert checked >= 70 and not bad, (checked, bad)


def test_abi_version(libgbr):
    libgbr.gbr_abi_version.restype = ctypes.c_uint32
    from wgpu_gb300 import _abi as A

    assert libgbr.gbr_abi_version() == A.GBR_ABI_VERSION == 2


def test_device_create_without_gpu_fails_cleanly(libgbr):
    """With no CUDA device the call returns an error status instead of crashing."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from wgpu_gb300 import _abi as A

    cfg = A.DeviceConfig()
    cfg.abi_version = A.GBR_ABI_VERSION
    out = ctypes.c_uint64()
    lib = A.Lib(libgbr, "gbr_")
    st = lib.device_create(ctypes.byref(cfg), ctypes.byref(out))
    assert st != 0
    assert lib.error_text()


STRUCTS = ["gbr_device_config", "gbr_limits", "gbr_texture_desc", "gbr_texel_copy_buffer_layout", "gbr_sampler_desc",
           "gbr_vertex_attribute", "gbr_vertex_buffer_layout", "gbr_color_target_state", "gbr_primitive_state",
           "gbr_depth_stencil_state", "gbr_render_pipeline_desc", "gbr_bind_group_entry", "gbr_bind_group_desc",
           "gbr_submission_stats", "gbr_color_attachment", "gbr_depth_attachment", "gbr_cmd_begin_render_pass",
           "gbr_cmd_set_bind_group", "gbr_cmd_set_index_buffer", "gbr_cmd_set_vertex_buffer", "gbr_cmd_set_viewport",
           "gbr_cmd_draw", "gbr_cmd_draw_indexed", "gbr_cmd_copy_buffer_to_buffer", "gbr_texel_copy_texture_info",
           "gbr_cmd_copy_buffer_texture", "gbr_cmd_copy_texture_to_texture", "gbr_cmd_clear_buffer",
           "gbr_cmd_clear_texture", "gbr_buffer_write", "gbr_pipeline_constant"]
PY = ["DeviceConfig", "Limits", "TextureDesc", "TexelCopyBufferLayout", "SamplerDesc", "VertexAttribute",
      "VertexBufferLayout", "ColorTargetState", "PrimitiveState", "DepthStencilState", "RenderPipelineDesc",
      "BindGroupEntry", "BindGroupDesc", "SubmissionStats", "ColorAttachment", "DepthAttachment",
      "CmdBeginRenderPass", "CmdSetBindGroup", "CmdSetIndexBuffer", "CmdSetVertexBuffer", "CmdSetViewport",
      "CmdDraw", "CmdDrawIndexed", "CmdCopyBufferToBuffer", "TexelCopyTextureInfo", "CmdCopyBufferTexture",
      "CmdCopyTextureToTexture", "CmdClearBuffer", "CmdClearTexture", "BufferWrite", "PipelineConstant"]


def test_ctypes_layouts_match_header(tmp_path):
    from wgpu_gb300 import _abi as A

    src = tmp_path / "sizes.c"
    src.write_text('#include "gbr.h"\n#include <stdio.h>\nint main(void){\n' +
                   "".join(f'printf("%zu\\n", sizeof({s}));\n' for s in STRUCTS) + "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    for c_name, py_name, n in zip(STRUCTS, PY, sizes):
        assert ctypes.sizeof(getattr(A, py_name)) == n, (c_name, ctypes.sizeof(getattr(A, py_name)), n)


def test_gpu_path_has_no_fallback(monkeypatch, tmp_path):
    """The product raises when libgbr.so is absent instead of routing anywhere else."""
    from wgpu_gb300 import api

    monkeypatch.setattr(api, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(api, "_gpu_lib", None)
    with pytest.raises(RuntimeError):
        api.gpu_lib()
