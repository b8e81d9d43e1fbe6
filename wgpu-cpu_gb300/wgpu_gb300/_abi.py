"""ctypes mirror of include/gbr.h (layouts must stay identical to the C header)."""

from __future__ import annotations

import ctypes as C

GBR_ABI_VERSION = 2

# status codes
OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_OUT_OF_MEMORY = -2
ERR_UNSUPPORTED = -3
ERR_VALIDATION = -4
ERR_DEVICE_LOST = -5
ERR_TIMEOUT = -6
ERR_SHADER = -7
ERR_CUDA = -8

STATUS_NAMES = {
    OK: "OK", ERR_INVALID_ARGUMENT: "INVALID_ARGUMENT", ERR_OUT_OF_MEMORY: "OUT_OF_MEMORY",
    ERR_UNSUPPORTED: "UNSUPPORTED", ERR_VALIDATION: "VALIDATION", ERR_DEVICE_LOST: "DEVICE_LOST",
    ERR_TIMEOUT: "TIMEOUT", ERR_SHADER: "SHADER", ERR_CUDA: "CUDA",
}

MAX_VERTEX_BUFFERS = 8
MAX_VERTEX_ATTRIBUTES = 16
MAX_COLOR_TARGETS = 4
MAX_BIND_GROUPS = 4
MAX_BIND_GROUP_ENTRIES = 8
MAX_ENTRY_POINT_NAME = 64

# opcodes
OP_BEGIN_RENDER_PASS = 1
OP_END_RENDER_PASS = 2
OP_SET_PIPELINE = 3
OP_SET_BIND_GROUP = 4
OP_SET_INDEX_BUFFER = 5
OP_SET_VERTEX_BUFFER = 6
OP_SET_VIEWPORT = 7
OP_SET_SCISSOR_RECT = 8
OP_SET_BLEND_CONSTANT = 9
OP_SET_STENCIL_REFERENCE = 10
OP_DRAW = 11
OP_DRAW_INDEXED = 12
OP_COPY_BUFFER_TO_BUFFER = 13
OP_COPY_BUFFER_TO_TEXTURE = 14
OP_COPY_TEXTURE_TO_BUFFER = 15
OP_COPY_TEXTURE_TO_TEXTURE = 16
OP_CLEAR_BUFFER = 17
OP_CLEAR_TEXTURE = 18

u32, u64, i32, f32, f64 = C.c_uint32, C.c_uint64, C.c_int32, C.c_float, C.c_double


class DeviceConfig(C.Structure):
    _fields_ = [("abi_version", u32), ("profile", u32), ("device_ordinal", u32), ("tile_size", u32),
                ("bin_capacity", u32), ("warps_per_tile", u32), ("launch_mode", u32), ("batch_submissions", u32),
                ("use_graphs", u32), ("time_kernels", u32), ("hbm_budget_bytes", u64), ("raster_order", u32),
                ("raster_rule", u32), ("reserved", u64 * 3)]


class Limits(C.Structure):
    _fields_ = [("max_texture_dimension_2d", u32), ("max_bind_groups", u32), ("max_vertex_buffers", u32),
                ("max_vertex_attributes", u32), ("max_color_attachments", u32),
                ("max_inter_stage_components", u32), ("max_buffer_size", u64)]


class Extent3d(C.Structure):
    _fields_ = [("width", u32), ("height", u32), ("depth_or_array_layers", u32)]


class TextureDesc(C.Structure):
    _fields_ = [("size", Extent3d), ("mip_level_count", u32), ("sample_count", u32), ("dimension", u32),
                ("format", u32), ("usage", u32), ("_pad", u32)]


class TexelCopyBufferLayout(C.Structure):
    _fields_ = [("offset", u64), ("bytes_per_row", u32), ("rows_per_image", u32)]


class BufferWrite(C.Structure):
    _fields_ = [("buffer", u64), ("offset", u64), ("data", C.c_void_p), ("size", u64)]


class SamplerDesc(C.Structure):
    _fields_ = [("address_mode_u", u32), ("address_mode_v", u32), ("address_mode_w", u32),
                ("mag_filter", u32), ("min_filter", u32), ("mipmap_filter", u32),
                ("lod_min_clamp", f32), ("lod_max_clamp", f32), ("compare", u32), ("anisotropy_clamp", u32)]


class VertexAttribute(C.Structure):
    _fields_ = [("format", u32), ("shader_location", u32), ("offset", u64)]


class VertexBufferLayout(C.Structure):
    _fields_ = [("array_stride", u64), ("step_mode", u32), ("attribute_count", u32),
                ("attributes", VertexAttribute * MAX_VERTEX_ATTRIBUTES)]


class BlendComponent(C.Structure):
    _fields_ = [("src_factor", u32), ("dst_factor", u32), ("operation", u32)]


class ColorTargetState(C.Structure):
    _fields_ = [("format", u32), ("has_blend", u32), ("color", BlendComponent), ("alpha", BlendComponent),
                ("write_mask", u32)]


class PrimitiveState(C.Structure):
    _fields_ = [("topology", u32), ("strip_index_format", u32), ("front_face", u32), ("cull_mode", u32),
                ("polygon_mode", u32), ("unclipped_depth", u32)]


class DepthStencilState(C.Structure):
    _fields_ = [("format", u32), ("depth_write_enabled", u32), ("depth_compare", u32), ("_pad", u32)]


class RenderPipelineDesc(C.Structure):
    _fields_ = [("vertex_module", u64), ("vertex_entry_point", C.c_char * MAX_ENTRY_POINT_NAME),
                ("vertex_buffer_count", u32), ("_pad0", u32),
                ("vertex_buffers", VertexBufferLayout * MAX_VERTEX_BUFFERS), ("primitive", PrimitiveState),
                ("has_depth_stencil", u32), ("_pad1", u32), ("depth_stencil", DepthStencilState),
                ("multisample_count", u32), ("has_fragment", u32), ("fragment_module", u64),
                ("fragment_entry_point", C.c_char * MAX_ENTRY_POINT_NAME), ("color_target_count", u32),
                ("_pad2", u32), ("color_targets", ColorTargetState * MAX_COLOR_TARGETS),
                ("vertex_constants", C.c_void_p), ("fragment_constants", C.c_void_p),
                ("vertex_constant_count", u32), ("fragment_constant_count", u32)]


class PipelineConstant(C.Structure):
    _fields_ = [("key", C.c_char_p), ("value", f64)]


class BindGroupEntry(C.Structure):
    _fields_ = [("binding", u32), ("kind", u32), ("resource", u64), ("offset", u64), ("size", u64)]


class BindGroupDesc(C.Structure):
    _fields_ = [("entry_count", u32), ("_pad", u32), ("entries", BindGroupEntry * MAX_BIND_GROUP_ENTRIES)]


class SubmissionStats(C.Structure):
    _fields_ = [("submission_index", u64), ("draws", u64), ("primitives_in", u64), ("fragments_shaded", u64),
                ("kernel_launches", u64), ("queue_wait_ms", f64), ("gpu_ms", f64), ("submit_to_fence_ms", f64),
                ("batched_with", u32), ("generic_setup_prims", u32), ("raster_ms", f64),
                ("split_tile_chunks", u32), ("tile_shape", u32), ("fs_invocations", u64),
                ("texture_fs_invocations", u64)]


class CmdHeader(C.Structure):
    _fields_ = [("opcode", u32), ("payload_bytes", u32)]


class ColorAttachment(C.Structure):
    _fields_ = [("view", u64), ("load_op", u32), ("store_op", u32), ("clear_value", f64 * 4),
                ("depth_slice", u32), ("_pad", u32)]


class DepthAttachment(C.Structure):
    _fields_ = [("view", u64), ("has_depth_ops", u32), ("depth_load_op", u32), ("depth_store_op", u32),
                ("depth_clear_value", f32)]


class CmdBeginRenderPass(C.Structure):
    _fields_ = [("color_attachment_count", u32), ("has_depth_attachment", u32),
                ("color_attachments", ColorAttachment * MAX_COLOR_TARGETS), ("depth_attachment", DepthAttachment)]


class CmdSetPipeline(C.Structure):
    _fields_ = [("pipeline", u64)]


class CmdSetBindGroup(C.Structure):
    _fields_ = [("index", u32), ("dynamic_offset_count", u32), ("bind_group", u64)]


class CmdSetIndexBuffer(C.Structure):
    _fields_ = [("buffer", u64), ("index_format", u32), ("_pad", u32), ("offset", u64), ("size", u64)]


class CmdSetVertexBuffer(C.Structure):
    _fields_ = [("slot", u32), ("_pad", u32), ("buffer", u64), ("offset", u64), ("size", u64)]


class CmdSetViewport(C.Structure):
    _fields_ = [("x", f32), ("y", f32), ("width", f32), ("height", f32), ("min_depth", f32), ("max_depth", f32)]


class CmdSetScissorRect(C.Structure):
    _fields_ = [("x", u32), ("y", u32), ("width", u32), ("height", u32)]


class CmdSetBlendConstant(C.Structure):
    _fields_ = [("color", f64 * 4)]


class CmdDraw(C.Structure):
    _fields_ = [("vertex_start", u32), ("vertex_end", u32), ("instance_start", u32), ("instance_end", u32)]


class CmdDrawIndexed(C.Structure):
    _fields_ = [("index_start", u32), ("index_end", u32), ("base_vertex", i32), ("instance_start", u32),
                ("instance_end", u32), ("_pad", u32)]


class CmdCopyBufferToBuffer(C.Structure):
    _fields_ = [("source", u64), ("source_offset", u64), ("destination", u64), ("destination_offset", u64),
                ("size", u64)]


class TexelCopyTextureInfo(C.Structure):
    _fields_ = [("texture", u64), ("mip_level", u32), ("origin_x", u32), ("origin_y", u32), ("origin_z", u32)]


class CmdCopyBufferTexture(C.Structure):
    _fields_ = [("buffer", u64), ("layout", TexelCopyBufferLayout), ("texture", TexelCopyTextureInfo),
                ("size", Extent3d), ("_pad", u32)]


class CmdCopyTextureToTexture(C.Structure):
    _fields_ = [("source", TexelCopyTextureInfo), ("destination", TexelCopyTextureInfo), ("size", Extent3d),
                ("_pad", u32)]


class CmdClearBuffer(C.Structure):
    _fields_ = [("buffer", u64), ("offset", u64), ("size", u64)]


class CmdClearTexture(C.Structure):
    _fields_ = [("texture", u64), ("base_mip_level", u32), ("mip_level_count", u32), ("base_array_layer", u32),
                ("array_layer_count", u32)]


P = C.POINTER
SIGNATURES = {
    "last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "abi_version": (u32, []),
    "device_create": (i32, [P(DeviceConfig), P(u64)]),
    "device_destroy": (i32, [u64]),
    "device_limits": (i32, [u64, P(Limits)]),
    "buffer_create": (i32, [u64, u64, u32, P(u64)]),
    "buffer_destroy": (i32, [u64, u64]),
    "queue_write_buffer": (i32, [u64, u64, u64, C.c_void_p, u64]),
    "buffer_read": (i32, [u64, u64, u64, C.c_void_p, u64]),
    "texture_create": (i32, [u64, P(TextureDesc), P(u64)]),
    "texture_destroy": (i32, [u64, u64]),
    "queue_write_texture": (i32, [u64, u64, u32, C.c_void_p, u64, P(TexelCopyBufferLayout), Extent3d]),
    "texture_read": (i32, [u64, u64, u32, C.c_void_p, u64]),
    "sampler_create": (i32, [u64, P(SamplerDesc), P(u64)]),
    "sampler_destroy": (i32, [u64, u64]),
    "shader_module_create_native": (i32, [u64, C.c_char_p, P(u64)]),
    "shader_module_destroy": (i32, [u64, u64]),
    "render_pipeline_create": (i32, [u64, P(RenderPipelineDesc), P(u64)]),
    "render_pipeline_destroy": (i32, [u64, u64]),
    "bind_group_create": (i32, [u64, P(BindGroupDesc), P(u64)]),
    "bind_group_destroy": (i32, [u64, u64]),
    "queue_submit": (i32, [u64, C.c_void_p, u64, P(u64)]),
    "device_poll": (i32, [u64, u32, u32, u64, u64, P(u32)]),
    "submission_stats_get": (i32, [u64, u64, P(SubmissionStats)]),
}
OPTIONAL = {
    "shader_module_create": (i32, [u64, C.c_char_p, u64, P(u64)]),
    "device_elapsed_ms": (i32, [u64, u64, u64, P(f64)]),
    "device_flush_caches": (i32, [u64]),
    "render_pipeline_eval_vertices": (i32, [u64, u64, u32, u32, P(C.c_float), P(u32)]),
    "wgsl_translate": (i32, [C.c_char_p, u64, C.c_char_p, C.c_char_p, C.c_char_p, u64, P(u64)]),
    "wgsl_compile_check": (i32, [C.c_char_p, u64, C.c_char_p, C.c_char_p, C.c_char_p, u64]),
    "textures_read": (i32, [u64, u32, P(u64), P(u32), P(C.c_void_p), P(u64)]),
    "queue_read_textures": (i32, [u64, u32, P(u64), P(u32), P(C.c_void_p), P(u64), P(u64)]),
    "queue_write_buffers": (i32, [u64, u32, C.c_void_p]),
    "device_memory": (i32, [u64, P(u64), P(u64)]),
}

# admission (include/gbr.h): a group adds this much to the sum of its submissions' estimates,
# each estimated at ADMISSION_BYTES_PER_PRIMITIVE per primitive slot + pixels / 16 + 4 KiB
ADMISSION_GROUP_BYTES = 64 << 20
ADMISSION_BYTES_PER_PRIMITIVE = 512


class Lib:
    """Binds the C ABI of one library (GPU library: prefix 'gbr_')."""

    def __init__(self, cdll: C.CDLL, prefix: str = "gbr_"):
        self.cdll = cdll
        self.prefix = prefix
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(cdll, prefix + name)
            fn.restype = res
            fn.argtypes = args
            setattr(self, name, fn)
        for name, (res, args) in OPTIONAL.items():
            fn = getattr(cdll, prefix + name, None)
            if fn is not None:
                fn.restype = res
                fn.argtypes = args
            setattr(self, name, fn)

    def error_text(self) -> str:
        buf = C.create_string_buffer(1024)
        self.last_error(buf, 1024)
        return buf.value.decode(errors="replace")
