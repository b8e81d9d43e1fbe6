//! `#[repr(C)]` mirrors of `include/gbr.h` and its `extern "C"` entry points.
//!
//! The layouts follow the header field for field (the header pads every struct explicitly, so
//! the Rust and C sizes agree without `packed`).  `tests/test_capi_cpu.py` checks the same
//! layouts for the Python mirror against the C compiler.

#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_void};

pub type gbr_status = i32;
pub type gbr_device = u64;
pub type gbr_buffer = u64;
pub type gbr_texture = u64;
pub type gbr_sampler = u64;
pub type gbr_shader_module = u64;
pub type gbr_render_pipeline = u64;
pub type gbr_bind_group = u64;

pub const GBR_ABI_VERSION: u32 = 2;

pub const GBR_OK: gbr_status = 0;
pub const GBR_ERR_INVALID_ARGUMENT: gbr_status = -1;
pub const GBR_ERR_OUT_OF_MEMORY: gbr_status = -2;
pub const GBR_ERR_UNSUPPORTED: gbr_status = -3;
pub const GBR_ERR_VALIDATION: gbr_status = -4;
pub const GBR_ERR_DEVICE_LOST: gbr_status = -5;
pub const GBR_ERR_TIMEOUT: gbr_status = -6;
pub const GBR_ERR_SHADER: gbr_status = -7;
pub const GBR_ERR_CUDA: gbr_status = -8;

pub const GBR_MAX_VERTEX_BUFFERS: usize = 8;
pub const GBR_MAX_VERTEX_ATTRIBUTES: usize = 16;
pub const GBR_MAX_COLOR_TARGETS: usize = 4;
pub const GBR_MAX_BIND_GROUPS: usize = 4;
pub const GBR_MAX_BIND_GROUP_ENTRIES: usize = 8;
pub const GBR_MAX_ENTRY_POINT_NAME: usize = 64;

// gbr_opcode
pub const GBR_OP_BEGIN_RENDER_PASS: u32 = 1;
pub const GBR_OP_END_RENDER_PASS: u32 = 2;
pub const GBR_OP_SET_PIPELINE: u32 = 3;
pub const GBR_OP_SET_BIND_GROUP: u32 = 4;
pub const GBR_OP_SET_INDEX_BUFFER: u32 = 5;
pub const GBR_OP_SET_VERTEX_BUFFER: u32 = 6;
pub const GBR_OP_SET_VIEWPORT: u32 = 7;
pub const GBR_OP_SET_SCISSOR_RECT: u32 = 8;
pub const GBR_OP_SET_BLEND_CONSTANT: u32 = 9;
pub const GBR_OP_SET_STENCIL_REFERENCE: u32 = 10;
pub const GBR_OP_DRAW: u32 = 11;
pub const GBR_OP_DRAW_INDEXED: u32 = 12;
pub const GBR_OP_COPY_BUFFER_TO_BUFFER: u32 = 13;
pub const GBR_OP_COPY_BUFFER_TO_TEXTURE: u32 = 14;
pub const GBR_OP_COPY_TEXTURE_TO_BUFFER: u32 = 15;
pub const GBR_OP_COPY_TEXTURE_TO_TEXTURE: u32 = 16;
pub const GBR_OP_CLEAR_BUFFER: u32 = 17;
pub const GBR_OP_CLEAR_TEXTURE: u32 = 18;

pub const GBR_LOAD_OP_LOAD: u32 = 0;
pub const GBR_LOAD_OP_CLEAR: u32 = 1;
pub const GBR_STORE_OP_STORE: u32 = 0;
pub const GBR_STORE_OP_DISCARD: u32 = 1;

pub const GBR_BINDING_BUFFER: u32 = 0;
pub const GBR_BINDING_SAMPLER: u32 = 1;
pub const GBR_BINDING_TEXTURE_VIEW: u32 = 2;

pub const GBR_POLL_WAIT_SUCCEEDED: u32 = 0;
pub const GBR_POLL_QUEUE_EMPTY: u32 = 1;
pub const GBR_POLL_POLL: u32 = 2;

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_device_config {
    pub abi_version: u32,
    pub profile: u32,
    pub device_ordinal: u32,
    pub tile_size: u32,
    pub bin_capacity: u32,
    pub warps_per_tile: u32,
    pub launch_mode: u32,
    pub batch_submissions: u32,
    pub use_graphs: u32,
    pub time_kernels: u32,
    pub hbm_budget_bytes: u64,
    pub raster_order: u32,
    pub raster_rule: u32,
    pub reserved: [u64; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_limits {
    pub max_texture_dimension_2d: u32,
    pub max_bind_groups: u32,
    pub max_vertex_buffers: u32,
    pub max_vertex_attributes: u32,
    pub max_color_attachments: u32,
    pub max_inter_stage_components: u32,
    pub max_buffer_size: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_extent3d {
    pub width: u32,
    pub height: u32,
    pub depth_or_array_layers: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_texture_desc {
    pub size: gbr_extent3d,
    pub mip_level_count: u32,
    pub sample_count: u32,
    pub dimension: u32,
    pub format: u32,
    pub usage: u32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_texel_copy_buffer_layout {
    pub offset: u64,
    pub bytes_per_row: u32,
    pub rows_per_image: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_sampler_desc {
    pub address_mode_u: u32,
    pub address_mode_v: u32,
    pub address_mode_w: u32,
    pub mag_filter: u32,
    pub min_filter: u32,
    pub mipmap_filter: u32,
    pub lod_min_clamp: f32,
    pub lod_max_clamp: f32,
    pub compare: u32,
    pub anisotropy_clamp: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_vertex_attribute {
    pub format: u32,
    pub shader_location: u32,
    pub offset: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_vertex_buffer_layout {
    pub array_stride: u64,
    pub step_mode: u32,
    pub attribute_count: u32,
    pub attributes: [gbr_vertex_attribute; GBR_MAX_VERTEX_ATTRIBUTES],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_blend_component {
    pub src_factor: u32,
    pub dst_factor: u32,
    pub operation: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_color_target_state {
    pub format: u32,
    pub has_blend: u32,
    pub color: gbr_blend_component,
    pub alpha: gbr_blend_component,
    pub write_mask: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_primitive_state {
    pub topology: u32,
    pub strip_index_format: u32,
    pub front_face: u32,
    pub cull_mode: u32,
    pub polygon_mode: u32,
    pub unclipped_depth: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_depth_stencil_state {
    pub format: u32,
    pub depth_write_enabled: u32,
    pub depth_compare: u32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gbr_pipeline_constant {
    pub key: *const c_char,
    pub value: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gbr_render_pipeline_desc {
    pub vertex_module: gbr_shader_module,
    pub vertex_entry_point: [c_char; GBR_MAX_ENTRY_POINT_NAME],
    pub vertex_buffer_count: u32,
    pub _pad0: u32,
    pub vertex_buffers: [gbr_vertex_buffer_layout; GBR_MAX_VERTEX_BUFFERS],
    pub primitive: gbr_primitive_state,
    pub has_depth_stencil: u32,
    pub _pad1: u32,
    pub depth_stencil: gbr_depth_stencil_state,
    pub multisample_count: u32,
    pub has_fragment: u32,
    pub fragment_module: gbr_shader_module,
    pub fragment_entry_point: [c_char; GBR_MAX_ENTRY_POINT_NAME],
    pub color_target_count: u32,
    pub _pad2: u32,
    pub color_targets: [gbr_color_target_state; GBR_MAX_COLOR_TARGETS],
    pub vertex_constants: *const gbr_pipeline_constant,
    pub fragment_constants: *const gbr_pipeline_constant,
    pub vertex_constant_count: u32,
    pub fragment_constant_count: u32,
}

impl Default for gbr_render_pipeline_desc {
    fn default() -> Self {
        // all-zero is the header's "nothing set" value for every field
        unsafe { std::mem::zeroed() }
    }
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_bind_group_entry {
    pub binding: u32,
    pub kind: u32,
    pub resource: u64,
    pub offset: u64,
    pub size: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_bind_group_desc {
    pub entry_count: u32,
    pub _pad: u32,
    pub entries: [gbr_bind_group_entry; GBR_MAX_BIND_GROUP_ENTRIES],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_submission_stats {
    pub submission_index: u64,
    pub draws: u64,
    pub primitives_in: u64,
    pub fragments_shaded: u64,
    pub kernel_launches: u64,
    pub queue_wait_ms: f64,
    pub gpu_ms: f64,
    pub submit_to_fence_ms: f64,
    pub batched_with: u32,
    pub generic_setup_prims: u32,
    pub raster_ms: f64,
    pub split_tile_chunks: u32,
    pub tile_shape: u32,
    pub fs_invocations: u64,
    pub texture_fs_invocations: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_header {
    pub opcode: u32,
    pub payload_bytes: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_copy_buffer_to_buffer {
    pub source: gbr_buffer,
    pub source_offset: u64,
    pub destination: gbr_buffer,
    pub destination_offset: u64,
    pub size: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_texel_copy_texture_info {
    pub texture: gbr_texture,
    pub mip_level: u32,
    pub origin_x: u32,
    pub origin_y: u32,
    pub origin_z: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_copy_buffer_texture {
    pub buffer: gbr_buffer,
    pub layout: gbr_texel_copy_buffer_layout,
    pub texture: gbr_texel_copy_texture_info,
    pub size: gbr_extent3d,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_copy_texture_to_texture {
    pub source: gbr_texel_copy_texture_info,
    pub destination: gbr_texel_copy_texture_info,
    pub size: gbr_extent3d,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_clear_buffer {
    pub buffer: gbr_buffer,
    pub offset: u64,
    pub size: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_clear_texture {
    pub texture: gbr_texture,
    pub base_mip_level: u32,
    pub mip_level_count: u32,
    pub base_array_layer: u32,
    pub array_layer_count: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_color_attachment {
    pub view: gbr_texture,
    pub load_op: u32,
    pub store_op: u32,
    pub clear_value: [f64; 4],
    pub depth_slice: u32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_depth_attachment {
    pub view: gbr_texture,
    pub has_depth_ops: u32,
    pub depth_load_op: u32,
    pub depth_store_op: u32,
    pub depth_clear_value: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_begin_render_pass {
    pub color_attachment_count: u32,
    pub has_depth_attachment: u32,
    pub color_attachments: [gbr_color_attachment; GBR_MAX_COLOR_TARGETS],
    pub depth_attachment: gbr_depth_attachment,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_set_pipeline {
    pub pipeline: gbr_render_pipeline,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_set_bind_group {
    pub index: u32,
    pub dynamic_offset_count: u32,
    pub bind_group: gbr_bind_group,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_set_index_buffer {
    pub buffer: gbr_buffer,
    pub index_format: u32,
    pub _pad: u32,
    pub offset: u64,
    pub size: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_set_vertex_buffer {
    pub slot: u32,
    pub _pad: u32,
    pub buffer: gbr_buffer,
    pub offset: u64,
    pub size: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_set_viewport {
    pub x: f32,
    pub y: f32,
    pub width: f32,
    pub height: f32,
    pub min_depth: f32,
    pub max_depth: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_set_scissor_rect {
    pub x: u32,
    pub y: u32,
    pub width: u32,
    pub height: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_set_blend_constant {
    pub color: [f64; 4],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_draw {
    pub vertex_start: u32,
    pub vertex_end: u32,
    pub instance_start: u32,
    pub instance_end: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_cmd_draw_indexed {
    pub index_start: u32,
    pub index_end: u32,
    pub base_vertex: i32,
    pub instance_start: u32,
    pub instance_end: u32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gbr_buffer_write {
    pub buffer: gbr_buffer,
    pub offset: u64,
    pub data: *const c_void,
    pub size: u64,
}

#[link(name = "gbr")]
unsafe /// Render state of the allocation-free entry point (gbr_render_triangles_noalloc).
#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gbr_noalloc_state {
    pub cull_mode: u32,
    pub front_face: u32,
    pub depth_compare: u32,
    pub depth_write_enabled: u32,
    pub color_load_op: u32,
    pub depth_load_op: u32,
    pub clear_color: [f32; 4],
    pub clear_depth: f32,
    pub _pad: u32,
}

pub const GBR_NOALLOC_SCRATCH_BYTES: u32 = 24 << 20;
pub const GBR_NOALLOC_MAX_TRIANGLES: u32 = 32768;
pub const GBR_NOALLOC_MAX_CLIPPED: u32 = 8192;
pub const GBR_NOALLOC_MAX_DIM: u32 = 2048;
pub const GBR_NOALLOC_MAX_BIN_ENTRIES: u32 = 3_800_000;

extern "C" {
    pub fn gbr_last_error(buf: *mut c_char, buf_len: usize) -> usize;
    pub fn gbr_abi_version() -> u32;
    pub fn gbr_device_create(config: *const gbr_device_config, out_device: *mut gbr_device) -> gbr_status;
    pub fn gbr_device_destroy(device: gbr_device) -> gbr_status;
    pub fn gbr_device_limits(device: gbr_device, out_limits: *mut gbr_limits) -> gbr_status;
    pub fn gbr_buffer_create(device: gbr_device, size: u64, usage: u32, out_buffer: *mut gbr_buffer) -> gbr_status;
    pub fn gbr_buffer_destroy(device: gbr_device, buffer: gbr_buffer) -> gbr_status;
    pub fn gbr_queue_write_buffer(
        device: gbr_device,
        buffer: gbr_buffer,
        offset: u64,
        data: *const c_void,
        size: u64,
    ) -> gbr_status;
    pub fn gbr_queue_write_buffers(device: gbr_device, count: u32, writes: *const gbr_buffer_write) -> gbr_status;
    pub fn gbr_buffer_read(device: gbr_device, buffer: gbr_buffer, offset: u64, dst: *mut c_void, size: u64)
        -> gbr_status;
    pub fn gbr_texture_create(device: gbr_device, desc: *const gbr_texture_desc, out_texture: *mut gbr_texture)
        -> gbr_status;
    pub fn gbr_texture_destroy(device: gbr_device, texture: gbr_texture) -> gbr_status;
    pub fn gbr_queue_write_texture(
        device: gbr_device,
        texture: gbr_texture,
        mip_level: u32,
        data: *const c_void,
        data_size: u64,
        layout: *const gbr_texel_copy_buffer_layout,
        size: gbr_extent3d,
    ) -> gbr_status;
    pub fn gbr_texture_read(device: gbr_device, texture: gbr_texture, mip_level: u32, dst: *mut c_void, size: u64)
        -> gbr_status;
    pub fn gbr_textures_read(
        device: gbr_device,
        count: u32,
        textures: *const gbr_texture,
        mip_levels: *const u32,
        dsts: *const *mut c_void,
        sizes: *const u64,
    ) -> gbr_status;
    pub fn gbr_queue_read_textures(
        device: gbr_device,
        count: u32,
        textures: *const gbr_texture,
        mip_levels: *const u32,
        dsts: *const *mut c_void,
        sizes: *const u64,
        out_index: *mut u64,
    ) -> gbr_status;
    pub fn gbr_sampler_create(device: gbr_device, desc: *const gbr_sampler_desc, out_sampler: *mut gbr_sampler)
        -> gbr_status;
    pub fn gbr_sampler_destroy(device: gbr_device, sampler: gbr_sampler) -> gbr_status;
    pub fn gbr_shader_module_create(
        device: gbr_device,
        wgsl: *const c_char,
        wgsl_len: u64,
        out_module: *mut gbr_shader_module,
    ) -> gbr_status;
    pub fn gbr_shader_module_destroy(device: gbr_device, module: gbr_shader_module) -> gbr_status;
    pub fn gbr_render_pipeline_create(
        device: gbr_device,
        desc: *const gbr_render_pipeline_desc,
        out_pipeline: *mut gbr_render_pipeline,
    ) -> gbr_status;
    pub fn gbr_render_pipeline_destroy(device: gbr_device, pipeline: gbr_render_pipeline) -> gbr_status;
    pub fn gbr_bind_group_create(
        device: gbr_device,
        desc: *const gbr_bind_group_desc,
        out_bind_group: *mut gbr_bind_group,
    ) -> gbr_status;
    pub fn gbr_bind_group_destroy(device: gbr_device, bind_group: gbr_bind_group) -> gbr_status;
    pub fn gbr_queue_submit(
        device: gbr_device,
        commands: *const c_void,
        commands_len: u64,
        out_submission_index: *mut u64,
    ) -> gbr_status;
    pub fn gbr_device_poll(
        device: gbr_device,
        wait: u32,
        has_index: u32,
        submission_index: u64,
        timeout_ns: u64,
        out_status: *mut u32,
    ) -> gbr_status;
    pub fn gbr_submission_stats_get(
        device: gbr_device,
        submission_index: u64,
        out_stats: *mut gbr_submission_stats,
    ) -> gbr_status;

    // extensions, diagnostics and the allocation-free entry point (not behind a wgpu trait)
    pub fn gbr_shader_module_create_native(
        device: gbr_device,
        name: *const c_char,
        out_module: *mut gbr_shader_module,
    ) -> gbr_status;
    pub fn gbr_render_pipeline_eval_vertices(
        device: gbr_device,
        pipeline: gbr_render_pipeline,
        first_vertex: u32,
        count: u32,
        out: *mut f32,
        errors: *mut u32,
    ) -> gbr_status;
    pub fn gbr_wgsl_translate(
        wgsl: *const c_char,
        wgsl_len: u64,
        vertex_entry: *const c_char,
        fragment_entry: *const c_char,
        out: *mut c_char,
        capacity: u64,
        needed: *mut u64,
    ) -> gbr_status;
    pub fn gbr_wgsl_compile_check(
        wgsl: *const c_char,
        wgsl_len: u64,
        vertex_entry: *const c_char,
        fragment_entry: *const c_char,
        log: *mut c_char,
        capacity: u64,
    ) -> gbr_status;
    pub fn gbr_device_elapsed_ms(
        device: gbr_device,
        first_submission: u64,
        last_submission: u64,
        out_ms: *mut f64,
    ) -> gbr_status;
    pub fn gbr_device_memory(device: gbr_device, out_resident_bytes: *mut u64, out_transient_bytes: *mut u64)
        -> gbr_status;
    pub fn gbr_device_flush_caches(device: gbr_device) -> gbr_status;
    pub fn gbr_selftest_division(samples: u64, seed: u64, out_mismatches: *mut u64, first_mismatch: *mut f32)
        -> gbr_status;
    pub fn gbr_render_triangles_noalloc(
        clip_positions: *const f32,
        colors: *const f32,
        triangle_count: u32,
        color_target: *mut u8,
        depth_target: *mut f32,
        width: u32,
        height: u32,
        state: *const gbr_noalloc_state,
        stream: *mut c_void,
    ) -> gbr_status;
}

/// The thread's last error text (gbr_last_error).
pub fn last_error() -> String {
    let mut buf = vec![0 as c_char; 1024];
    let n = unsafe { gbr_last_error(buf.as_mut_ptr(), buf.len()) };
    let n = n.min(buf.len() - 1);
    let bytes: Vec<u8> = buf[..n].iter().map(|&c| c as u8).collect();
    String::from_utf8_lossy(&bytes).into_owned()
}
