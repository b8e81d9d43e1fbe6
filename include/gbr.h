/*
 * gbr.h — C ABI of the GB300 render-pass path (drop-in for wgpu-cpu's render-pass hot path).
 *
 * Every entry point below replaces one method of the wgpu 28 "custom backend" traits that
 * wgpu-cpu implements in Rust.  The reference method is cited beside each declaration as
 * `file:line` relative to the wgpu-cpu repository.  A Rust `wgpu::custom` shim binds these
 * symbols with `extern "C"` declarations and forwards each trait method to one of them.
 *
 * Conventions
 *  - Objects are opaque 64-bit handles owned by the library; 0 is never a valid handle.
 *  - Every call returns a gbr_status (0 = GBR_OK).  Nothing unwinds across the ABI: where the
 *    reference panics (`todo!`, `unwrap`, `expect`), the call returns an error status and
 *    gbr_last_error() gives the thread-local message.
 *  - Host memory passed in is copied before the call returns; the caller keeps ownership.
 *  - All structs are plain C, little-endian, with explicit padding so that ctypes/cgo/Rust
 *    `#[repr(C)]` mirrors have identical layouts.
 *  - Enum values follow the numbering of the corresponding wgpu-types enums where one exists.
 */
#ifndef GBR_H
#define GBR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define GBR_API __declspec(dllexport)
#else
#define GBR_API __attribute__((visibility("default")))
#endif

#define GBR_ABI_VERSION 2u

typedef int32_t gbr_status;
enum {
    GBR_OK = 0,
    GBR_ERR_INVALID_ARGUMENT = -1, /* bad handle / null pointer / malformed descriptor        */
    GBR_ERR_OUT_OF_MEMORY = -2,    /* device allocation failed or HBM budget exceeded        */
    GBR_ERR_UNSUPPORTED = -3,      /* the reference has `todo!()`/panics for this feature    */
    GBR_ERR_VALIDATION = -4,       /* the reference would panic (assert/expect/out of range) */
    GBR_ERR_DEVICE_LOST = -5,      /* a kernel reported a fault; the device must be recreated */
    GBR_ERR_TIMEOUT = -6,          /* gbr_device_poll ran out of time                          */
    GBR_ERR_SHADER = -7,           /* shader parse / translate / NVRTC compile error           */
    GBR_ERR_CUDA = -8              /* a CUDA runtime call failed                               */
};

typedef uint64_t gbr_device;
typedef uint64_t gbr_buffer;
typedef uint64_t gbr_texture;
typedef uint64_t gbr_sampler;
typedef uint64_t gbr_shader_module;
typedef uint64_t gbr_render_pipeline;
typedef uint64_t gbr_bind_group;

/* ---------------------------------------------------------------- enums (wgpu-types numbering) */

enum gbr_texture_format {
    GBR_TEXTURE_FORMAT_UNDEFINED = 0,
    GBR_TEXTURE_FORMAT_R8_UNORM = 1,
    GBR_TEXTURE_FORMAT_RG8_UNORM = 2,
    GBR_TEXTURE_FORMAT_RGBA8_UNORM = 3,
    GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB = 4,
    GBR_TEXTURE_FORMAT_BGRA8_UNORM = 5,
    GBR_TEXTURE_FORMAT_BGRA8_UNORM_SRGB = 6,
    GBR_TEXTURE_FORMAT_RGBA16_FLOAT = 7,
    GBR_TEXTURE_FORMAT_RGBA32_FLOAT = 8,
    GBR_TEXTURE_FORMAT_DEPTH32_FLOAT = 9
};

enum gbr_vertex_format {
    GBR_VERTEX_FORMAT_FLOAT32 = 1,
    GBR_VERTEX_FORMAT_FLOAT32X2 = 2,
    GBR_VERTEX_FORMAT_FLOAT32X3 = 3,
    GBR_VERTEX_FORMAT_FLOAT32X4 = 4,
    GBR_VERTEX_FORMAT_UINT32 = 5,
    GBR_VERTEX_FORMAT_SINT32 = 6,
    GBR_VERTEX_FORMAT_FLOAT16X2 = 7,
    GBR_VERTEX_FORMAT_FLOAT16X4 = 8,
    GBR_VERTEX_FORMAT_UNORM8X4 = 9
};

enum gbr_vertex_step_mode { GBR_STEP_VERTEX = 0, GBR_STEP_INSTANCE = 1 };
enum gbr_index_format { GBR_INDEX_NONE = 0, GBR_INDEX_UINT16 = 1, GBR_INDEX_UINT32 = 2 };

enum gbr_primitive_topology {
    GBR_TOPOLOGY_POINT_LIST = 0,
    GBR_TOPOLOGY_LINE_LIST = 1,
    GBR_TOPOLOGY_LINE_STRIP = 2,
    GBR_TOPOLOGY_TRIANGLE_LIST = 3,
    GBR_TOPOLOGY_TRIANGLE_STRIP = 4
};
enum gbr_front_face { GBR_FRONT_FACE_CCW = 0, GBR_FRONT_FACE_CW = 1 };
enum gbr_cull_mode { GBR_CULL_NONE = 0, GBR_CULL_FRONT = 1, GBR_CULL_BACK = 2 };
enum gbr_polygon_mode { GBR_POLYGON_FILL = 0, GBR_POLYGON_LINE = 1, GBR_POLYGON_POINT = 2 };

enum gbr_compare_function {
    GBR_COMPARE_UNDEFINED = 0,
    GBR_COMPARE_NEVER = 1,
    GBR_COMPARE_LESS = 2,
    GBR_COMPARE_EQUAL = 3,
    GBR_COMPARE_LESS_EQUAL = 4,
    GBR_COMPARE_GREATER = 5,
    GBR_COMPARE_NOT_EQUAL = 6,
    GBR_COMPARE_GREATER_EQUAL = 7,
    GBR_COMPARE_ALWAYS = 8
};

enum gbr_blend_factor {
    GBR_BLEND_ZERO = 0,
    GBR_BLEND_ONE = 1,
    GBR_BLEND_SRC = 2,
    GBR_BLEND_ONE_MINUS_SRC = 3,
    GBR_BLEND_SRC_ALPHA = 4,
    GBR_BLEND_ONE_MINUS_SRC_ALPHA = 5,
    GBR_BLEND_DST = 6,
    GBR_BLEND_ONE_MINUS_DST = 7,
    GBR_BLEND_DST_ALPHA = 8,
    GBR_BLEND_ONE_MINUS_DST_ALPHA = 9,
    GBR_BLEND_CONSTANT = 11,
    GBR_BLEND_ONE_MINUS_CONSTANT = 12
};
enum gbr_blend_operation {
    GBR_BLEND_OP_ADD = 0,
    GBR_BLEND_OP_SUBTRACT = 1,
    GBR_BLEND_OP_REVERSE_SUBTRACT = 2,
    GBR_BLEND_OP_MIN = 3,
    GBR_BLEND_OP_MAX = 4
};

enum gbr_address_mode {
    GBR_ADDRESS_CLAMP_TO_EDGE = 0,
    GBR_ADDRESS_REPEAT = 1,
    GBR_ADDRESS_MIRROR_REPEAT = 2,
    GBR_ADDRESS_CLAMP_TO_BORDER = 3
};
enum gbr_filter_mode { GBR_FILTER_NEAREST = 0, GBR_FILTER_LINEAR = 1 };

enum gbr_load_op { GBR_LOAD_OP_LOAD = 0, GBR_LOAD_OP_CLEAR = 1 };
enum gbr_store_op { GBR_STORE_OP_STORE = 0, GBR_STORE_OP_DISCARD = 1 };

/* Semantics profile of a device.
 *  PARITY    — exactly the reference's behaviour: blend state ignored (overwrite), sRGB formats
 *              read/written as linear, sampler filters ignored (nearest), perspective
 *              interpolation and f16/f32 colour targets rejected with GBR_ERR_UNSUPPORTED.
 *  EXTENSION — the same coverage and depth rule, plus WebGPU-spec blending, Rgba16Float /
 *              Rgba32Float targets, sRGB encode/decode, linear/mip filtering and
 *              perspective-correct interpolation (features the reference leaves `todo!`). */
enum gbr_profile { GBR_PROFILE_PARITY = 0, GBR_PROFILE_EXTENSION = 1 };

/* ---------------------------------------------------------------- descriptors */

typedef struct gbr_device_config {
    uint32_t abi_version;       /* must be GBR_ABI_VERSION                                   */
    uint32_t profile;           /* gbr_profile                                               */
    uint32_t device_ordinal;    /* CUDA device                                               */
    uint32_t tile_size;         /* raster tile side: 8, 16 or 32 (0 = default 16)            */
    uint32_t bin_capacity;      /* max primitives sorted per tile in one window (0 = auto)   */
    uint32_t warps_per_tile;    /* 1..8 (0 = default)                                        */
    uint32_t launch_mode;       /* gbr_launch_mode                                           */
    uint32_t batch_submissions; /* 1 = the worker merges queued submissions into one launch  */
    uint32_t use_graphs;        /* 1 = replay per-shape CUDA graphs                          */
    uint32_t time_kernels;      /* 1 = CUDA events around the raster kernels (stats.raster_ms) */
    uint64_t hbm_budget_bytes;  /* HBM for resident resources + transient scratch; 0 = 80 GB  */
    uint32_t raster_order;      /* gbr_raster_order                                          */
    uint32_t raster_rule;       /* gbr_raster_rule (EDGE requires the extension profile)     */
    uint64_t reserved[3];
} gbr_device_config;

/* How draws map to kernel launches.
 *  BATCHED  — consecutive render passes without dependencies between them (no pass writes or
 *             samples a texture another pass of the group writes) share one setup/bin/raster
 *             launch sequence over all their targets and draws.  The default.
 *  PER_DRAW — the plain drop-in: one launch sequence per draw, each over the whole target.
 *  PER_PASS — one launch sequence per render pass. */
enum gbr_launch_mode { GBR_LAUNCH_BATCHED = 0, GBR_LAUNCH_PER_DRAW = 1, GBR_LAUNCH_PER_PASS = 2 };

/* How a tile's fragments are resolved.
 *  AUTO     — batches whose draws all write depth with Less/LessEqual/Greater/GreaterEqual, do
 *             not blend and never discard resolve each pixel's surviving fragment by an atomic
 *             (depth, order) minimum and shade only that one (same colour, depth and fragment
 *             count as the ordered walk); every other batch walks its fragments in order.
 *  ORDERED  — always walk fragments in primitive order. */
enum gbr_raster_order { GBR_RASTER_AUTO = 0, GBR_RASTER_ORDERED = 1 };

/* Which pixels a triangle covers.
 *  SCANLINE — the reference's rule (raster.rs:280-363, util/scanline.rs): integer framebuffer
 *             vertices, inclusive spans walked by its scanline state machine, attributes
 *             sampled at the integer pixel corner.  Bit-exact with wgpu-cpu.
 *  EDGE     — extension profile: vertices snapped to 1/256 pixel, fixed-point edge functions
 *             evaluated at pixel centres with the top-left rule (shared edges cover each pixel
 *             exactly once), attributes sampled at the pixel centre.  Lines and points keep
 *             the reference's Bresenham rule. */
enum gbr_raster_rule { GBR_RASTER_RULE_SCANLINE = 0, GBR_RASTER_RULE_EDGE = 1 };

typedef struct gbr_limits {
    uint32_t max_texture_dimension_2d;
    uint32_t max_bind_groups;
    uint32_t max_vertex_buffers;
    uint32_t max_vertex_attributes;
    uint32_t max_color_attachments;
    uint32_t max_inter_stage_components;
    uint64_t max_buffer_size;
} gbr_limits;

typedef struct gbr_extent3d {
    uint32_t width, height, depth_or_array_layers;
} gbr_extent3d;

typedef struct gbr_texture_desc {
    gbr_extent3d size;
    uint32_t mip_level_count;
    uint32_t sample_count;
    uint32_t dimension; /* 2 = D2 (only D2 is used on the path) */
    uint32_t format;    /* gbr_texture_format */
    uint32_t usage;     /* wgpu::TextureUsages bits (informational) */
    uint32_t _pad;
} gbr_texture_desc;

/* wgpu::TexelCopyBufferLayout */
typedef struct gbr_texel_copy_buffer_layout {
    uint64_t offset;
    uint32_t bytes_per_row; /* 0 = None */
    uint32_t rows_per_image; /* 0 = None */
} gbr_texel_copy_buffer_layout;

typedef struct gbr_sampler_desc {
    uint32_t address_mode_u, address_mode_v, address_mode_w; /* gbr_address_mode */
    uint32_t mag_filter, min_filter, mipmap_filter;          /* gbr_filter_mode  */
    float lod_min_clamp, lod_max_clamp;
    uint32_t compare; /* gbr_compare_function, 0 = none */
    uint32_t anisotropy_clamp;
} gbr_sampler_desc;

typedef struct gbr_vertex_attribute {
    uint32_t format; /* gbr_vertex_format */
    uint32_t shader_location;
    uint64_t offset;
} gbr_vertex_attribute;

#define GBR_MAX_VERTEX_BUFFERS 8
#define GBR_MAX_VERTEX_ATTRIBUTES 16
#define GBR_MAX_COLOR_TARGETS 4
#define GBR_MAX_BIND_GROUPS 4
#define GBR_MAX_BIND_GROUP_ENTRIES 8
#define GBR_MAX_ENTRY_POINT_NAME 64

typedef struct gbr_vertex_buffer_layout {
    uint64_t array_stride;
    uint32_t step_mode; /* gbr_vertex_step_mode */
    uint32_t attribute_count;
    gbr_vertex_attribute attributes[GBR_MAX_VERTEX_ATTRIBUTES];
} gbr_vertex_buffer_layout;

typedef struct gbr_blend_component {
    uint32_t src_factor, dst_factor, operation;
} gbr_blend_component;

typedef struct gbr_color_target_state {
    uint32_t format;     /* gbr_texture_format */
    uint32_t has_blend;  /* 0 = blend: None */
    gbr_blend_component color, alpha;
    uint32_t write_mask; /* wgpu::ColorWrites bits: R=1 G=2 B=4 A=8 */
} gbr_color_target_state;

typedef struct gbr_primitive_state {
    uint32_t topology;           /* gbr_primitive_topology */
    uint32_t strip_index_format; /* gbr_index_format, NONE = no primitive restart */
    uint32_t front_face;         /* gbr_front_face */
    uint32_t cull_mode;          /* gbr_cull_mode */
    uint32_t polygon_mode;       /* gbr_polygon_mode */
    uint32_t unclipped_depth;
} gbr_primitive_state;

typedef struct gbr_depth_stencil_state {
    uint32_t format;              /* GBR_TEXTURE_FORMAT_DEPTH32_FLOAT */
    uint32_t depth_write_enabled;
    uint32_t depth_compare;       /* gbr_compare_function */
    uint32_t _pad;
} gbr_depth_stencil_state;

/* One pipeline-overridable constant (wgpu::PipelineCompilationOptions::constants entry): `key`
 * is an `override`'s @id as a decimal string, or its name; `value` is converted to the override's
 * type as naga's process_overrides does (shader.rs:52-74).  Read during the call only. */
typedef struct gbr_pipeline_constant {
    const char* key;
    double value;
} gbr_pipeline_constant;

typedef struct gbr_render_pipeline_desc {
    gbr_shader_module vertex_module;
    char vertex_entry_point[GBR_MAX_ENTRY_POINT_NAME];
    uint32_t vertex_buffer_count;
    uint32_t _pad0;
    gbr_vertex_buffer_layout vertex_buffers[GBR_MAX_VERTEX_BUFFERS];
    gbr_primitive_state primitive;
    uint32_t has_depth_stencil;
    uint32_t _pad1;
    gbr_depth_stencil_state depth_stencil;
    uint32_t multisample_count;
    uint32_t has_fragment;
    gbr_shader_module fragment_module;
    char fragment_entry_point[GBR_MAX_ENTRY_POINT_NAME];
    uint32_t color_target_count;
    uint32_t _pad2;
    gbr_color_target_state color_targets[GBR_MAX_COLOR_TARGETS];
    /* VertexState / FragmentState compilation_options.constants (WGSL modules only) */
    const gbr_pipeline_constant* vertex_constants;
    const gbr_pipeline_constant* fragment_constants;
    uint32_t vertex_constant_count;
    uint32_t fragment_constant_count;
} gbr_render_pipeline_desc;

enum gbr_binding_kind { GBR_BINDING_BUFFER = 0, GBR_BINDING_SAMPLER = 1, GBR_BINDING_TEXTURE_VIEW = 2 };

typedef struct gbr_bind_group_entry {
    uint32_t binding;
    uint32_t kind;     /* gbr_binding_kind */
    uint64_t resource; /* gbr_buffer / gbr_sampler / gbr_texture handle */
    uint64_t offset;   /* buffer bindings */
    uint64_t size;     /* buffer bindings, 0 = rest of buffer */
} gbr_bind_group_entry;

typedef struct gbr_bind_group_desc {
    uint32_t entry_count;
    uint32_t _pad;
    gbr_bind_group_entry entries[GBR_MAX_BIND_GROUP_ENTRIES];
} gbr_bind_group_desc;

/* Per-submission record kept for metrics (the reference logs these with `tracing` only:
 * render_pass/mod.rs:392-393, render_pass/state.rs:516-517,592). */
typedef struct gbr_submission_stats {
    uint64_t submission_index;
    uint64_t draws;
    uint64_t primitives_in;        /* primitives assembled (incl. culled) */
    uint64_t fragments_shaded;     /* fragment-shader invocations, counted as the reference */
    uint64_t kernel_launches;
    double queue_wait_ms;          /* submit -> start of device work  */
    double gpu_ms;                 /* device time of the submission   */
    double submit_to_fence_ms;     /* submit -> fence signalled       */
    uint32_t batched_with;         /* number of submissions merged into the same launch */
    uint32_t generic_setup_prims;  /* primitives set up by the generic (clipping) setup kernel */
    double raster_ms;              /* device time of the raster kernels (config.time_kernels) */
    uint32_t split_tile_chunks;    /* visibility raster: work items of tiles split by record count */
    uint32_t tile_shape;           /* tile side << 8 | warps per tile of the submission's largest batch */
    /* Fragment-stage runs.  The reference runs the fragment stage for every fragment it counts
     * (fragments_shaded) unless an @early_depth_test rejects it first; the visibility raster
     * (gbr_raster_order AUTO) runs it once per pixel, for the fragment whose output survives,
     * with the same resulting colours and depths. */
    uint64_t fs_invocations;
    uint64_t texture_fs_invocations; /* the part of fs_invocations whose program samples a texture */
} gbr_submission_stats;

/* ---------------------------------------------------------------- command stream
 *
 * A command buffer is a flat little-endian byte stream of records
 *     [u32 opcode][u32 payload_bytes][payload ... padded to 8 bytes]
 * mirroring `RenderPassSubCommand` (render_pass/mod.rs:397-423) wrapped in begin/end pass
 * records (`Command::RenderPass`, command.rs:188-190).  Streams are consumed at submit.
 */
enum gbr_opcode {
    GBR_OP_BEGIN_RENDER_PASS = 1,  /* payload: gbr_cmd_begin_render_pass */
    GBR_OP_END_RENDER_PASS = 2,    /* payload: none */
    GBR_OP_SET_PIPELINE = 3,       /* payload: gbr_cmd_set_pipeline */
    GBR_OP_SET_BIND_GROUP = 4,     /* payload: gbr_cmd_set_bind_group */
    GBR_OP_SET_INDEX_BUFFER = 5,   /* payload: gbr_cmd_set_index_buffer */
    GBR_OP_SET_VERTEX_BUFFER = 6,  /* payload: gbr_cmd_set_vertex_buffer */
    GBR_OP_SET_VIEWPORT = 7,       /* payload: gbr_cmd_set_viewport */
    GBR_OP_SET_SCISSOR_RECT = 8,   /* payload: gbr_cmd_set_scissor_rect */
    GBR_OP_SET_BLEND_CONSTANT = 9, /* payload: gbr_cmd_set_blend_constant */
    GBR_OP_SET_STENCIL_REFERENCE = 10, /* payload: u32 + pad */
    GBR_OP_DRAW = 11,              /* payload: gbr_cmd_draw */
    GBR_OP_DRAW_INDEXED = 12,      /* payload: gbr_cmd_draw_indexed */
    /* Encoder commands outside render passes.  The reference leaves every one `todo!`
     * (command.rs:37-115): the parity profile rejects them with GBR_ERR_UNSUPPORTED; the
     * extension profile executes them with WebGPU semantics, in order with the passes. */
    GBR_OP_COPY_BUFFER_TO_BUFFER = 13,   /* payload: gbr_cmd_copy_buffer_to_buffer */
    GBR_OP_COPY_BUFFER_TO_TEXTURE = 14,  /* payload: gbr_cmd_copy_buffer_texture */
    GBR_OP_COPY_TEXTURE_TO_BUFFER = 15,  /* payload: gbr_cmd_copy_buffer_texture */
    GBR_OP_COPY_TEXTURE_TO_TEXTURE = 16, /* payload: gbr_cmd_copy_texture_to_texture */
    GBR_OP_CLEAR_BUFFER = 17,            /* payload: gbr_cmd_clear_buffer */
    GBR_OP_CLEAR_TEXTURE = 18            /* payload: gbr_cmd_clear_texture */
};

typedef struct gbr_cmd_header {
    uint32_t opcode;
    uint32_t payload_bytes;
} gbr_cmd_header;

/* CommandEncoderInterface::copy_buffer_to_buffer (command.rs:37-46).  Offsets and size are
 * multiples of 4, source and destination differ; size = UINT64_MAX copies to the source's end. */
typedef struct gbr_cmd_copy_buffer_to_buffer {
    gbr_buffer source;
    uint64_t source_offset;
    gbr_buffer destination;
    uint64_t destination_offset;
    uint64_t size;
} gbr_cmd_copy_buffer_to_buffer;

/* wgpu::TexelCopyTextureInfo: a mip level of a texture and the texel origin (x, y, array layer). */
typedef struct gbr_texel_copy_texture_info {
    gbr_texture texture;
    uint32_t mip_level;
    uint32_t origin_x, origin_y, origin_z;
} gbr_texel_copy_texture_info;

/* copy_buffer_to_texture / copy_texture_to_buffer (command.rs:48-64): `size` texels per layer
 * row/column/layer; the buffer side is laid out by `layout` (bytes_per_row a multiple of 256
 * when the copy has more than one row, 0 = tightly packed single row; rows_per_image 0 = height). */
typedef struct gbr_cmd_copy_buffer_texture {
    gbr_buffer buffer;
    gbr_texel_copy_buffer_layout layout;
    gbr_texel_copy_texture_info texture;
    gbr_extent3d size;
    uint32_t _pad;
} gbr_cmd_copy_buffer_texture;

/* copy_texture_to_texture (command.rs:66-73): same format, different textures or ranges. */
typedef struct gbr_cmd_copy_texture_to_texture {
    gbr_texel_copy_texture_info source;
    gbr_texel_copy_texture_info destination;
    gbr_extent3d size;
    uint32_t _pad;
} gbr_cmd_copy_texture_to_texture;

/* clear_buffer (command.rs:108-115): zeroes [offset, offset + size); size = UINT64_MAX to the end. */
typedef struct gbr_cmd_clear_buffer {
    gbr_buffer buffer;
    uint64_t offset;
    uint64_t size;
} gbr_cmd_clear_buffer;

/* clear_texture (command.rs:100-106): zeroes the mip levels and array layers of the subresource
 * range (counts of 0 = all remaining). */
typedef struct gbr_cmd_clear_texture {
    gbr_texture texture;
    uint32_t base_mip_level, mip_level_count;
    uint32_t base_array_layer, array_layer_count;
} gbr_cmd_clear_texture;

typedef struct gbr_color_attachment {
    gbr_texture view;      /* texture (mip 0, layer `depth_slice`) */
    uint32_t load_op;      /* gbr_load_op */
    uint32_t store_op;     /* gbr_store_op */
    double clear_value[4]; /* wgpu::Color (f64) */
    uint32_t depth_slice;
    uint32_t _pad;
} gbr_color_attachment;

typedef struct gbr_depth_attachment {
    gbr_texture view;
    uint32_t has_depth_ops;
    uint32_t depth_load_op;
    uint32_t depth_store_op;
    float depth_clear_value;
} gbr_depth_attachment;

typedef struct gbr_cmd_begin_render_pass {
    uint32_t color_attachment_count;
    uint32_t has_depth_attachment;
    gbr_color_attachment color_attachments[GBR_MAX_COLOR_TARGETS]; /* view 0 = None */
    gbr_depth_attachment depth_attachment;
} gbr_cmd_begin_render_pass;

typedef struct gbr_cmd_set_pipeline { gbr_render_pipeline pipeline; } gbr_cmd_set_pipeline;
typedef struct gbr_cmd_set_bind_group {
    uint32_t index;
    uint32_t dynamic_offset_count; /* dynamic offsets are ignored, as in state.rs:194-205 */
    gbr_bind_group bind_group;     /* 0 = unset */
} gbr_cmd_set_bind_group;
typedef struct gbr_cmd_set_index_buffer {
    gbr_buffer buffer;
    uint32_t index_format;
    uint32_t _pad;
    uint64_t offset;
    uint64_t size; /* 0 = rest of buffer */
} gbr_cmd_set_index_buffer;
typedef struct gbr_cmd_set_vertex_buffer {
    uint32_t slot;
    uint32_t _pad;
    gbr_buffer buffer;
    uint64_t offset;
    uint64_t size; /* 0 = rest of buffer */
} gbr_cmd_set_vertex_buffer;
typedef struct gbr_cmd_set_viewport { float x, y, width, height, min_depth, max_depth; } gbr_cmd_set_viewport;
typedef struct gbr_cmd_set_scissor_rect { uint32_t x, y, width, height; } gbr_cmd_set_scissor_rect;
typedef struct gbr_cmd_set_blend_constant { double color[4]; } gbr_cmd_set_blend_constant;
typedef struct gbr_cmd_draw {
    uint32_t vertex_start, vertex_end;     /* Range<u32> */
    uint32_t instance_start, instance_end; /* Range<u32> */
} gbr_cmd_draw;
typedef struct gbr_cmd_draw_indexed {
    uint32_t index_start, index_end;
    int32_t base_vertex;
    uint32_t instance_start, instance_end;
    uint32_t _pad;
} gbr_cmd_draw_indexed;

/* ---------------------------------------------------------------- entry points */

/* Thread-local text of the last error on this thread; returns the full message length. */
GBR_API size_t gbr_last_error(char* buf, size_t buf_len);
GBR_API uint32_t gbr_abi_version(void);

/* wgpu_cpu::instance (lib.rs:25-27) -> Instance::request_adapter (instance.rs:72-102) ->
 * Adapter::request_device (adapter.rs:24-42) -> create_device_and_queue (device.rs:40-74),
 * which spawns the engine thread (engine.rs:12-24).  One call creates device + queue + worker. */
GBR_API gbr_status gbr_device_create(const gbr_device_config* config, gbr_device* out_device);
/* Drop of Queue / QueueReceiver (device.rs:480-487, 543-549): stops the worker, frees all objects. */
GBR_API gbr_status gbr_device_destroy(gbr_device device);
/* AdapterInterface::limits (adapter.rs:60-62). */
GBR_API gbr_status gbr_device_limits(gbr_device device, gbr_limits* out_limits);

/* DeviceInterface::create_buffer (device.rs:157-159 -> buffer.rs:40-52). */
GBR_API gbr_status gbr_buffer_create(gbr_device device, uint64_t size, uint32_t usage, gbr_buffer* out_buffer);
GBR_API gbr_status gbr_buffer_destroy(gbr_device device, gbr_buffer buffer);
/* QueueInterface::write_buffer (device.rs:332-344).  Ordered with later submissions. */
GBR_API gbr_status gbr_queue_write_buffer(gbr_device device, gbr_buffer buffer, uint64_t offset,
                                          const void* data, uint64_t size);
/* Many QueueInterface::write_buffer calls (device.rs:332-344) in one: the writes are queued in
 * array order, as that many gbr_queue_write_buffer calls would queue them, after every entry has
 * been validated (an invalid entry queues none of them).  Serving loops that upload a fixed set
 * of buffers every frame pass one prepared array instead of crossing the ABI per buffer. */
typedef struct gbr_buffer_write {
    gbr_buffer buffer;
    uint64_t offset;
    const void* data;
    uint64_t size;
} gbr_buffer_write;
GBR_API gbr_status gbr_queue_write_buffers(gbr_device device, uint32_t count, const gbr_buffer_write* writes);
/* BufferInterface::map_async + get_mapped_range for reads (buffer.rs:112-136): waits for all
 * prior submissions, then copies `size` bytes at `offset` into `dst`. */
GBR_API gbr_status gbr_buffer_read(gbr_device device, gbr_buffer buffer, uint64_t offset, void* dst, uint64_t size);

/* DeviceInterface::create_texture (device.rs:161-163 -> texture.rs:34-43). */
GBR_API gbr_status gbr_texture_create(gbr_device device, const gbr_texture_desc* desc, gbr_texture* out_texture);
GBR_API gbr_status gbr_texture_destroy(gbr_device device, gbr_texture texture);
/* QueueInterface::write_texture (device.rs:371-434).  As in the reference, the copy extent
 * is the whole texture and whole rows are copied; `mip_level` > 0 is accepted only by the
 * extension profile (the reference has `todo!` at device.rs:378-380). */
GBR_API gbr_status gbr_queue_write_texture(gbr_device device, gbr_texture texture, uint32_t mip_level,
                                           const void* data, uint64_t data_size,
                                           const gbr_texel_copy_buffer_layout* layout, gbr_extent3d size);
/* wgpu_cpu::image::rgba_texture_image (lib.rs:158-173): waits for prior submissions and
 * copies the whole mip level (tightly packed rows) into `dst`. */
GBR_API gbr_status gbr_texture_read(gbr_device device, gbr_texture texture, uint32_t mip_level, void* dst, uint64_t size);
/* No reference counterpart (readback of many targets): gbr_texture_read for `count` textures in
 * one queue operation — one wait for prior submissions, the copies back to back, one return.
 * dsts[k] receives mip level mips[k] of textures[k] and must hold sizes[k] >= its bytes; pinned
 * destinations (cudaHostAlloc / cudaHostRegister) move at full DMA speed. */
GBR_API gbr_status gbr_textures_read(gbr_device device, uint32_t count, const gbr_texture* textures,
                                     const uint32_t* mip_levels, void* const* dsts, const uint64_t* sizes);
/* CommandEncoder::copy_texture_to_buffer + BufferSlice::map_async (buffer.rs:112-136) for
 * `count` textures, without blocking: validates like gbr_textures_read, enqueues the readback
 * behind every earlier queue operation and returns.  The readback takes the next submission
 * index (*out_index): the destinations hold the bytes once gbr_device_poll(device, 1, 1,
 * *out_index, ...) has returned GBR_OK, and the caller keeps them valid, and does not read them,
 * until then.  A frame loop can so enqueue frame k + 1 while frame k's readback runs. */
GBR_API gbr_status gbr_queue_read_textures(gbr_device device, uint32_t count, const gbr_texture* textures,
                                           const uint32_t* mip_levels, void* const* dsts, const uint64_t* sizes,
                                           uint64_t* out_index);

/* DeviceInterface::create_sampler (device.rs:185-187 -> sampler.rs:4-29). */
GBR_API gbr_status gbr_sampler_create(gbr_device device, const gbr_sampler_desc* desc, gbr_sampler* out_sampler);
GBR_API gbr_status gbr_sampler_destroy(gbr_device device, gbr_sampler sampler);

/* DeviceInterface::create_shader_module (device.rs:91-100 -> shader.rs:31-50): parses and
 * validates WGSL.  Entry points are translated to CUDA C and compiled with NVRTC when a
 * pipeline that uses them is created (shader.rs:52-74 `for_pipeline`). */
GBR_API gbr_status gbr_shader_module_create(gbr_device device, const char* wgsl, uint64_t wgsl_len,
                                            gbr_shader_module* out_module);
/* No reference counterpart: selects one of the library's precompiled CUDA shader programs by
 * name (e.g. "colored_triangle", "mesh_color", "mesh_tex_lambert", "quad_color").  Used to pin
 * the WGSL translator against hand-written programs and by callers without NVRTC. */
GBR_API gbr_status gbr_shader_module_create_native(gbr_device device, const char* name,
                                                   gbr_shader_module* out_module);
GBR_API gbr_status gbr_shader_module_destroy(gbr_device device, gbr_shader_module module);

/* DeviceInterface::create_render_pipeline (device.rs:129-134 -> pipeline.rs:57-76). */
GBR_API gbr_status gbr_render_pipeline_create(gbr_device device, const gbr_render_pipeline_desc* desc,
                                              gbr_render_pipeline* out_pipeline);
GBR_API gbr_status gbr_render_pipeline_destroy(gbr_device device, gbr_render_pipeline pipeline);

/* No reference counterpart (test and tooling entry points of the WGSL translator).
 * gbr_render_pipeline_eval_vertices runs the vertex stage of a WGSL pipeline alone for vertex
 *   indices first..first+count-1 (no vertex buffers, no bindings): per vertex, 4 position
 *   floats followed by 16 inter-stage floats (integer outputs of a vertex-only program as
 *   their bits) in `out`, and 0 or a device error code in `errors`.
 * gbr_wgsl_translate writes the CUDA C a vertex (+ fragment, when fragment_entry is not null)
 *   program translates to; `needed` receives its size including the terminator.
 * gbr_wgsl_compile_check translates and compiles with NVRTC (no GPU needed), returning the log. */
GBR_API gbr_status gbr_render_pipeline_eval_vertices(gbr_device device, gbr_render_pipeline pipeline,
                                                     uint32_t first_vertex, uint32_t count, float* out,
                                                     uint32_t* errors);
GBR_API gbr_status gbr_wgsl_translate(const char* wgsl, uint64_t wgsl_len, const char* vertex_entry,
                                      const char* fragment_entry, char* out, uint64_t capacity, uint64_t* needed);
GBR_API gbr_status gbr_wgsl_compile_check(const char* wgsl, uint64_t wgsl_len, const char* vertex_entry,
                                          const char* fragment_entry, char* log, uint64_t capacity);

/* DeviceInterface::create_bind_group (device.rs:115-120 -> bind_group.rs:58-72,91-117). */
GBR_API gbr_status gbr_bind_group_create(gbr_device device, const gbr_bind_group_desc* desc,
                                         gbr_bind_group* out_bind_group);
GBR_API gbr_status gbr_bind_group_destroy(gbr_device device, gbr_bind_group bind_group);

/* QueueInterface::submit (device.rs:436-462): validates and enqueues one command buffer
 * (the flat stream above) for the worker; returns its submission index.  Never blocks on
 * device work (it may block on HBM admission when the transient budget is exhausted). */
GBR_API gbr_status gbr_queue_submit(gbr_device device, const void* commands, uint64_t commands_len,
                                    uint64_t* out_submission_index);

enum gbr_poll_status { GBR_POLL_WAIT_SUCCEEDED = 0, GBR_POLL_QUEUE_EMPTY = 1, GBR_POLL_POLL = 2 };
/* DeviceInterface::poll (device.rs:237-295).  wait = 0 is PollType::Poll.  With wait = 1 and
 * has_index = 1, waits until `submission_index` is done; with has_index = 0 waits for one
 * more submission to finish, as the reference does.  timeout_ns = UINT64_MAX waits forever.
 * Returns GBR_ERR_TIMEOUT when the wait runs out (PollError::Timeout). */
GBR_API gbr_status gbr_device_poll(gbr_device device, uint32_t wait, uint32_t has_index,
                                   uint64_t submission_index, uint64_t timeout_ns, uint32_t* out_status);

/* Metrics of a finished submission (tracing events in the reference, see struct comment); the
 * newest 16,384 finished submissions stay queryable. */
GBR_API gbr_status gbr_submission_stats_get(gbr_device device, uint64_t submission_index,
                                            gbr_submission_stats* out_stats);
/* No reference counterpart (measurement): device time in milliseconds from the start of
 * submission `first` to the end of submission `last`, from CUDA events on the device stream. */
GBR_API gbr_status gbr_device_elapsed_ms(gbr_device device, uint64_t first_submission, uint64_t last_submission,
                                         double* out_ms);
/* No reference counterpart (serving): the device's HBM use as admission counts it.
 * resident_bytes: live buffers and textures; transient_bytes: the worker's scratch arena
 * (grow-only).  With batch_submissions, the worker merges the submissions queued behind the one
 * it starts while resident_bytes + GBR_ADMISSION_GROUP_BYTES + the sum of their estimates stays
 * within hbm_budget_bytes; a submission is estimated at GBR_ADMISSION_BYTES_PER_PRIMITIVE per
 * primitive slot + one byte per 16 target pixels + 4 KiB.  The first submission of a group always
 * runs; a group whose scratch and the resident resources exceed the budget fails with
 * GBR_ERR_OUT_OF_MEMORY. */
#define GBR_ADMISSION_GROUP_BYTES (64ull << 20)
#define GBR_ADMISSION_BYTES_PER_PRIMITIVE 512u
GBR_API gbr_status gbr_device_memory(gbr_device device, uint64_t* out_resident_bytes, uint64_t* out_transient_bytes);
/* No reference counterpart (measurement): enqueues a write of a 256 MiB scratch buffer on the
 * device stream, evicting the L2 cache between timed submissions. */
GBR_API gbr_status gbr_device_flush_caches(gbr_device device);
/* No reference counterpart (verification): runs `samples` seeded quotients through the
 * raster kernels' division by a precomputed reciprocal (exact.cuh, div_by_recip) on the current
 * CUDA device and counts results whose bits differ from CUDA's __fdiv_rn.  The same samples go
 * through the packed f32x2 helpers (f2add, f2mul, f2fma, and a packed product feeding a packed
 * sum), which must give the bits of the scalar __fadd_rn / __fmul_rn / __fmaf_rn, and seeded
 * integer pairs through the span rule's truncating division (div_trunc_span), which must equal
 * exact integer division.  `first_mismatch` receives (a, b) of the first difference found, if any. */
GBR_API gbr_status gbr_selftest_division(uint64_t samples, uint64_t seed, uint64_t* out_mismatches,
                                         float* first_mismatch);

/* ---------------------------------------------------------------- allocation-free rendering
 *
 * No counterpart in the reference: wgpu-cpu has no entry point of this kind.
 *
 * gbr_render_triangles_noalloc draws a non-indexed triangle list whose vertices are already in
 * clip space into caller-owned device memory, and allocates no memory at all: no cudaMalloc,
 * no cudaFree, no allocating library routine.  It is meant for callers that cannot allocate
 * device memory themselves or let a library do it: a plugin running inside a host application
 * that owns every byte of the device, or a frame loop that must not take the implicit device
 * synchronisation that cudaMalloc/cudaFree perform.
 *
 * The rasterisation is the same as the device/queue path's (same kernels, same bit-exact
 * coverage, interpolation, depth test and Rgba8Unorm encoding, parity profile): the per-vertex
 * colour is interpolated linearly and written as the fragment colour.  Its scratch space
 * (triangle records, tile bins, counters) is one fixed array in the library's device memory,
 * GBR_NOALLOC_SCRATCH_BYTES large, which every GPU that loads the library keeps until the
 * process exits.  Limits: at most GBR_NOALLOC_MAX_TRIANGLES triangles, targets of at most
 * GBR_NOALLOC_MAX_DIM x GBR_NOALLOC_MAX_DIM pixels, and at most GBR_NOALLOC_MAX_CLIPPED extra
 * sub-triangles from clipping and GBR_NOALLOC_MAX_BIN_ENTRIES triangle/tile pairs; beyond
 * them the call returns GBR_ERR_OUT_OF_MEMORY with a message saying which limit was hit, and
 * the targets are left unchanged.
 *
 * Every call shares that one scratch array and overwrites what the previous call left there,
 * so calls whose GPU work overlaps (two host threads, or two streams) race with each other:
 * serialise them.  The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream capture.  Every
 * call ends by reading its status back to the host and waiting for `stream`, so it returns after
 * the work on `stream` has finished, and it cannot be made while `stream` is being captured
 * into a CUDA graph.  color_load_op and depth_load_op must be GBR_LOAD_OP_LOAD or
 * GBR_LOAD_OP_CLEAR (anything else returns GBR_ERR_INVALID_ARGUMENT).
 *
 *   clip_positions  device pointer, 3 * triangle_count float4 (x, y, z, w), 16-byte aligned
 *   colors          device pointer, 3 * triangle_count float4 (r, g, b, a), 16-byte aligned
 *   color_target    device pointer, width * height Rgba8Unorm texels, 4-byte aligned
 *   depth_target    device pointer to width * height f32 (Depth32Float), or NULL for none
 *   stream          a cudaStream_t, or NULL for the default stream
 */
#define GBR_NOALLOC_SCRATCH_BYTES (24u << 20)
#define GBR_NOALLOC_MAX_TRIANGLES 32768u
#define GBR_NOALLOC_MAX_CLIPPED 8192u
#define GBR_NOALLOC_MAX_DIM 2048u
#define GBR_NOALLOC_MAX_BIN_ENTRIES 3800000u

typedef struct gbr_noalloc_state {
    uint32_t cull_mode;           /* gbr_cull_mode */
    uint32_t front_face;          /* gbr_front_face */
    uint32_t depth_compare;       /* gbr_compare_function, used when depth_target != NULL */
    uint32_t depth_write_enabled;
    uint32_t color_load_op;       /* gbr_load_op */
    uint32_t depth_load_op;       /* gbr_load_op */
    float clear_color[4];
    float clear_depth;
    uint32_t _pad;
} gbr_noalloc_state;

GBR_API gbr_status gbr_render_triangles_noalloc(const float* clip_positions, const float* colors,
                                                uint32_t triangle_count, uint8_t* color_target, float* depth_target,
                                                uint32_t width, uint32_t height, const gbr_noalloc_state* state,
                                                void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBR_H */
