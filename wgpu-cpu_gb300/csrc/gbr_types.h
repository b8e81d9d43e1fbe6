// gbr_types.h — plain-old-data structures shared by the host runtime and the CUDA kernels of
// the render-pass path.  Everything here is device-resident per launch batch.
#pragma once

#ifdef __CUDACC_RTC__
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
typedef unsigned long long uintptr_t;
#else
#include <stdint.h>
#endif

#ifdef __CUDACC__
#define GBR_HD __host__ __device__
#else
#define GBR_HD
#endif

namespace gbr {

enum : uint32_t {
    MAX_VARYING_LOCATIONS = 4,  // inter-stage @location slots carried per vertex
    MAX_VARYING_FLOATS = 16,    // 4 locations x vec4
    SUBTRI_BITS = 6,            // a clipped triangle yields at most 2^6 sub-triangles
};

// Native shader programs compiled into the library (the same WGSL programs as
// shaders/*.wgsl, written by hand in CUDA).
enum Program : uint32_t {
    PROG_COLORED_TRIANGLE = 0,
    PROG_MESH_COLOR = 1,
    PROG_MESH_COLOR_PERSPECTIVE = 2,
    PROG_MESH_COLOR_DISCARD = 3,
    PROG_MESH_TEX_LAMBERT = 4,
    PROG_QUAD_COLOR = 5,
    PROG_CLIP_PASSTHROUGH = 6,
    PROG_JIT = 7,  // a WGSL program compiled into its own module (jit_vs / jit_fs)
    PROG_CLIP_FLAT = 8,     // clip_passthrough with the colour @interpolate(flat)
    PROG_CLIP_FLAT_ID = 9,  // an integer @interpolate(flat) vertex id and a linear colour
    PROG_CLIP_DISCARD = 10, // clip_passthrough that discards where red < 0.5
    PROG_COUNT = 11
};

// @early_depth_test of a fragment entry point (naga::EarlyDepthTest, read by
// render_pass/fragment.rs:83-86, 166-194): none = the late test only, Force = the early test
// only, Allow = the early test and then the late test again at the colour output.
enum EarlyDepth : uint32_t { EARLY_DEPTH_NONE = 0, EARLY_DEPTH_FORCE = 1, EARLY_DEPTH_ALLOW = 2 };

enum Interp : uint8_t { INTERP_LINEAR = 0, INTERP_PERSPECTIVE = 1, INTERP_FLAT = 2 };

enum ErrorCode : uint32_t {
    ERR_NONE = 0,
    ERR_W_ZERO = 1,            // clip position w == 0 (primitive.rs:177, raster.rs:146)
    ERR_INDEX_OOB = 2,         // index buffer read out of range
    ERR_VERTEX_OOB = 3,        // vertex attribute read out of range
    ERR_BASE_VERTEX = 4,       // index + base_vertex overflows u32 (index.rs:55-57)
    ERR_OVERFLOW_RECORDS = 5,  // more clipped sub-triangles than scratch slots (retried)
    ERR_OVERFLOW_BINS = 6,     // more tile entries than scratch slots (retried)
    ERR_SPAN_RANGE = 7,        // scanline coordinate outside u32 (scanline.rs:156-170)
    ERR_UNSUPPORTED = 8,
    ERR_SHADER_TRAP = 9,  // a shader divided an integer by zero (EntryPointError::DivisionByZero)
};

// gbr_texture_format values the kernels test (gbr.h is not seen by NVRTC modules), and the
// colour-target codes of sRGB targets in the extension profile, which encode linear -> sRGB on
// write and decode on blending reads (the parity profile writes Srgb formats as Unorm).
enum : uint32_t {
    TEXFMT_RGBA8_UNORM_SRGB = 4,
    TFMT_RGBA8_SRGB_ENCODE = 20,
    TFMT_BGRA8_SRGB_ENCODE = 21,
};

// One texture binding as seen by the kernels.
struct TexDesc {
    const uint8_t* data;  // mip 0 .. mip n-1 back to back
    uint32_t width, height;
    uint32_t format;      // gbr_texture_format
    uint32_t mip_count;
    uint64_t mip_offset[16];
};

struct SamplerDescDev {
    uint32_t address_u, address_v;
    uint32_t mag_filter, min_filter, mip_filter;
    float lod_min, lod_max;
    uint32_t _pad;
};

// Where one vertex-shader input location comes from.
struct AttrDesc {
    int32_t buffer;   // -1 = absent
    uint32_t format;  // gbr_vertex_format
    uint32_t offset;
    uint32_t _pad;
};

// A colour/depth target of a batch.
struct TargetDesc {
    uint8_t* color;        // null = no colour attachment
    float* depth;          // null = no depth attachment
    uint32_t width, height;
    uint32_t color_format; // gbr_texture_format
    uint32_t color_bpp;
    uint32_t color_load;   // 1 = clear
    uint32_t depth_load;   // 1 = clear, 0 = load, 2 = no depth ops (load)
    float clear[4];        // colour clear value (f32, from wgpu::Color f64)
    float depth_clear;
    uint32_t tiles_x, tiles_y;
    uint32_t tile_base;    // first global tile id of this target
    uint32_t slice_offset; // byte offset of the depth_slice layer
    uint32_t _pad;
    // three counters of this target (or null): [0] covered fragments, counted as the reference
    // counts fragment_processing calls; [1] fragment-stage invocations; [2] those of programs
    // that sample a texture
    unsigned long long* frag_count;
};

// One draw call of a batch, fully resolved on the host.
struct DrawDesc {
    // primitive stream
    uint32_t topology;       // gbr_primitive_topology
    uint32_t index_format;   // 0 = direct draw, 1 = u16, 2 = u32
    uint32_t first;          // first vertex (direct) or first index
    uint32_t count;          // vertex / index count
    int32_t base_vertex;
    uint32_t instance_start;
    uint32_t instance_count;
    uint32_t prims_per_instance;
    uint32_t prim_base;      // first global primitive id of this draw in the batch
    uint32_t target;         // index into the batch's TargetDesc array
    const uint8_t* index_data;
    uint64_t index_bytes;
    // vertex buffers
    const uint8_t* vb_data[8];
    uint64_t vb_size[8];
    uint32_t vb_stride_vertex[8];
    uint32_t vb_stride_instance[8];
    AttrDesc attr[16];
    // bindings
    const uint8_t* uniform[4][8];
    uint64_t uniform_size[4][8];
    TexDesc tex;             // the one texture binding native programs use (group 1, binding 0)
    SamplerDescDev samp;     // group 1, binding 1
    // programs
    uint32_t program;        // Program (VS and FS come from the same native module)
    uint32_t has_fragment;
    uint32_t num_varyings;   // floats per vertex carried to the FS
    uint32_t profile;        // gbr_profile
    // raster state
    uint32_t cull_mode, front_face;
    float vp_tx, vp_ty, vp_sx, vp_sy;
    uint32_t sc_x0, sc_y0, sc_x1, sc_y1;  // scissor [x0, x1) x [y0, y1)
    uint32_t depth_test;                  // pipeline has depth state AND target has depth
    uint32_t depth_compare, depth_write;
    uint32_t blend_enabled;
    uint32_t blend_color[3], blend_alpha[3];  // src, dst, op
    uint32_t write_mask;
    float blend_constant[4];
    // setup
    uint32_t fast_vs;        // FastVs: the vertex stage the fast setup path runs, or FAST_VS_NONE
    uint32_t interp;         // INTERP_LINEAR / INTERP_PERSPECTIVE of the program's inter-stage values
    uint32_t may_discard;    // the fragment stage can discard
    uint32_t strip_restart;  // triangle strip with primitive restart (separator indices)
    uint32_t strip_table;    // first entry of this draw's strip table in BatchParams::strip_info
    uint32_t lod_var;        // extension-profile sampling: 1 + varying index of u (v follows), 0 = none
    uint32_t raster_rule;    // RASTER_RULE_SCANLINE / RASTER_RULE_EDGE
    uint32_t fast_vcount;    // fast setup: every vertex index below this fetches its FastVs attributes in range
    uint32_t flat_mask;      // bit k: inter-stage float k is @interpolate(flat) (vertex 0's value, bits kept)
    uint32_t early_depth;    // EarlyDepth of the fragment entry point
    // fast setup of FAST_VS_MVP_COLOR / FAST_VS_MVP_TEX: 1 when the shape's attributes are one
    // per-vertex buffer's whole vertex, packed from offset 0 (stride 24 / 32) in an 8- / 16-byte
    // aligned buffer, so each vertex is read with 8- / 16-byte loads
    uint32_t fast_packed;
    uint32_t _pad_setup[3];
};

// Vertex stages the fast setup kernel specialises on: every input an f32 attribute of exactly
// the program's width.  Anything else (other formats, clipping, errors) goes through the
// generic setup kernel.
enum FastVs : uint32_t {
    FAST_VS_NONE = 0,
    FAST_VS_MVP_COLOR = 1,  // mesh_color*: f32x3 position, f32x3 colour, MVP from group 0
    FAST_VS_MVP_TEX = 2,    // mesh_tex_lambert: f32x3 position, f32x3 normal, f32x2 uv
    FAST_VS_QUAD = 3,       // quad_color: f32x3 position, f32x4 colour
    FAST_VS_CLIP = 4,       // clip_passthrough: f32x4 clip position, f32x4 colour
    FAST_VS_TRIANGLE = 5,   // colored_triangle: no inputs
    FAST_VS_QUAD_F16 = 6,   // quad_color, extension profile: f32x3 position, f16x4 colour
};

// Per-sub-triangle record written by the setup kernel and read by binning and raster.
// Fixed header followed by 3 x num_varyings floats (stride set per batch).
struct TriRecord {
    uint32_t key;        // global order key: prim << SUBTRI_BITS | sub
    uint32_t draw;
    uint32_t prim_index; // per-instance primitive index (the @builtin(primitive_index))
    uint32_t flags;      // bit 0 front_facing, bit 1 empty, bits 2-3 span mode
    int32_t row0, row1;  // rows emitted by the scanline state machine (inclusive)
    int32_t xmin, xmax;  // min / max framebuffer x of the three vertices
    int32_t sx[3], sy[3];// framebuffer vertices sorted by y (bubblesort3 order)
    float vpx[3], vpy[3];// viewport coordinates of rasterize()'s a, b, c
    float area;          // total_area (shoelace of a, b, c)
    float fz[3], fw[3];  // fragment z and 1/w of a, b, c
    float cb[9];         // clip barycentrics of a, b, c (3 x 3)
    float inv_w0[3];     // 1/w of the unclipped vertices (perspective interpolation)
    uint32_t ovf;        // primary record: first overflow slot of sub-triangles 1..nsub-1
    uint32_t nsub;       // primary record: number of sub-triangles
    float lod;           // extension-profile texture LOD of the draw's sampler (0 without one)
    uint32_t _pad[2];
    // float var[3][num_varyings] follows (16-byte aligned: vector loads of the varyings)
};
static_assert(sizeof(TriRecord) % 16 == 0, "varyings start on a 16-byte boundary");

enum : uint32_t {
    TRI_RECORD_HEADER_BYTES = sizeof(TriRecord),
    SPAN_DEGENERATE = 1,  // all three vertices on one row: single span xmin..xmax
    SPAN_EDGE = 2,        // edge-function rule: pixel centres, top-left, 8-bit sub-pixel snapping
};

// How triangles cover pixels (gbr_raster_rule): the reference's scanline walk at integer pixel
// corners, or (extension profile) fixed-point edge functions at pixel centres.
enum : uint32_t { RASTER_RULE_SCANLINE = 0, RASTER_RULE_EDGE = 1 };

// Device-side status of a batch (zeroed before launch).
constexpr uint32_t kTargetCounters = 3;  // per-target counters behind TargetDesc::frag_count

struct BatchStatus {
    uint32_t error;
    uint32_t error_detail;
    uint32_t ovf_used;        // overflow record slots used (may exceed capacity -> retry)
    uint32_t slow_count;      // primitives queued for the generic setup kernel
    unsigned long long bin_entries;   // tile entries needed
    unsigned long long fragments;     // fragment-shader invocations
    unsigned long long primitives;    // primitives assembled
    uint32_t split_items;     // visibility raster: chunk work items of the split tiles (k_scan)
    uint32_t _pad_s;
};

// Visibility raster: a tile binned more than BatchParams::split_chunk records (VIS_SPLIT_CHUNK
// unless the device is told otherwise) is rasterised as chunks of that many records, one work
// item each, taken ahead of the other tiles; each chunk leaves its survivor keys in global memory
// and the last chunk to finish merges them and shades the tile.
constexpr uint32_t VIS_SPLIT_CHUNK = 2048;

// Bits of the global tile index in a setup binning hint (BatchParams::tile_hint).
constexpr uint32_t TILE_HINT_TILE_BITS = 26;

struct BatchParams {
    const DrawDesc* draws;
    const TargetDesc* targets;
    uint32_t num_draws;
    uint32_t num_targets;
    uint32_t total_prims;     // sum over draws of prims_per_instance * instance_count
    uint32_t total_tiles;
    uint32_t tile_size;       // T
    uint32_t tile_shift;      // log2(T)
    uint32_t record_stride;   // bytes per record
    uint32_t num_varyings;    // max floats per vertex over the batch's programs
    uint8_t* records;         // total_prims primary records
    uint8_t* ovf_records;     // overflow records
    uint32_t ovf_capacity;
    uint32_t bin_capacity;    // entries in `bins`
    uint32_t* tile_count;     // [total_tiles + 1]
    uint32_t* tile_offset;    // [total_tiles + 1]
    uint32_t* tile_cursor;    // [total_tiles]
    uint32_t* bins;           // keys
    uint32_t* work_counter;   // persistent raster work queue
    BatchStatus* status;
    uint32_t* abort_flag;        // set by a failed batch; later batches of the submission skip
    uint32_t* slow_prims;        // [total_prims] primitives the fast setup path hands on
    uint32_t* tile_hint;         // [total_prims] binning hint per primary record (null: none), TILE_HINT_*
    uint32_t* strip_info;        // strip tables of the restart draws (null when there are none)
    void* states;                // visibility raster: per-draw fragment-stage state (RasterState)
    uint32_t vis_compare;        // visibility raster: the batch's depth compare function
    uint32_t raster_rule;        // RASTER_RULE_*: which instantiation of the kernels runs the batch
    // visibility raster, split tiles (split_heavy null: no tile is split)
    uint32_t* split_tile;        // [total_tiles] for a tile over split_chunk records: its heavy-list index, ~0 = not split
    uint32_t* split_heavy;       // [split_cap_heavy][4] per split tile: tile, chunks, first work item, chunks finished
    uint32_t* split_item;        // [split_cap_items] heavy-list index of each chunk work item
    unsigned long long* split_keys;  // [split_cap_items][T * T] survivor keys each chunk leaves
    uint32_t split_cap_heavy, split_cap_items;
    uint32_t split_chunk;        // records per chunk work item (> 0 when split_heavy is set)
    uint32_t fvs_mask;           // bit f: a draw of the batch has FastVs shape f (0: unknown, one generic setup launch)
    // draw-aligned setup groups per FastVs shape f: entries [sg_off[f], sg_off[f + 1]) of
    // shape_groups are pairs (draw, first 32-primitive group of the draw, counted over the shape's
    // draws in batch order), the last pair (~0, the shape's group count); none when no draw of the
    // shape has primitives
    const uint32_t* shape_groups;
    uint32_t sg_off[8];
    const uint32_t* draw_base;   // [num_draws] prim_base of each draw, contiguous (null: read the descriptors)
    uint32_t slow_builds_states; // k_setup_slow also builds the visibility raster's per-draw states
};

}  // namespace gbr
