// kernels.cu — instantiates the render-pass kernels for the supported tile shapes under the
// reference's raster rule (kernels_edge.cu: the edge-function rule) and launches one batch
// (setup -> scan -> fill -> raster) on a stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "gbr.h"
#include "kernels.h"
#include "launch.cuh"
#include "raster_lines.cuh"

namespace gbr {

extern template cudaError_t launch_batch_t<true>(const BatchParams&, int, int, int, cudaStream_t, uint32_t*,
                                                 cudaEvent_t*, int);


size_t raster_state_bytes() { return sizeof(RasterState); }

// One block per segment (grid-stride over segments): 16-byte copies where the destination, the
// source and the size allow, else 4-byte, else bytes.
__global__ void __launch_bounds__(256) k_scatter_writes(const uint64_t* desc, uint32_t n) {
    for (uint32_t seg = blockIdx.x; seg < n; seg += gridDim.x) {
        uint8_t* dst = reinterpret_cast<uint8_t*>(desc[3 * seg]);
        const uint8_t* src = reinterpret_cast<const uint8_t*>(desc[3 * seg + 1]);
        const uint64_t size = desc[3 * seg + 2];
        const uintptr_t a = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src);
        if ((a & 15) == 0 && (size & 15) == 0) {
            for (uint64_t k = threadIdx.x; k < size / 16; k += blockDim.x)
                reinterpret_cast<uint4*>(dst)[k] = reinterpret_cast<const uint4*>(src)[k];
        } else if ((a & 3) == 0 && (size & 3) == 0) {
            for (uint64_t k = threadIdx.x; k < size / 4; k += blockDim.x)
                reinterpret_cast<uint32_t*>(dst)[k] = reinterpret_cast<const uint32_t*>(src)[k];
        } else {
            for (uint64_t k = threadIdx.x; k < size; k += blockDim.x) dst[k] = src[k];
        }
    }
}
cudaError_t launch_scatter_writes(const uint64_t* desc, uint32_t n, cudaStream_t s) {
    if (!n) return cudaSuccess;
    k_scatter_writes<<<n < 1024u ? n : 1024u, 256, 0, s>>>(desc, n);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) k_copy_out(CopyOutJobs j) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (uint64_t)gridDim.x * blockDim.x;
    for (uint32_t k = 0; k < j.n; ++k) {
        const uint64_t n16 = j.bytes[k] >> 4;
        const uint4* src = reinterpret_cast<const uint4*>(j.src[k]);
        uint4* dst = reinterpret_cast<uint4*>(j.dst[k]);
        for (uint64_t i = t; i < n16; i += nt) dst[i] = src[i];
        for (uint64_t i = (n16 << 4) + t; i < j.bytes[k]; i += nt) j.dst[k][i] = j.src[k][i];
    }
}
cudaError_t launch_copy_out(const CopyOutJobs& jobs, int num_sms, cudaStream_t s) {
    if (!jobs.n) return cudaSuccess;
    k_copy_out<<<num_sms * 4, 256, 0, s>>>(jobs);
    return cudaGetLastError();
}

cudaError_t launch_lines(const BatchParams& bp, int num_sms, cudaStream_t s, uint32_t* launches, cudaEvent_t* ev_raster) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(bp.status, 0, sizeof(BatchStatus), s)) != cudaSuccess) return e;
    unsigned int ev_flags = cudaEventRecordDefault;
    if (ev_raster) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return e;
        if (cs == cudaStreamCaptureStatusActive) ev_flags = cudaEventRecordExternal;
    }
    k_clear_targets<<<num_sms * 4, 256, 0, s>>>(bp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (ev_raster && (e = cudaEventRecordWithFlags(ev_raster[0], s, ev_flags)) != cudaSuccess) return e;
    k_lines_points<<<1, kLineThreads, 0, s>>>(bp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    *launches += 2;
    if (ev_raster) e = cudaEventRecordWithFlags(ev_raster[1], s, ev_flags);
    return e;
}
size_t setup_stage_bytes_host(uint32_t record_stride) { return setup_stage_bytes(record_stride); }
size_t ordered_raster_smem_host(int warps, uint32_t record_stride) {
    return (launch_detail::kCap + 2 * (size_t)warps * 32) * sizeof(uint32_t) + (size_t)launch_detail::kRW * record_stride;
}

// Seeded inputs for the arithmetic self-test: random bit patterns, raster-like magnitudes,
// exact multiples and neighbours of powers of two, in rotation.
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ float selftest_value(uint64_t r, uint32_t kind) {
    const uint32_t lo = (uint32_t)r, hi = (uint32_t)(r >> 32);
    switch (kind & 3u) {
        case 0: return __uint_as_float(lo);                                      // any bit pattern
        case 1: return (float)((int32_t)(lo & 0x3FFFFFF) - 0x2000000) * 0.013f;  // pixel-scale values
        case 2: return __uint_as_float((lo & 0x807FFFFFu) | ((100u + (hi & 63u)) << 23));
        default: return ldexpf(1.0f + (float)(lo & 7u) * 0x1p-23f * (hi & 1u ? -1.0f : 1.0f), (int)(hi % 80u) - 40);
    }
}
__global__ void k_selftest_division(uint64_t n, uint64_t seed, unsigned long long* mismatches, float* first) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t r0 = splitmix64(seed ^ (i * 2 + 0)), r1 = splitmix64(seed ^ (i * 2 + 1));
        const float a = selftest_value(r0, (uint32_t)(i & 3u));
        float b = selftest_value(r1, (uint32_t)((i >> 2) & 3u));
        if ((i >> 4) % 5u == 0) b = __fmul_rn(a, (float)(1 + (r1 & 15)));  // quotients 1/k
        const float y = __frcp_rn(b);
        const float q = div_by_recip(a, b, y, div_fast_ok(b));
        const float ref = __fdiv_rn(a, b);
        // the setup kernel also takes RN(1/w) from __frcp_rn for the reference's `1.0 / w`
        const float one_over = __fdiv_rn(1.0f, b);
        // packed f32x2 helpers against the scalar operations, and scalar products feeding a
        // packed sum (f2mul_rn + f2add), which must keep both roundings
        const float c = selftest_value(splitmix64(r0 ^ (r1 << 1)), (uint32_t)((i >> 6) & 3u));
        const float2 pm = f2mul(make_float2(a, c), make_float2(c, b));
        const float2 ps = f2add(f2mul_rn(make_float2(a, b), make_float2(b, c)), make_float2(c, a));
        const float2 pf = f2fma(make_float2(a, c), make_float2(b, a), make_float2(c, b));
        const float sm[2] = {__fmul_rn(a, c), __fmul_rn(c, b)};
        const float ss[2] = {__fadd_rn(__fmul_rn(a, b), c), __fadd_rn(__fmul_rn(b, c), a)};
        const float sf[2] = {__fmaf_rn(a, b, c), __fmaf_rn(c, a, b)};
        auto bits_eq = [](float u, float v) { return __float_as_uint(u) == __float_as_uint(v) || (u != u && v != v); };
        const bool packed_same = bits_eq(pm.x, sm[0]) && bits_eq(pm.y, sm[1]) && bits_eq(ps.x, ss[0]) &&
                                 bits_eq(ps.y, ss[1]) && bits_eq(pf.x, sf[0]) && bits_eq(pf.y, sf[1]);
        // the span rule's integer division: div_trunc_span against exact integer division, for
        // |n|, d < 2^22 (its fast path) and beyond, with exact multiples of d and their neighbours
        const int64_t dd = ((int64_t)((r1 >> 20) & 0x3FFFFF) >> ((r0 >> 59) % 22u)) + 1;
        int64_t nn = (int64_t)((r0 >> 10) & 0x7FFFFF) - 0x3FFFFF;
        if ((i & 7u) == 0) nn = (nn / dd) * dd + (int64_t)(r1 & 3u) - 1;
        if ((i & 63u) == 1) nn *= 1 + (int64_t)(r1 & 1023u);  // past the fast path's range
        const int64_t exact = nn >= INT32_MIN && nn <= INT32_MAX ? (int64_t)((int32_t)nn / (int32_t)dd) : nn / dd;
        const bool int_same = div_trunc_span(nn, dd) == exact;
        const bool same = bits_eq(q, ref) && bits_eq(y, one_over) && packed_same && int_same;
        if (!same && atomicAdd(mismatches, 1ull) == 0ull) {
            first[0] = a;
            first[1] = b;
        }
    }
}

bool raster_config_supported(int tile, int warps) {
    return launch_detail::ordered_config_supported(tile, warps) || launch_detail::vis_config_supported(tile, warps);
}

uint32_t batch_kernel_launches(uint32_t total_prims, int tile, int warps, int kind, uint32_t fvs_mask) {
    if (kind == 3 && !launch_detail::vis_config_supported(tile, warps)) kind = 0;
    // scan + raster, one setup launch per FastVs shape (one when unknown) + generic setup + fill
    // when there are primitives, the states of the visibility raster when there are none (the
    // generic setup builds them otherwise; the strip table is counted by the caller)
    const uint32_t setups = fvs_mask ? (uint32_t)__builtin_popcount(fvs_mask) : 1u;
    return 2u + (total_prims ? setups + 2u : 0u) + (kind == 3 && !total_prims ? 1u : 0u);
}

uint32_t fast_vs_kind(const DrawDesc& d) {
    if (d.strip_restart) return FAST_VS_NONE;  // the strip table is read by the generic setup
    auto f32 = [&](int loc, uint32_t fmt) {
        const AttrDesc& a = d.attr[loc];
        return a.buffer >= 0 && a.format == fmt && a.offset % 4 == 0 && d.vb_stride_vertex[a.buffer] % 4 == 0 &&
               d.vb_stride_instance[a.buffer] % 4 == 0 && reinterpret_cast<uintptr_t>(d.vb_data[a.buffer]) % 4 == 0;
    };
    switch (d.program) {
        case PROG_MESH_COLOR:
        case PROG_MESH_COLOR_PERSPECTIVE:
        case PROG_MESH_COLOR_DISCARD:
            return f32(0, GBR_VERTEX_FORMAT_FLOAT32X3) && f32(1, GBR_VERTEX_FORMAT_FLOAT32X3) ? FAST_VS_MVP_COLOR
                                                                                               : FAST_VS_NONE;
        case PROG_MESH_TEX_LAMBERT:
            return f32(0, GBR_VERTEX_FORMAT_FLOAT32X3) && f32(1, GBR_VERTEX_FORMAT_FLOAT32X3) &&
                           f32(2, GBR_VERTEX_FORMAT_FLOAT32X2)
                       ? FAST_VS_MVP_TEX
                       : FAST_VS_NONE;
        case PROG_QUAD_COLOR: {
            if (!f32(0, GBR_VERTEX_FORMAT_FLOAT32X3)) return FAST_VS_NONE;
            if (f32(1, GBR_VERTEX_FORMAT_FLOAT32X4)) return FAST_VS_QUAD;
            const AttrDesc& a = d.attr[1];
            const bool h = a.buffer >= 0 && a.format == GBR_VERTEX_FORMAT_FLOAT16X4 && a.offset % 2 == 0 &&
                           d.vb_stride_vertex[a.buffer] % 2 == 0 && d.vb_stride_instance[a.buffer] % 2 == 0 &&
                           reinterpret_cast<uintptr_t>(d.vb_data[a.buffer]) % 2 == 0;
            return h && d.profile == GBR_PROFILE_EXTENSION ? FAST_VS_QUAD_F16 : FAST_VS_NONE;
        }
        case PROG_CLIP_PASSTHROUGH:
        case PROG_CLIP_FLAT:
        case PROG_CLIP_DISCARD:
            return f32(0, GBR_VERTEX_FORMAT_FLOAT32X4) && f32(1, GBR_VERTEX_FORMAT_FLOAT32X4) ? FAST_VS_CLIP
                                                                                               : FAST_VS_NONE;
        case PROG_COLORED_TRIANGLE: return FAST_VS_TRIANGLE;
        default: return FAST_VS_NONE;
    }
}

uint32_t fast_vs_packed(const DrawDesc& d) {
    if (d.fast_vs != FAST_VS_MVP_COLOR && d.fast_vs != FAST_VS_MVP_TEX) return 0;
    const bool tex = d.fast_vs == FAST_VS_MVP_TEX;
    const int b = d.attr[0].buffer;
    if (b < 0 || d.attr[0].offset != 0 || d.attr[1].buffer != b || d.attr[1].offset != 12) return 0;
    if (tex && (d.attr[2].buffer != b || d.attr[2].offset != 24)) return 0;
    if (d.vb_stride_vertex[b] != (tex ? 32u : 24u) || d.vb_stride_instance[b] != 0) return 0;
    return reinterpret_cast<uintptr_t>(d.vb_data[b]) % (tex ? 16u : 8u) == 0 ? 1u : 0u;
}

uint32_t fast_vs_vcount(const DrawDesc& d) {
    // (location, bytes) of the attributes each FastVs shape fetches, as fast_vertex_in_range
    struct Use { int loc; uint32_t bytes; };
    Use u[3];
    int n = 0;
    switch (d.fast_vs) {
        case FAST_VS_MVP_COLOR: u[n++] = {0, 12}; u[n++] = {1, 12}; break;
        case FAST_VS_MVP_TEX: u[n++] = {0, 12}; u[n++] = {1, 12}; u[n++] = {2, 8}; break;
        case FAST_VS_QUAD: u[n++] = {0, 12}; u[n++] = {1, 16}; break;
        case FAST_VS_QUAD_F16: u[n++] = {0, 12}; u[n++] = {1, 8}; break;
        case FAST_VS_CLIP: u[n++] = {0, 16}; u[n++] = {1, 16}; break;
        case FAST_VS_TRIANGLE: return 0xFFFFFFFFu;
        default: return 0;
    }
    // the last instance reads furthest (instance strides are not negative)
    const uint64_t inst = d.instance_count ? (uint64_t)d.instance_start + d.instance_count - 1 : d.instance_start;
    uint64_t count = 0xFFFFFFFFull;
    for (int k = 0; k < n; ++k) {
        const AttrDesc& a = d.attr[u[k].loc];
        if (a.buffer < 0) return 0;
        const uint64_t base = inst * d.vb_stride_instance[a.buffer] + a.offset + u[k].bytes;
        const uint64_t size = d.vb_size[a.buffer];
        if (base > size) return 0;
        const uint64_t stride = d.vb_stride_vertex[a.buffer];
        if (stride) count = std::min<uint64_t>(count, (size - base) / stride + 1);
    }
    return (uint32_t)count;
}

cudaError_t launch_batch(const BatchParams& bp, int tile, int warps, int num_sms, cudaStream_t s,
                         uint32_t* launches, cudaEvent_t* ev_raster, int kind) {
    return bp.raster_rule == RASTER_RULE_EDGE ? launch_batch_t<true>(bp, tile, warps, num_sms, s, launches, ev_raster, kind)
                                              : launch_batch_t<false>(bp, tile, warps, num_sms, s, launches, ev_raster, kind);
}

}  // namespace gbr

// ============================================================================================
// gbr_render_triangles_noalloc: the render-pass kernels above, with every byte of scratch taken
// from one file-scope device array instead of allocated memory (see include/gbr.h).
#include <cstdio>
#include <cstring>

#include "gbr.h"

namespace gbr {
void set_thread_error(const char* msg);  // runtime.cu: the text gbr_last_error() returns
}

namespace {

using namespace gbr;

// The whole scratch of the allocation-free entry point.  It lives in the library's device
// memory on every GPU that loads the library, until the process exits.
static __device__ __align__(256) uint8_t g_noalloc_scratch[GBR_NOALLOC_SCRATCH_BYTES];

// Layout of g_noalloc_scratch (byte offsets).
constexpr size_t kNaAbort = 0, kNaStatus = 256, kNaWork = 512, kNaDraw = 1024, kNaTarget = 4096;
constexpr size_t kNaTiles = 8192, kNaRecords = 262144;
constexpr uint32_t kNaVaryings = 4;  // clip_passthrough carries one vec4f colour
constexpr uint32_t kNaStride = (uint32_t)((sizeof(TriRecord) + 3 * kNaVaryings * sizeof(float) + 15) & ~size_t(15));
constexpr size_t kNaOvf = kNaRecords + (size_t)GBR_NOALLOC_MAX_TRIANGLES * kNaStride;
constexpr size_t kNaBins = kNaOvf + (size_t)GBR_NOALLOC_MAX_CLIPPED * kNaStride;
constexpr size_t kNaSlow = kNaBins + (size_t)GBR_NOALLOC_MAX_BIN_ENTRIES * sizeof(uint32_t);
constexpr uint32_t kNaTile = 16, kNaWarps = 8;
constexpr uint32_t kNaMaxTiles = (GBR_NOALLOC_MAX_DIM / kNaTile) * (GBR_NOALLOC_MAX_DIM / kNaTile);
static_assert(sizeof(DrawDesc) <= kNaTarget - kNaDraw, "DrawDesc does not fit its slot");
static_assert(sizeof(TargetDesc) <= kNaTiles - kNaTarget, "TargetDesc does not fit its slot");
static_assert(kNaTiles + 3 * (kNaMaxTiles + 1) * sizeof(uint32_t) <= kNaRecords, "tile arrays do not fit");
static_assert(kNaSlow + (size_t)GBR_NOALLOC_MAX_TRIANGLES * sizeof(uint32_t) <= GBR_NOALLOC_SCRATCH_BYTES,
              "bins do not fit the scratch array");

std::mutex g_na_mu;
constexpr int kNaMaxDevices = 64;
uint8_t* g_na_scratch[kNaMaxDevices] = {};  // device address of g_noalloc_scratch, per device

gbr_status na_fail(gbr_status st, const char* msg) {
    set_thread_error(msg);
    return st;
}

}  // namespace

extern "C" GBR_API gbr_status gbr_render_triangles_noalloc(const float* clip_positions, const float* colors,
                                                           uint32_t triangle_count, uint8_t* color_target,
                                                           float* depth_target, uint32_t width, uint32_t height,
                                                           const gbr_noalloc_state* state, void* stream) {
    char msg[256];
    if (!state || !color_target || (triangle_count && (!clip_positions || !colors)))
        return na_fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
    if (width == 0 || height == 0) return na_fail(GBR_ERR_INVALID_ARGUMENT, "zero-sized target");
    if (triangle_count > GBR_NOALLOC_MAX_TRIANGLES) {
        snprintf(msg, sizeof msg, "triangle_count %u exceeds GBR_NOALLOC_MAX_TRIANGLES (%u)", triangle_count,
                 GBR_NOALLOC_MAX_TRIANGLES);
        return na_fail(GBR_ERR_OUT_OF_MEMORY, msg);
    }
    if (width > GBR_NOALLOC_MAX_DIM || height > GBR_NOALLOC_MAX_DIM) {
        snprintf(msg, sizeof msg, "target %ux%u exceeds GBR_NOALLOC_MAX_DIM (%u)", width, height, GBR_NOALLOC_MAX_DIM);
        return na_fail(GBR_ERR_OUT_OF_MEMORY, msg);
    }
    if (((uintptr_t)clip_positions | (uintptr_t)colors) % 16 || (uintptr_t)color_target % 4 ||
        (uintptr_t)depth_target % 4)
        return na_fail(GBR_ERR_INVALID_ARGUMENT, "misaligned device pointer");
    if (state->depth_compare > GBR_COMPARE_ALWAYS || state->cull_mode > GBR_CULL_BACK || state->front_face > 1)
        return na_fail(GBR_ERR_INVALID_ARGUMENT, "invalid raster state");
    if ((state->color_load_op != GBR_LOAD_OP_LOAD && state->color_load_op != GBR_LOAD_OP_CLEAR) ||
        (state->depth_load_op != GBR_LOAD_OP_LOAD && state->depth_load_op != GBR_LOAD_OP_CLEAR))
        return na_fail(GBR_ERR_INVALID_ARGUMENT, "load op must be GBR_LOAD_OP_LOAD or GBR_LOAD_OP_CLEAR");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kNaMaxDevices) return na_fail(GBR_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    uint8_t* scratch = nullptr;
    {
        // Set-up, once per device with that device current: the host-side name of the array is
        // only a stand-in, so its device address is looked up and passed to the kernels.
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_scratch[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return na_fail(GBR_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch) failed");
            g_na_scratch[dev] = static_cast<uint8_t*>(p);
        }
        scratch = g_na_scratch[dev];
    }
    int num_sms = 0;
    e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // The draw and its target, resolved as the queue path resolves a clip_passthrough draw.
    DrawDesc d;
    std::memset(&d, 0, sizeof d);
    d.topology = GBR_TOPOLOGY_TRIANGLE_LIST;
    d.count = 3 * triangle_count;
    d.instance_count = 1;
    d.prims_per_instance = triangle_count;
    d.vb_data[0] = reinterpret_cast<const uint8_t*>(clip_positions);
    d.vb_data[1] = reinterpret_cast<const uint8_t*>(colors);
    d.vb_size[0] = d.vb_size[1] = (uint64_t)d.count * 16;
    d.vb_stride_vertex[0] = d.vb_stride_vertex[1] = 16;
    for (auto& a : d.attr) a = AttrDesc{-1, 0, 0, 0};
    d.attr[0] = AttrDesc{0, GBR_VERTEX_FORMAT_FLOAT32X4, 0, 0};
    d.attr[1] = AttrDesc{1, GBR_VERTEX_FORMAT_FLOAT32X4, 0, 0};
    d.program = PROG_CLIP_PASSTHROUGH;
    d.has_fragment = 1;
    d.num_varyings = kNaVaryings;
    d.interp = INTERP_LINEAR;
    d.profile = GBR_PROFILE_PARITY;
    d.cull_mode = state->cull_mode;
    d.front_face = state->front_face;
    volatile float vw = (float)width, vh = (float)height;  // ToRaster::new with the default viewport
    d.vp_tx = 0.0f + 0.5f * vw;
    d.vp_ty = 0.0f + 0.5f * vh;
    d.vp_sx = 0.5f * vw;
    d.vp_sy = (0.5f * vh) * -1.0f;
    d.sc_x1 = width;
    d.sc_y1 = height;
    d.depth_test = depth_target ? 1u : 0u;
    d.depth_compare = state->depth_compare;
    d.depth_write = state->depth_write_enabled;
    d.write_mask = 0xF;
    d.fast_vs = fast_vs_kind(d);
    d.fast_vcount = fast_vs_vcount(d);
    d.fast_packed = fast_vs_packed(d);
    TargetDesc t;
    std::memset(&t, 0, sizeof t);
    t.color = color_target;
    t.depth = depth_target;
    t.width = width;
    t.height = height;
    t.color_format = GBR_TEXTURE_FORMAT_RGBA8_UNORM;
    t.color_bpp = 4;
    t.color_load = state->color_load_op == GBR_LOAD_OP_CLEAR ? 1u : 0u;
    t.depth_load = state->depth_load_op == GBR_LOAD_OP_CLEAR ? 1u : 0u;
    for (int k = 0; k < 4; ++k) t.clear[k] = state->clear_color[k];
    t.depth_clear = state->clear_depth;
    t.tiles_x = (width + kNaTile - 1) / kNaTile;
    t.tiles_y = (height + kNaTile - 1) / kNaTile;

    BatchParams bp{};
    std::memset(&bp, 0, sizeof bp);
    bp.draws = reinterpret_cast<const DrawDesc*>(scratch + kNaDraw);
    bp.targets = reinterpret_cast<const TargetDesc*>(scratch + kNaTarget);
    bp.num_draws = triangle_count ? 1 : 0;
    bp.num_targets = 1;
    bp.total_prims = triangle_count;
    bp.total_tiles = t.tiles_x * t.tiles_y;
    bp.tile_size = kNaTile;
    bp.tile_shift = 4;
    bp.record_stride = kNaStride;
    bp.num_varyings = kNaVaryings;
    bp.records = scratch + kNaRecords;
    bp.ovf_records = scratch + kNaOvf;
    bp.ovf_capacity = GBR_NOALLOC_MAX_CLIPPED;
    bp.bin_capacity = GBR_NOALLOC_MAX_BIN_ENTRIES;
    uint32_t* tiles = reinterpret_cast<uint32_t*>(scratch + kNaTiles);
    bp.tile_count = tiles;
    bp.tile_offset = tiles + (kNaMaxTiles + 1);
    bp.tile_cursor = tiles + 2 * (kNaMaxTiles + 1);
    bp.bins = reinterpret_cast<uint32_t*>(scratch + kNaBins);
    bp.slow_prims = reinterpret_cast<uint32_t*>(scratch + kNaSlow);
    bp.work_counter = reinterpret_cast<uint32_t*>(scratch + kNaWork);
    bp.status = reinterpret_cast<BatchStatus*>(scratch + kNaStatus);
    bp.abort_flag = reinterpret_cast<uint32_t*>(scratch + kNaAbort);

    // The array keeps whatever the previous call left: clear the flag the kernels read first
    // (launch_batch zeroes the tile counts, the status and the work counter itself).
    if ((e = cudaMemsetAsync(scratch + kNaAbort, 0, sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(scratch + kNaDraw, &d, sizeof d, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(scratch + kNaTarget, &t, sizeof t, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    uint32_t launches = 0;
    if ((e = launch_batch(bp, kNaTile, kNaWarps, num_sms, s, &launches)) != cudaSuccess)
        return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    BatchStatus st;
    if ((e = cudaMemcpyAsync(&st, scratch + kNaStatus, sizeof st, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    switch (st.error) {
        case ERR_NONE: return GBR_OK;
        case ERR_OVERFLOW_RECORDS:
            snprintf(msg, sizeof msg, "clipping produced more than GBR_NOALLOC_MAX_CLIPPED (%u) extra sub-triangles",
                     GBR_NOALLOC_MAX_CLIPPED);
            return na_fail(GBR_ERR_OUT_OF_MEMORY, msg);
        case ERR_OVERFLOW_BINS:
            snprintf(msg, sizeof msg, "%llu triangle/tile pairs exceed GBR_NOALLOC_MAX_BIN_ENTRIES (%u)",
                     (unsigned long long)st.bin_entries, GBR_NOALLOC_MAX_BIN_ENTRIES);
            return na_fail(GBR_ERR_OUT_OF_MEMORY, msg);
        case ERR_W_ZERO: return na_fail(GBR_ERR_VALIDATION, "clip position w=0 (primitive.rs:177 / raster.rs:146)");
        default:
            snprintf(msg, sizeof msg, "device error %u (primitive %u)", st.error, st.error_detail);
            return na_fail(GBR_ERR_VALIDATION, msg);
    }
}

extern "C" GBR_API gbr_status gbr_selftest_division(uint64_t samples, uint64_t seed, uint64_t* out_mismatches,
                                                    float* first_mismatch) {
    if (!out_mismatches) return na_fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
    unsigned long long* d_count = nullptr;
    float* d_first = nullptr;
    cudaError_t e = cudaMalloc(&d_count, sizeof(unsigned long long) + 2 * sizeof(float));
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    d_first = reinterpret_cast<float*>(d_count + 1);
    unsigned long long h_count = 0;
    float h_first[2] = {0.0f, 0.0f};
    int dev = 0, sms = 0;
    if ((e = cudaMemset(d_count, 0, sizeof(unsigned long long) + 2 * sizeof(float))) == cudaSuccess &&
        (e = cudaGetDevice(&dev)) == cudaSuccess &&
        (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) == cudaSuccess) {
        gbr::k_selftest_division<<<sms * 8, 256>>>(samples, seed, d_count, d_first);
        if ((e = cudaGetLastError()) == cudaSuccess &&
            (e = cudaMemcpy(&h_count, d_count, sizeof h_count, cudaMemcpyDeviceToHost)) == cudaSuccess)
            e = cudaMemcpy(h_first, d_first, sizeof h_first, cudaMemcpyDeviceToHost);
    }
    cudaFree(d_count);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    *out_mismatches = h_count;
    if (first_mismatch) {
        first_mismatch[0] = h_first[0];
        first_mismatch[1] = h_first[1];
    }
    return GBR_OK;
}
