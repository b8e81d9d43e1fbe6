// launch.cuh — the launch sequence of one batch (setup -> scan -> fill -> raster) with its tile-
// shape dispatch, templated on the raster rule: kernels.cu instantiates it for the reference's
// scanline rule and kernels_edge.cu for the edge-function rule, so each rule's kernels carry only
// their own coverage code (and the two translation units compile in parallel).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "kernels.h"
#include "raster.cuh"
#include "raster_vis.cuh"

namespace gbr {

namespace launch_detail {

constexpr int kCap = 4096;  // keys per tile sorted in shared memory; larger bins sort in place
constexpr int kRW = 64;     // records staged in shared memory per window

// Launch configuration of one kernel, kept per CUDA device: cudaFuncSetAttribute applies to the
// current device only, so the dynamic shared memory a kernel may use is raised on each device the
// first time a launch there needs it, and its resident blocks per SM are looked up per device and
// shared-memory size.
struct LaunchCache {
    std::mutex mu;
    std::map<int, size_t> smem_allowed;              // device -> dynamic smem the kernel may use
    std::map<std::pair<int, size_t>, int> resident;  // (device, dynamic smem) -> blocks per SM
};

// Blocks of `kern` an SM holds with `threads` threads and `smem` bytes of dynamic shared memory
// on the current device (at least 1), raising the kernel's dynamic shared-memory limit first.
template <class Kernel>
cudaError_t resident_blocks(LaunchCache& c, Kernel kern, int threads, size_t smem, int* out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(c.mu);
    auto allowed = c.smem_allowed.find(dev);
    if (smem && (allowed == c.smem_allowed.end() || allowed->second < smem)) {
        if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
            return e;
        c.smem_allowed[dev] = smem;
    }
    auto it = c.resident.find({dev, smem});
    if (it == c.resident.end()) {
        int blocks = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, threads, smem)) != cudaSuccess) return e;
        it = c.resident.emplace(std::make_pair(dev, smem), std::max(blocks, 1)).first;
    }
    *out = it->second;
    return cudaSuccess;
}

template <int T, int W, int KIND, bool EDGE>
cudaError_t launch_raster(const BatchParams& bp, int num_sms, cudaStream_t s) {
    if constexpr (EDGE && KIND == 2) {
        return cudaErrorInvalidValue;  // the textured specialisation is parity-profile only
    } else {
    auto kern = k_raster<T, W, kCap, kRW, KIND, EDGE>;
    const size_t smem = (kCap + 2 * W * 32) * sizeof(uint32_t) + (size_t)kRW * bp.record_stride;
    static LaunchCache cache;
    int blocks_per_sm = 1;
    if (cudaError_t e = resident_blocks(cache, kern, W * 32, smem, &blocks_per_sm); e != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)num_sms * blocks_per_sm, bp.total_tiles);
    kern<<<grid ? grid : 1, W * 32, smem, s>>>(bp);
    return cudaGetLastError();
    }
}

template <int T, int W, bool EDGE>
cudaError_t launch_raster_vis(const BatchParams& bp, int num_sms, cudaStream_t s) {
    auto kern = k_raster_vis<T, W, EDGE>;
    static LaunchCache cache;
    int blocks_per_sm = 1;
    if (cudaError_t e = resident_blocks(cache, kern, W * 32, 0, &blocks_per_sm); e != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)num_sms * blocks_per_sm, bp.total_tiles);
    kern<<<grid ? grid : 1, W * 32, 0, s>>>(bp);
    return cudaGetLastError();
}


// Tile shapes of the ordered raster kernel.
inline bool ordered_config_supported(int tile, int warps) {
    switch (tile) {
        case 8: return warps == 1 || warps == 2;
        case 16: return warps == 2 || warps == 4 || warps == 8;
        case 32: return warps == 4 || warps == 8;
        default: return false;
    }
}
// Tile shapes of the visibility raster kernel.
inline bool vis_config_supported(int tile, int warps) {
    switch (tile) {
        case 8: return warps == 1 || warps == 2;
        case 16: case 32: return warps == 1 || warps == 2 || warps == 4 || warps == 8;
        default: return false;
    }
}

// One k_setup launch (all shapes when ONLY < 0), grid-stride over one wave of resident blocks.
template <bool EDGE, int ONLY>
cudaError_t launch_setup(const BatchParams& bp, int num_sms, cudaStream_t s) {
    const size_t smem = setup_stage_bytes(bp.record_stride);
    int resident = 1;  // k_setup blocks an SM holds at this stage size
    static LaunchCache cache;
    cudaError_t e = resident_blocks(cache, k_setup<EDGE, ONLY>, kSetupWarps * 32, smem, &resident);
    if (e != cudaSuccess) return e;
    const uint32_t cap = (uint32_t)num_sms * 16;
    const uint32_t g = std::min((bp.total_prims + 127) / 128, std::min(cap, (uint32_t)(resident * num_sms)));
    k_setup<EDGE, ONLY><<<g, kSetupWarps * 32, smem, s>>>(bp);
    return cudaGetLastError();
}

}  // namespace launch_detail

// The setup launches of a batch: one per FastVs shape its draws use (each kernel holds one
// vertex-stage variant), or one generic launch when the shapes are not known.
template <bool EDGE>
cudaError_t launch_setups(const BatchParams& bp, int num_sms, cudaStream_t s, uint32_t* launches) {
    using namespace launch_detail;
    if (!bp.fvs_mask) {
        ++*launches;
        return launch_setup<EDGE, -1>(bp, num_sms, s);
    }
    for (int f = 0; f < 7; ++f) {
        if (!((bp.fvs_mask >> f) & 1u)) continue;
        cudaError_t e;
        switch (f) {
            case FAST_VS_NONE: e = launch_setup<EDGE, FAST_VS_NONE>(bp, num_sms, s); break;
            case FAST_VS_MVP_COLOR: e = launch_setup<EDGE, FAST_VS_MVP_COLOR>(bp, num_sms, s); break;
            case FAST_VS_MVP_TEX: e = launch_setup<EDGE, FAST_VS_MVP_TEX>(bp, num_sms, s); break;
            case FAST_VS_QUAD: e = launch_setup<EDGE, FAST_VS_QUAD>(bp, num_sms, s); break;
            case FAST_VS_CLIP: e = launch_setup<EDGE, FAST_VS_CLIP>(bp, num_sms, s); break;
            case FAST_VS_TRIANGLE: e = launch_setup<EDGE, FAST_VS_TRIANGLE>(bp, num_sms, s); break;
            default: e = launch_setup<EDGE, FAST_VS_QUAD_F16>(bp, num_sms, s); break;
        }
        if (e != cudaSuccess) return e;
        ++*launches;
    }
    return cudaSuccess;
}

template <bool EDGE>
cudaError_t launch_batch_t(const BatchParams& bp, int tile, int warps, int num_sms, cudaStream_t s,
                           uint32_t* launches, cudaEvent_t* ev_raster, int kind) {
    using namespace launch_detail;
    cudaError_t e;
    if ((e = cudaMemsetAsync(bp.tile_count, 0, (bp.total_tiles + 1) * sizeof(uint32_t), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bp.status, 0, sizeof(BatchStatus), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bp.work_counter, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
    const uint32_t items = bp.total_prims;
    const uint32_t cap = (uint32_t)num_sms * 16;
    if (bp.strip_info && items) {
        k_strip_table<><<<bp.num_draws, 1024, 0, s>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ++*launches;
    }
    // with primitives, the generic setup also builds the visibility raster's states
    const bool slow_states = kind == 3 && items;
    if (items) {
        if ((e = launch_setups<EDGE>(bp, num_sms, s, launches)) != cudaSuccess) return e;
        BatchParams sp = bp;
        sp.slow_builds_states = slow_states ? 1u : 0u;
        k_setup_slow<EDGE><<<std::min((items + 127) / 128, (uint32_t)num_sms * 4), 128, 0, s>>>(sp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ++*launches;
    }
    k_scan<><<<1, 1024, 0, s>>>(bp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ++*launches;
    if (items) {
        uint32_t g = std::min((items + bp.ovf_capacity + 127) / 128, cap);
        k_fill<EDGE><<<g, 128, 0, s>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ++*launches;
    }
    // Inside a stream capture the raster events must become event-record nodes of the graph
    // (cudaEventRecordExternal); outside one that flag is not accepted.
    unsigned int ev_flags = cudaEventRecordDefault;
    if (ev_raster) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return e;
        if (cs == cudaStreamCaptureStatusActive) ev_flags = cudaEventRecordExternal;
    }
    if (kind == 3 && !slow_states) {
        k_build_states<><<<(bp.num_draws + 127) / 128, 128, 0, s>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ++*launches;
    }
    if (ev_raster && (e = cudaEventRecordWithFlags(ev_raster[0], s, ev_flags)) != cudaSuccess) return e;
    if (kind == 3 && !vis_config_supported(tile, warps)) kind = 0;
    if (EDGE && kind == 2) kind = 0;  // no textured specialisation under the edge rule
    // the ordered kernel for a warps-per-tile it has no instantiation for: the tile's default
    if (kind != 3 && !ordered_config_supported(tile, warps)) warps = tile == 8 ? 2 : 8;
    for (;;) {
    switch ((tile * 16 + warps) * 4 + (kind & 3)) {
        case (8 * 16 + 1) * 4: e = launch_raster<8, 1, 0, EDGE>(bp, num_sms, s); break;
        case (8 * 16 + 2) * 4: e = launch_raster<8, 2, 0, EDGE>(bp, num_sms, s); break;
        case (8 * 16 + 2) * 4 + 1: e = launch_raster<8, 2, 1, EDGE>(bp, num_sms, s); break;
        case (8 * 16 + 2) * 4 + 2: e = launch_raster<8, 2, 2, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 2) * 4: e = launch_raster<16, 2, 0, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 2) * 4 + 1: e = launch_raster<16, 2, 1, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 2) * 4 + 2: e = launch_raster<16, 2, 2, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 4) * 4: e = launch_raster<16, 4, 0, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 4) * 4 + 1: e = launch_raster<16, 4, 1, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 4) * 4 + 2: e = launch_raster<16, 4, 2, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 8) * 4: e = launch_raster<16, 8, 0, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 8) * 4 + 1: e = launch_raster<16, 8, 1, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 8) * 4 + 2: e = launch_raster<16, 8, 2, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 4) * 4: e = launch_raster<32, 4, 0, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 4) * 4 + 1: e = launch_raster<32, 4, 1, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 8) * 4: e = launch_raster<32, 8, 0, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 8) * 4 + 1: e = launch_raster<32, 8, 1, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 8) * 4 + 2: e = launch_raster<32, 8, 2, EDGE>(bp, num_sms, s); break;
        case (8 * 16 + 1) * 4 + 3: e = launch_raster_vis<8, 1, EDGE>(bp, num_sms, s); break;
        case (8 * 16 + 2) * 4 + 3: e = launch_raster_vis<8, 2, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 1) * 4 + 3: e = launch_raster_vis<16, 1, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 2) * 4 + 3: e = launch_raster_vis<16, 2, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 4) * 4 + 3: e = launch_raster_vis<16, 4, EDGE>(bp, num_sms, s); break;
        case (16 * 16 + 8) * 4 + 3: e = launch_raster_vis<16, 8, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 1) * 4 + 3: e = launch_raster_vis<32, 1, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 2) * 4 + 3: e = launch_raster_vis<32, 2, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 4) * 4 + 3: e = launch_raster_vis<32, 4, EDGE>(bp, num_sms, s); break;
        case (32 * 16 + 8) * 4 + 3: e = launch_raster_vis<32, 8, EDGE>(bp, num_sms, s); break;
        default:
            if (kind == 0) return cudaErrorInvalidValue;
            kind = 0;  // no specialised instantiation for this tile shape: the generic kernel
            continue;
    }
    break;
    }
    if (e != cudaSuccess) return e;
    ++*launches;
    if (ev_raster) e = cudaEventRecordWithFlags(ev_raster[1], s, ev_flags);
    return e;
}

}  // namespace gbr
