// kernels.cu — instantiates the render-pass kernels for the supported tile shapes and launches
// one batch (setup -> scan -> fill -> raster) on a stream.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.h"
#include "raster.cuh"

namespace gbr {

namespace {

constexpr int kCap = 4096;  // keys per tile sorted in shared memory; larger bins sort in place
constexpr int kRB = 32;     // records staged in shared memory per step

template <int T, int W>
cudaError_t launch_raster(const BatchParams& bp, int num_sms, cudaStream_t s) {
    auto kern = k_raster<T, W, kCap, kRB>;
    const size_t smem = kCap * sizeof(uint32_t) + (size_t)kRB * bp.record_stride;
    static std::mutex mu;
    static size_t configured = 0;
    static int blocks_per_sm = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (configured < smem) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, W * 32, smem);
            if (e != cudaSuccess) return e;
            if (blocks_per_sm < 1) blocks_per_sm = 1;
            configured = smem;
        }
    }
    const uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)num_sms * blocks_per_sm, bp.total_tiles);
    kern<<<grid ? grid : 1, W * 32, smem, s>>>(bp);
    return cudaGetLastError();
}

}  // namespace

bool raster_config_supported(int tile, int warps) {
    switch (tile) {
        case 8: return warps == 1 || warps == 2;
        case 16: return warps == 2 || warps == 4 || warps == 8;
        case 32: return warps == 4 || warps == 8;
        default: return false;
    }
}

cudaError_t launch_batch(const BatchParams& bp, int tile, int warps, int num_sms, cudaStream_t s,
                         uint32_t* launches, cudaEvent_t* ev_raster) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(bp.tile_count, 0, (bp.total_tiles + 1) * sizeof(uint32_t), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bp.status, 0, sizeof(BatchStatus), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bp.work_counter, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
    const uint32_t items = bp.total_prims;
    const uint32_t cap = (uint32_t)num_sms * 16;
    if (items) {
        uint32_t g = std::min((items + 127) / 128, cap);
        k_setup<<<g, 128, 0, s>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ++*launches;
    }
    k_scan<<<1, 1024, 0, s>>>(bp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ++*launches;
    if (items) {
        uint32_t g = std::min((items + bp.ovf_capacity + 127) / 128, cap);
        k_fill<<<g, 128, 0, s>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ++*launches;
    }
    if (ev_raster && (e = cudaEventRecord(ev_raster[0], s)) != cudaSuccess) return e;
    switch (tile * 16 + warps) {
        case 8 * 16 + 1: e = launch_raster<8, 1>(bp, num_sms, s); break;
        case 8 * 16 + 2: e = launch_raster<8, 2>(bp, num_sms, s); break;
        case 16 * 16 + 2: e = launch_raster<16, 2>(bp, num_sms, s); break;
        case 16 * 16 + 4: e = launch_raster<16, 4>(bp, num_sms, s); break;
        case 16 * 16 + 8: e = launch_raster<16, 8>(bp, num_sms, s); break;
        case 32 * 16 + 4: e = launch_raster<32, 4>(bp, num_sms, s); break;
        case 32 * 16 + 8: e = launch_raster<32, 8>(bp, num_sms, s); break;
        default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    ++*launches;
    if (ev_raster) e = cudaEventRecord(ev_raster[1], s);
    return e;
}

}  // namespace gbr
