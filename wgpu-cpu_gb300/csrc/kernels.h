// kernels.h — host entry points of the render-pass kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "gbr_types.h"

namespace gbr {

// Enqueues memsets + k_setup + k_scan + k_fill + k_raster for one batch on `s`.
// `launches` is incremented by the number of kernels enqueued.  When `ev_raster` is non-null,
// ev_raster[0] / ev_raster[1] are recorded just before / after the raster kernel.
//
// `kind` selects a raster kernel specialised for one fragment pipeline (0 = generic, which
// handles everything; see fragment_kind() in runtime.cu for the conditions of 1 and 2) or, for
// kind 3, the visibility raster (k_raster_vis) of opaque depth-tested batches.
cudaError_t launch_batch(const BatchParams& bp, int tile, int warps, int num_sms, cudaStream_t s, uint32_t* launches,
                         cudaEvent_t* ev_raster = nullptr, int kind = 0);

// The one line / point draw of a batch (k_clear_targets + k_lines_points, primitive order).
cudaError_t launch_lines(const BatchParams& bp, int num_sms, cudaStream_t s, uint32_t* launches, cudaEvent_t* ev_raster);

// Tile side / warps-per-tile pairs compiled into the library.
bool raster_config_supported(int tile, int warps);

// Bytes of the per-draw fragment-stage state the visibility raster (kind 3) reads from
// BatchParams::states (one entry per draw of the batch).
size_t raster_state_bytes();

// Kernels launch_batch enqueues for a batch (its `launches` increment).
uint32_t batch_kernel_launches(uint32_t total_prims, int tile, int warps, int kind, uint32_t fvs_mask);

// The FastVs shape of a resolved draw (FAST_VS_NONE when the fast setup path cannot run it).
uint32_t fast_vs_kind(const DrawDesc& d);
// Vertex indices below the result fetch every attribute of the draw's FastVs shape in range, for
// every instance of the draw (0 when none does, or no shape applies).
uint32_t fast_vs_vcount(const DrawDesc& d);
// 1 when the fast setup can read each vertex of the draw with 8- or 16-byte loads (DrawDesc::fast_packed).
uint32_t fast_vs_packed(const DrawDesc& d);

// Places n coalesced write segments: segment k copies desc[3k + 2] bytes from the device address
// desc[3k + 1] to the device address desc[3k]; the segments do not overlap.
cudaError_t launch_scatter_writes(const uint64_t* desc, uint32_t n, cudaStream_t s);

// Copies of device textures into host memory the device can address (pinned, mapped): up to
// kCopyOutMax per launch, every source and destination 16-byte aligned.  All SMs take part in
// every copy (grid-stride over 16-byte words, the ragged tail byte by byte).
constexpr uint32_t kCopyOutMax = 64;
struct CopyOutJobs {
    uint32_t n;
    uint32_t _pad;
    const uint8_t* src[kCopyOutMax];
    uint8_t* dst[kCopyOutMax];
    uint64_t bytes[kCopyOutMax];
};
cudaError_t launch_copy_out(const CopyOutJobs& jobs, int num_sms, cudaStream_t s);

}  // namespace gbr
