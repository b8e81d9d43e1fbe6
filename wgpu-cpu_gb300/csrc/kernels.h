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
// handles everything; see fragment_kind() in runtime.cu for the conditions of 1 and 2).
cudaError_t launch_batch(const BatchParams& bp, int tile, int warps, int num_sms, cudaStream_t s, uint32_t* launches,
                         cudaEvent_t* ev_raster = nullptr, int kind = 0);

// Tile side / warps-per-tile pairs compiled into the library.
bool raster_config_supported(int tile, int warps);

}  // namespace gbr
