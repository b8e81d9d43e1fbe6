// kernels_edge.cu — the render-pass kernels instantiated for the extension profile's
// edge-function raster rule (the launch sequence of launch.cuh with EDGE = true).
#include "launch.cuh"

namespace gbr {

template cudaError_t launch_batch_t<true>(const BatchParams&, int, int, int, cudaStream_t, uint32_t*, cudaEvent_t*,
                                          int);

}  // namespace gbr
