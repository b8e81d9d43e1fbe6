// jit.h — NVRTC-compiled render-pass modules for WGSL programs (jit.cu).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gbr_types.h"

namespace gbr {

// The kernels of one WGSL program's module: the setup / scan / fill / raster sequence of
// kernels.cu compiled with that program as PROG_JIT, at one tile shape per raster kernel.
struct JitKernels {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t setup = nullptr, slow = nullptr, scan = nullptr, fill = nullptr, states = nullptr, vis = nullptr,
                 ordered = nullptr, eval = nullptr, strip = nullptr, clear = nullptr, lines = nullptr;
    int vis_tile = 16, vis_warps = 4, ord_tile = 16, ord_warps = 8;
    std::mutex mu;  // launch configuration below
    size_t setup_smem = 0, ord_smem = 0, setup_occ_smem = 0;
    int vis_blocks = 0, ord_blocks = 0, setup_blocks = 1;
    ~JitKernels();
};

// Whether NVRTC and the CUDA headers it needs are present (with the reason when not).
bool jit_available(std::string* why);

// Compiles emitted program code with the kernels (NVRTC, sm_103a) without loading it: the cubin
// and the kernels' lowered names, the kernels instantiated for the reference's raster rule or
// (edge) the edge-function rule.  False with the compiler log on failure.
bool jit_compile_cubin(const std::string& code, bool edge, std::vector<char>* cubin, std::vector<std::string>* lowered,
                       std::string* log);

// A loaded module for the code under one raster rule (cached while any pipeline holds it); null
// with *err on failure.
std::shared_ptr<JitKernels> jit_module(const std::string& code, bool edge, std::string* err);

// launch_batch (kernels.h) with a JIT module's kernels; kind 3 = visibility raster, else ordered.
cudaError_t launch_batch_jit(JitKernels& k, const BatchParams& bp, int num_sms, cudaStream_t s, uint32_t* launches,
                             cudaEvent_t* ev_raster, int kind);

// launch_lines (kernels.h) with a JIT module's kernels.
cudaError_t launch_lines_jit(JitKernels& k, const BatchParams& bp, int num_sms, cudaStream_t s, uint32_t* launches,
                             cudaEvent_t* ev_raster);

// Runs the vertex stage alone for vertices first..first+n-1 of the draw at d_dev: per vertex,
// 4 position floats and MAX_VARYING_FLOATS inter-stage floats at out_dev, an error code at errs_dev.
cudaError_t jit_eval_vertices(JitKernels& k, const DrawDesc* d_dev, uint32_t first, uint32_t n, float* out_dev,
                              uint32_t* errs_dev, cudaStream_t s);

// Host copies of kernel launch constants (kernels.cu).
size_t setup_stage_bytes_host(uint32_t record_stride);
size_t ordered_raster_smem_host(int warps, uint32_t record_stride);

}  // namespace gbr
