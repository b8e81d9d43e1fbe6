// jit.cu — compiles a WGSL program (CUDA emitted by wgsl.cpp) together with the render-pass
// kernels through NVRTC for sm_103a, loads the cubin (cudaLibraryLoadData) and launches a batch
// with its kernels.  NVRTC is opened at run time (dlopen), so the library loads on machines
// without it; only creating a WGSL pipeline needs it.  Modules are cached by program text.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "jit.h"
#include "jit_sources.inc"  // kJitHeaderNames / kJitHeaders: the kernel headers, generated at build time

namespace gbr {

namespace {

// ---- NVRTC, resolved at run time
typedef int nvrtcResult_t;
typedef struct _nvrtcProgram* nvrtcProgram_t;
struct Nvrtc {
    void* h = nullptr;
    nvrtcResult_t (*create)(nvrtcProgram_t*, const char*, const char*, int, const char* const*, const char* const*);
    nvrtcResult_t (*destroy)(nvrtcProgram_t*);
    nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char* const*);
    nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t*);
    nvrtcResult_t (*log)(nvrtcProgram_t, char*);
    nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t*);
    nvrtcResult_t (*cubin)(nvrtcProgram_t, char*);
    nvrtcResult_t (*add_name)(nvrtcProgram_t, const char*);
    nvrtcResult_t (*lowered)(nvrtcProgram_t, const char*, const char**);
    const char* (*err)(nvrtcResult_t);
    std::string include_dir;
};

const Nvrtc& nvrtc() {
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* names[] = {"libnvrtc.so.13", "libnvrtc.so.12", "libnvrtc.so",
                               "/usr/local/cuda/lib64/libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so"};
        for (const char* nm : names)
            if ((n.h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
        if (!n.h) return;
        auto sym = [&](const char* s) { return dlsym(n.h, s); };
        n.create = reinterpret_cast<decltype(n.create)>(sym("nvrtcCreateProgram"));
        n.destroy = reinterpret_cast<decltype(n.destroy)>(sym("nvrtcDestroyProgram"));
        n.compile = reinterpret_cast<decltype(n.compile)>(sym("nvrtcCompileProgram"));
        n.log_size = reinterpret_cast<decltype(n.log_size)>(sym("nvrtcGetProgramLogSize"));
        n.log = reinterpret_cast<decltype(n.log)>(sym("nvrtcGetProgramLog"));
        n.cubin_size = reinterpret_cast<decltype(n.cubin_size)>(sym("nvrtcGetCUBINSize"));
        n.cubin = reinterpret_cast<decltype(n.cubin)>(sym("nvrtcGetCUBIN"));
        n.add_name = reinterpret_cast<decltype(n.add_name)>(sym("nvrtcAddNameExpression"));
        n.lowered = reinterpret_cast<decltype(n.lowered)>(sym("nvrtcGetLoweredName"));
        n.err = reinterpret_cast<decltype(n.err)>(sym("nvrtcGetErrorString"));
        if (!n.create || !n.compile || !n.cubin || !n.lowered) {
            dlclose(n.h);
            n.h = nullptr;
            return;
        }
        // cuda_fp16.h for the kernels: the toolkit next to libnvrtc, or CUDA_HOME, or the default
        std::vector<std::string> cands;
        if (const char* ch = std::getenv("CUDA_HOME")) cands.push_back(std::string(ch) + "/include");
        Dl_info info;
        if (dladdr(reinterpret_cast<void*>(n.create), &info) && info.dli_fname) {
            std::string p = info.dli_fname;
            const size_t k = p.rfind('/');
            if (k != std::string::npos) cands.push_back(p.substr(0, k) + "/../include");
        }
        cands.push_back("/usr/local/cuda/include");
        for (const std::string& c : cands) {
            const std::string f = c + "/cuda_fp16.h";
            if (FILE* fp = std::fopen(f.c_str(), "r")) {
                std::fclose(fp);
                n.include_dir = c;
                break;
            }
        }
    });
    return n;
}

// The kernels a JIT module exports, by name expression, for the reference's raster rule and for
// the edge-function rule.
constexpr int kJitVisTile = 16, kJitVisWarps = 4, kJitOrdTile = 16, kJitOrdWarps = 8;
constexpr int kJitKernels = 11;
const char* const kKernelExprs[2][kJitKernels] = {
    {"&gbr::k_setup<false>", "&gbr::k_setup_slow<false>", "&gbr::k_scan<0>", "&gbr::k_fill<false>",
     "&gbr::k_build_states<0>", "&gbr::k_raster_vis<16, 4, false>", "&gbr::k_raster<16, 8, 4096, 64, 0, false>",
     "&gbr::k_eval_vs", "&gbr::k_strip_table<0>", "&gbr::k_clear_targets", "&gbr::k_lines_points"},
    {"&gbr::k_setup<true>", "&gbr::k_setup_slow<true>", "&gbr::k_scan<0>", "&gbr::k_fill<true>",
     "&gbr::k_build_states<0>", "&gbr::k_raster_vis<16, 4, true>", "&gbr::k_raster<16, 8, 4096, 64, 0, true>",
     "&gbr::k_eval_vs", "&gbr::k_strip_table<0>", "&gbr::k_clear_targets", "&gbr::k_lines_points"}};

std::string program_source(const std::string& code) {
    std::string s;
    s += "#define GBR_JIT 1\n#include \"wgsl_rt.cuh\"\nnamespace gbr {\n";
    s += code;
    s += "\n// evaluation of the vertex stage alone (tests): position + inter-stage floats per vertex\n"
         "__global__ void k_eval_vs(const DrawDesc* d, uint32_t first, uint32_t n, float* out, uint32_t* errs) {\n"
         "  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;\n"
         "  if (i >= n) return;\n"
         "  V4 pos{0.0f, 0.0f, 0.0f, 0.0f};\n  float var[MAX_VARYING_FLOATS] = {};\n  uint32_t err = 0;\n"
         "  const bool ok = jit_vs(*d, first + i, 0u, pos, var, &err);\n"
         "  errs[i] = ok ? 0u : (err ? err : 1u);\n"
         "  float* o = out + (size_t)i * (4 + MAX_VARYING_FLOATS);\n"
         "  o[0] = pos.x; o[1] = pos.y; o[2] = pos.z; o[3] = pos.w;\n"
         "  for (int k = 0; k < MAX_VARYING_FLOATS; ++k) o[4 + k] = var[k];\n}\n";
    s += "}  // namespace gbr\n#include \"raster_vis.cuh\"\n#include \"raster_lines.cuh\"\n";
    return s;
}

std::mutex g_cache_mu;
std::map<std::string, std::weak_ptr<JitKernels>> g_cache;

}  // namespace

bool jit_available(std::string* why) {
    const Nvrtc& n = nvrtc();
    if (!n.h) {
        if (why) *why = "NVRTC (libnvrtc.so) could not be loaded";
        return false;
    }
    if (n.include_dir.empty()) {
        if (why) *why = "the CUDA headers (cuda_fp16.h) for NVRTC were not found";
        return false;
    }
    return true;
}

bool jit_compile_cubin(const std::string& code, bool edge, std::vector<char>* cubin, std::vector<std::string>* lowered,
                       std::string* log) {
    const char* const* exprs = kKernelExprs[edge ? 1 : 0];
    std::string why;
    if (!jit_available(&why)) {
        *log = why;
        return false;
    }
    const Nvrtc& n = nvrtc();
    const std::string src = program_source(code);
    nvrtcProgram_t prog = nullptr;
    const int nh = (int)(sizeof(kJitHeaders) / sizeof(kJitHeaders[0]));
    if (n.create(&prog, src.c_str(), "wgsl_program.cu", nh, kJitHeaders, kJitHeaderNames) != 0) {
        *log = "nvrtcCreateProgram failed";
        return false;
    }
    for (int i = 0; i < kJitKernels; ++i) n.add_name(prog, exprs[i]);
    const std::string inc = "-I" + n.include_dir;
    // no multiply-add contraction in the front end nor in ptxas
    const char* opts[] = {"--gpu-architecture=sm_103a", "-fmad=false", "--ptxas-options=--fmad=false", "--std=c++17",
                          inc.c_str()};
    const nvrtcResult_t rc = n.compile(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
    size_t ls = 0;
    n.log_size(prog, &ls);
    std::string lg(ls, '\0');
    if (ls) n.log(prog, &lg[0]);
    *log = lg;
    if (rc != 0) {
        n.destroy(&prog);
        return false;
    }
    size_t cs = 0;
    n.cubin_size(prog, &cs);
    cubin->resize(cs);
    n.cubin(prog, cubin->data());
    lowered->clear();
    for (int i = 0; i < kJitKernels; ++i) {
        const char* name = nullptr;
        n.lowered(prog, exprs[i], &name);
        lowered->push_back(name ? name : "");
    }
    n.destroy(&prog);
    return true;
}

JitKernels::~JitKernels() {
    if (lib) cudaLibraryUnload(lib);
}

std::shared_ptr<JitKernels> jit_module(const std::string& code, bool edge, std::string* err) {
    // one module per device: the kernels' shared-memory attributes and occupancy below are
    // per-device properties, so a module (and its cached launch settings) never serves two devices
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    const std::string key = std::to_string(dev) + (edge ? "\nedge\n" : "\nscanline\n") + code;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end())
            if (auto sp = it->second.lock()) return sp;
    }
    std::vector<char> cubin;
    std::vector<std::string> names;
    std::string log;
    if (!jit_compile_cubin(code, edge, &cubin, &names, &log)) {
        *err = "NVRTC: " + log;
        return nullptr;
    }
    auto k = std::make_shared<JitKernels>();
    cudaError_t e = cudaLibraryLoadData(&k->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        *err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
        return nullptr;
    }
    cudaKernel_t* slots[] = {&k->setup, &k->slow, &k->scan, &k->fill, &k->states, &k->vis, &k->ordered, &k->eval,
                             &k->strip, &k->clear, &k->lines};
    for (size_t i = 0; i < names.size(); ++i) {
        if ((e = cudaLibraryGetKernel(slots[i], k->lib, names[i].c_str())) != cudaSuccess) {
            *err = std::string("cudaLibraryGetKernel(") + names[i] + "): " + cudaGetErrorString(e);
            return nullptr;
        }
    }
    k->vis_tile = kJitVisTile;
    k->vis_warps = kJitVisWarps;
    k->ord_tile = kJitOrdTile;
    k->ord_warps = kJitOrdWarps;
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache[key] = k;
    return k;
}

namespace {
cudaError_t launch(cudaKernel_t k, uint32_t grid, uint32_t block, size_t smem, cudaStream_t s, const BatchParams& bp) {
    void* args[] = {const_cast<BatchParams*>(&bp)};
    return cudaLaunchKernel(reinterpret_cast<const void*>(k), dim3(grid ? grid : 1), dim3(block), args, smem, s);
}
}  // namespace

cudaError_t launch_batch_jit(JitKernels& k, const BatchParams& bp, int num_sms, cudaStream_t s, uint32_t* launches,
                             cudaEvent_t* ev_raster, int kind) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(bp.tile_count, 0, (bp.total_tiles + 1) * sizeof(uint32_t), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bp.status, 0, sizeof(BatchStatus), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bp.work_counter, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
    unsigned int ev_flags = cudaEventRecordDefault;
    if (ev_raster) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return e;
        if (cs == cudaStreamCaptureStatusActive) ev_flags = cudaEventRecordExternal;
    }
    std::lock_guard<std::mutex> lk(k.mu);
    const uint32_t items = bp.total_prims;
    if (bp.strip_info && items) {
        if ((e = launch(k.strip, bp.num_draws, 1024, 0, s, bp)) != cudaSuccess) return e;
        ++*launches;
    }
    if (items) {
        const size_t smem = setup_stage_bytes_host(bp.record_stride);
        if (k.setup_smem < smem) {
            if ((e = cudaFuncSetAttribute(reinterpret_cast<const void*>(k.setup), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem)) != cudaSuccess)
                return e;
            k.setup_smem = smem;
        }
        if (k.setup_occ_smem != smem) {  // blocks an SM holds at this stage size (grid-stride: one wave)
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k.setup_blocks, reinterpret_cast<const void*>(k.setup),
                                                                   128, smem)) != cudaSuccess)
                return e;
            k.setup_blocks = std::max(1, k.setup_blocks);
            k.setup_occ_smem = smem;
        }
        const uint32_t g = std::min((items + 127) / 128, std::min((uint32_t)num_sms * 16, (uint32_t)(num_sms * k.setup_blocks)));
        if ((e = launch(k.setup, g, 128, smem, s, bp)) != cudaSuccess) return e;
        if ((e = launch(k.slow, std::min((items + 127) / 128, (uint32_t)num_sms * 4), 128, 0, s, bp)) != cudaSuccess) return e;
        *launches += 2;
    }
    if ((e = launch(k.scan, 1, 1024, 0, s, bp)) != cudaSuccess) return e;
    ++*launches;
    if (items) {
        if ((e = launch(k.fill, std::min((items + 127) / 128, (uint32_t)num_sms * 16), 128, 0, s, bp)) != cudaSuccess) return e;
        ++*launches;
    }
    if (kind == 3) {
        if ((e = launch(k.states, (bp.num_draws + 127) / 128, 128, 0, s, bp)) != cudaSuccess) return e;
        ++*launches;
    }
    if (ev_raster && (e = cudaEventRecordWithFlags(ev_raster[0], s, ev_flags)) != cudaSuccess) return e;
    if (kind == 3) {
        if (!k.vis_blocks) {
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k.vis_blocks, reinterpret_cast<const void*>(k.vis),
                                                                   k.vis_warps * 32, 0)) != cudaSuccess)
                return e;
            k.vis_blocks = std::max(1, k.vis_blocks);
        }
        const uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)num_sms * k.vis_blocks, bp.total_tiles);
        if ((e = launch(k.vis, grid, k.vis_warps * 32, 0, s, bp)) != cudaSuccess) return e;
    } else {
        const size_t smem = ordered_raster_smem_host(k.ord_warps, bp.record_stride);
        if (k.ord_smem < smem) {
            if ((e = cudaFuncSetAttribute(reinterpret_cast<const void*>(k.ordered),
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
                return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k.ord_blocks, reinterpret_cast<const void*>(k.ordered),
                                                                   k.ord_warps * 32, smem)) != cudaSuccess)
                return e;
            k.ord_blocks = std::max(1, k.ord_blocks);
            k.ord_smem = smem;
        }
        const uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)num_sms * k.ord_blocks, bp.total_tiles);
        if ((e = launch(k.ordered, grid, k.ord_warps * 32, smem, s, bp)) != cudaSuccess) return e;
    }
    ++*launches;
    if (ev_raster) e = cudaEventRecordWithFlags(ev_raster[1], s, ev_flags);
    return e;
}

cudaError_t launch_lines_jit(JitKernels& k, const BatchParams& bp, int num_sms, cudaStream_t s, uint32_t* launches,
                             cudaEvent_t* ev_raster) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(bp.status, 0, sizeof(BatchStatus), s)) != cudaSuccess) return e;
    unsigned int ev_flags = cudaEventRecordDefault;
    if (ev_raster) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return e;
        if (cs == cudaStreamCaptureStatusActive) ev_flags = cudaEventRecordExternal;
    }
    if ((e = launch(k.clear, num_sms * 4, 256, 0, s, bp)) != cudaSuccess) return e;
    if (ev_raster && (e = cudaEventRecordWithFlags(ev_raster[0], s, ev_flags)) != cudaSuccess) return e;
    if ((e = launch(k.lines, 1, 256, 0, s, bp)) != cudaSuccess) return e;
    *launches += 2;
    if (ev_raster) e = cudaEventRecordWithFlags(ev_raster[1], s, ev_flags);
    return e;
}

cudaError_t jit_eval_vertices(JitKernels& k, const DrawDesc* d_dev, uint32_t first, uint32_t n, float* out_dev,
                              uint32_t* errs_dev, cudaStream_t s) {
    const DrawDesc* dp = d_dev;
    void* args[] = {&dp, &first, &n, &out_dev, &errs_dev};
    return cudaLaunchKernel(reinterpret_cast<const void*>(k.eval), dim3((n + 127) / 128), dim3(128), args, 0, s);
}

}  // namespace gbr
