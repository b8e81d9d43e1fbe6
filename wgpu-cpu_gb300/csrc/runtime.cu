// runtime.cu — the C ABI of include/gbr.h: objects, the queue worker, command-stream decoding,
// batch planning and the launch of the render-pass kernels.
//
// Threading mirrors wgpu-cpu (device.rs:40-74, 436-549; engine.rs:11-47): any thread may call
// the ABI; gbr_queue_submit decodes and validates on the caller's thread and enqueues; one worker
// thread per device owns the CUDA stream and executes queue items in order (buffer/texture
// writes, submissions, reads), so writes are ordered with submissions as wgpu's queue orders
// them.  A submission's render passes become launch batches (one per draw in the per-draw
// mode, one per pass otherwise); the worker waits for the submission's last kernel, checks
// each batch's device status and re-runs from a batch that ran out of scratch space.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gbr.h"
#include "gbr_types.h"
#include "jit.h"
#include "kernels.h"
#include "wgsl.h"

namespace gbr {
namespace {

thread_local std::string g_last_error;

struct Failure {
    gbr_status status;
    std::string msg;
};
[[noreturn]] void fail(gbr_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Failure{st, buf};
}
void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) fail(GBR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// [offset, offset + size) inside [0, total), written so that no sum can wrap around 2^64
// (the reference converts with try_into and slices, which panics on such ranges).
inline bool range_fits(uint64_t offset, uint64_t size, uint64_t total) {
    return size <= total && offset <= total - size;
}
// a + b * c + d without wrapping; UINT64_MAX when the true value does not fit (never "in range")
inline uint64_t span_end(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    uint64_t p, s, r;
    if (__builtin_mul_overflow(b, c, &p) || __builtin_add_overflow(a, p, &s) || __builtin_add_overflow(s, d, &r))
        return UINT64_MAX;
    return r;
}

using Clock = std::chrono::steady_clock;
double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// ---------------------------------------------------------------- formats and programs
uint32_t bytes_per_texel(uint32_t f) {
    switch (f) {
        case GBR_TEXTURE_FORMAT_R8_UNORM: return 1;
        case GBR_TEXTURE_FORMAT_RG8_UNORM: return 2;
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM:
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB:
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM:
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM_SRGB:
        case GBR_TEXTURE_FORMAT_DEPTH32_FLOAT: return 4;
        case GBR_TEXTURE_FORMAT_RGBA16_FLOAT: return 8;
        case GBR_TEXTURE_FORMAT_RGBA32_FLOAT: return 16;
        default: return 0;
    }
}
uint32_t vertex_format_bytes(uint32_t f) {
    switch (f) {
        case GBR_VERTEX_FORMAT_FLOAT32:
        case GBR_VERTEX_FORMAT_UINT32:
        case GBR_VERTEX_FORMAT_SINT32:
        case GBR_VERTEX_FORMAT_FLOAT16X2:
        case GBR_VERTEX_FORMAT_UNORM8X4: return 4;
        case GBR_VERTEX_FORMAT_FLOAT32X2:
        case GBR_VERTEX_FORMAT_FLOAT16X4: return 8;
        case GBR_VERTEX_FORMAT_FLOAT32X3: return 12;
        case GBR_VERTEX_FORMAT_FLOAT32X4: return 16;
        default: return 0;
    }
}

// Interface of the native programs (their code is in programs.cuh).
struct ProgramInfo {
    const char* name;
    uint32_t id;
    int num_inputs;
    int input_loc[16], input_comps[16];
    uint32_t num_varyings;
    bool perspective;
    uint32_t uniform_min;  // bytes required at @group(0) @binding(0), 0 = none
    bool uses_texture;     // @group(1) @binding(0) texture_2d + @binding(1) sampler
    // WGSL programs (PROG_JIT): every uniform binding's size, the sampled texture / sampler
    // bindings, inputs read as integers, discard
    bool jit = false;
    uint32_t uniform_req[4][8] = {};
    int tex_group = 1, tex_binding = 0, samp_group = 1, samp_binding = 1;
    int input_kind[16] = {};
    bool may_discard = false;
    uint32_t flat_mask = 0;    // inter-stage floats interpolated flat (bit per float)
    uint32_t early_depth = 0;  // EarlyDepth of the fragment entry point
};
// The native programs, and variants whose fragment entry point carries @early_depth_test(force)
// ("<name>@early_force") or @early_depth_test(<conservative>) ("<name>@early_allow").
const std::vector<ProgramInfo>& native_programs() {
    static const std::vector<ProgramInfo> table = [] {
        std::vector<ProgramInfo> v = {
            {"colored_triangle", PROG_COLORED_TRIANGLE, 0, {0, 0, 0}, {0, 0, 0}, 4, false, 0, false},
            {"mesh_color", PROG_MESH_COLOR, 2, {0, 1, 0}, {3, 3, 0}, 3, false, 64, false},
            {"mesh_color_perspective", PROG_MESH_COLOR_PERSPECTIVE, 2, {0, 1, 0}, {3, 3, 0}, 3, true, 64, false},
            {"mesh_color_discard", PROG_MESH_COLOR_DISCARD, 2, {0, 1, 0}, {3, 3, 0}, 3, false, 64, false},
            {"mesh_tex_lambert", PROG_MESH_TEX_LAMBERT, 3, {0, 1, 2}, {3, 3, 2}, 5, false, 80, true},
            {"quad_color", PROG_QUAD_COLOR, 2, {0, 1, 0}, {3, 4, 0}, 4, false, 0, false},
            {"clip_passthrough", PROG_CLIP_PASSTHROUGH, 2, {0, 1, 0}, {4, 4, 0}, 4, false, 0, false},
            {"clip_flat", PROG_CLIP_FLAT, 2, {0, 1, 0}, {4, 4, 0}, 4, false, 0, false},
            {"clip_flat_id", PROG_CLIP_FLAT_ID, 2, {0, 1, 0}, {4, 4, 0}, 4, false, 0, false},
            {"clip_discard", PROG_CLIP_DISCARD, 2, {0, 1, 0}, {4, 4, 0}, 4, false, 0, false},
        };
        for (auto& p : v) {
            if (p.id == PROG_CLIP_FLAT) p.flat_mask = 0xFu;
            if (p.id == PROG_CLIP_FLAT_ID) p.flat_mask = 0x1u;
            if (p.id == PROG_CLIP_DISCARD || p.id == PROG_MESH_COLOR_DISCARD) p.may_discard = true;
        }
        static const char* const kEarly[] = {"clip_passthrough", "clip_discard", "clip_flat_id", "mesh_color",
                                             "mesh_color_discard"};
        static std::vector<std::string> names;  // storage of the variants' names
        names.reserve(2 * (sizeof kEarly / sizeof kEarly[0]));
        const size_t base = v.size();
        for (const char* n : kEarly)
            for (uint32_t mode : {EARLY_DEPTH_FORCE, EARLY_DEPTH_ALLOW})
                for (size_t i = 0; i < base; ++i)
                    if (std::strcmp(v[i].name, n) == 0) {
                        names.push_back(std::string(n) + (mode == EARLY_DEPTH_FORCE ? "@early_force" : "@early_allow"));
                        ProgramInfo q = v[i];
                        q.name = names.back().c_str();
                        q.early_depth = mode;
                        v.push_back(q);
                    }
        return v;
    }();
    return table;
}
const ProgramInfo* find_program(const char* name) {
    for (const auto& p : native_programs())
        if (std::strcmp(p.name, name) == 0) return &p;
    return nullptr;
}

// WGSL front end with its errors as status codes
std::shared_ptr<wgsl::Module> parse_wgsl(const char* src, uint64_t len) {
    try {
        return wgsl::parse(std::string(src, len));
    } catch (const wgsl::Error& e) {
        fail(e.unsupported ? GBR_ERR_UNSUPPORTED : GBR_ERR_SHADER, "%s", e.what());
    }
}
wgsl::ProgramCode emit_wgsl(const wgsl::Module& vs, const std::string& ve, const wgsl::Module* fs, const std::string& fe,
                            const wgsl::Constants& vc = {}, const wgsl::Constants& fc = {}) {
    try {
        return wgsl::emit_program(vs, ve, fs, fe, vc, fc);
    } catch (const wgsl::Error& e) {
        fail(e.unsupported ? GBR_ERR_UNSUPPORTED : GBR_ERR_SHADER, "%s", e.what());
    }
}

// ---------------------------------------------------------------- objects
struct Object {
    virtual ~Object() {}
};
// Bytes of resident resources (buffers and textures) a device holds: admission counts them
// against the HBM budget.  Shared with the resources, which outlive their handles while a queued
// submission still uses them.
using ResidentCounter = std::shared_ptr<std::atomic<uint64_t>>;

struct Buffer : Object {
    uint8_t* ptr = nullptr;
    uint64_t size = 0;
    uint64_t allocated = 0;
    ResidentCounter resident;
    ~Buffer() override {
        if (ptr) cudaFree(ptr);
        if (resident) resident->fetch_sub(allocated);
    }
};
struct Texture : Object {
    gbr_texture_desc desc{};
    uint32_t bpp = 0;
    uint32_t mips_stored = 1;
    uint64_t mip_offset[16] = {};
    uint64_t bytes = 0;
    uint8_t* ptr = nullptr;
    uint32_t layers() const { return desc.size.depth_or_array_layers ? desc.size.depth_or_array_layers : 1; }
    uint32_t mip_w(uint32_t m) const { return std::max(1u, desc.size.width >> m); }
    uint32_t mip_h(uint32_t m) const { return std::max(1u, desc.size.height >> m); }
    uint64_t mip_bytes(uint32_t m) const { return (uint64_t)mip_w(m) * mip_h(m) * layers() * bpp; }
    ResidentCounter resident;
    ~Texture() override {
        if (ptr) cudaFree(ptr);
        if (resident) resident->fetch_sub(bytes);
    }
};
struct Sampler : Object {
    gbr_sampler_desc desc{};
};
struct ShaderModule : Object {
    const ProgramInfo* prog = nullptr;        // native program
    std::shared_ptr<wgsl::Module> wgsl;       // or a parsed WGSL module
};
struct Pipeline : Object {
    gbr_render_pipeline_desc desc{};
    const ProgramInfo* prog = nullptr;
    ProgramInfo own;                          // the WGSL program's info (prog points here)
    std::shared_ptr<JitKernels> jit;          // its kernels
    AttrDesc attr[16];
};
struct BindGroup : Object {
    gbr_bind_group_desc desc{};
    std::vector<std::shared_ptr<Object>> refs;  // the resources, kept alive with the group
};

// ---------------------------------------------------------------- decoded commands
struct Slice {
    std::shared_ptr<Buffer> buf;
    uint64_t offset = 0, size = 0;
};
struct DrawCmd {
    bool indexed = false;
    uint32_t start = 0, end = 0;
    int32_t base_vertex = 0;
    uint32_t inst_start = 0, inst_end = 1;
    std::shared_ptr<Pipeline> pipeline;  // state snapshot at the draw (state.rs:57-74)
    Slice index;
    uint32_t index_format = 0;
    Slice vb[GBR_MAX_VERTEX_BUFFERS];
    std::shared_ptr<BindGroup> groups[GBR_MAX_BIND_GROUPS];
    float viewport[6] = {};
    uint32_t scissor[4] = {};
    double blend_constant[4] = {};
};
// An encoder command outside render passes (extension profile): a copy or a clear, resolved and
// validated at submit.  Texture regions are (mip, origin x/y/layer) with an extent.
struct CopyCmd {
    uint32_t op = 0;  // gbr_opcode
    std::shared_ptr<Buffer> buf, buf2;
    std::shared_ptr<Texture> tex, tex2;
    uint64_t off = 0, off2 = 0, size = 0;
    gbr_texel_copy_buffer_layout layout{};
    uint32_t mip = 0, mip2 = 0;
    uint32_t ox = 0, oy = 0, oz = 0, ox2 = 0, oy2 = 0, oz2 = 0;
    gbr_extent3d ext{};
    uint32_t mip_count = 0, layer_count = 0;
};

struct PassCmd {
    std::shared_ptr<CopyCmd> copy;  // set: this entry is a copy or clear, not a render pass
    gbr_cmd_begin_render_pass begin{};
    std::shared_ptr<Texture> color;
    std::shared_ptr<Texture> depth;
    uint32_t width = 0, height = 0;
    std::vector<DrawCmd> draws;
};

// ---------------------------------------------------------------- queue items
struct Item {
    enum Kind { SUBMIT, WRITE_BUFFER, WRITE_TEXTURE, READ_BUFFER, READ_TEXTURE, READ_TEXTURES, FLUSH } kind = SUBMIT;
    uint64_t index = 0;
    std::vector<PassCmd> passes;
    std::shared_ptr<Buffer> buffer;
    std::shared_ptr<Texture> texture;
    uint32_t mip = 0;
    uint64_t offset = 0;
    std::vector<uint8_t> data;
    void* staged = nullptr;  // writes: the caller's bytes already on the device (freed by the worker)
    uint64_t staged_size = 0;
    gbr_texel_copy_buffer_layout layout{};
    std::vector<std::shared_ptr<Texture>> textures;  // READ_TEXTURES: texture, mip, destination each
    std::vector<uint32_t> mips;
    std::vector<void*> dsts;
    void* dst = nullptr;
    uint64_t size = 0;
    std::promise<Failure>* done = nullptr;  // reads: completion for the blocked caller
    bool indexed = false;  // a read that took a submission index (completion recorded like a submission's)
    Clock::time_point t_submit;
    uint32_t merged = 0;  // submissions executed together with this one (serving mode)
};

// Start / end events of a launch sequence, shared by the submissions it ran.
struct EventPair {
    cudaEvent_t start = nullptr, end = nullptr;
    EventPair() = default;
    EventPair(const EventPair&) = delete;
    EventPair& operator=(const EventPair&) = delete;
    ~EventPair() {
        if (start) cudaEventDestroy(start);
        if (end) cudaEventDestroy(end);
    }
};

struct SubmissionRecord {
    gbr_submission_stats stats{};
    gbr_status status = GBR_OK;
    std::string error;
    std::shared_ptr<EventPair> ev;
};

// Outcome of run_batches: the first batch that failed validation on the device (or the batch
// count), its error code and message.
struct RunResult {
    size_t bad;
    uint32_t error;
    std::string msg;
};

// What the launches of one submission group accumulate.
struct GroupRun {
    std::shared_ptr<EventPair> ev;
    bool started = false;
    uint32_t launches = 0;
    uint64_t slow_prims = 0;
    uint64_t split_chunks = 0;  // chunk work items of split visibility-raster tiles
    uint32_t tile_shape = 0, tile_shape_prims = 0;  // side << 8 | warps of the largest batch
    double raster_ms = 0.0;
};

// ---------------------------------------------------------------- scratch (grow-only)
struct DevBuf {
    void* ptr = nullptr;
    size_t size = 0;
    void ensure(size_t need, std::atomic<uint64_t>* total) {
        if (need <= size) return;
        size_t n = std::max(need, size + size / 2);
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        total->fetch_sub(size);
        size = 0;
        cuda_check(cudaMalloc(&ptr, n), "cudaMalloc(scratch)");
        size = n;
        total->fetch_add(n);
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        size = 0;
    }
};

struct Batch;

constexpr size_t kLazyWakeItems = 1024;  // queued writes that wake the worker by themselves
constexpr size_t kKeptRecords = 16384;   // finished submissions whose stats stay queryable

struct PlannedGroup;
class Planner;

struct Device {
    gbr_device_config cfg{};
    int ordinal = 0;
    int num_sms = 0;
    int tile = 16, warps = 8;
    cudaStream_t stream = nullptr;
    // Writes copy the caller's bytes to device staging at call time on copy_stream (not ordered
    // with the queue; a pinned source moves at full DMA speed), and the worker applies them in
    // queue order with a device-to-device copy.
    cudaStream_t copy_stream = nullptr;
    cudaMemPool_t staging_pool = nullptr;
    std::mutex copy_mu;
    // Asynchronous readbacks (gbr_queue_read_textures) run on rb_stream with the copy engines,
    // after the queue work before them (an event), so the kernels of later submissions overlap
    // them; a later writer of a texture that is being read first waits for that read's event.
    // Completion is recorded in queue order (finish_reads).  All of it is the worker's.
    cudaStream_t rb_stream = nullptr;
    struct ReadFence {
        cudaEvent_t ev = nullptr;
        ReadFence() = default;
        ReadFence(const ReadFence&) = delete;
        ReadFence& operator=(const ReadFence&) = delete;
        ~ReadFence() {
            if (ev) cudaEventDestroy(ev);
        }
    };
    struct PendingRead {
        uint64_t index = 0;
        std::shared_ptr<ReadFence> done;
        std::vector<std::shared_ptr<Texture>> keep;
        Clock::time_point t_submit;
    };
    std::map<const Texture*, std::shared_ptr<ReadFence>> read_fence;  // the last readback of each texture
    std::deque<PendingRead> pending_reads;                            // in index order
    // Readbacks whose place in the queue's stream is marked (`ready`) but whose copies are not
    // issued yet: the worker issues them while the next submission runs (issue_reads), or at once
    // when a writer of one of their textures comes first.
    struct DeferredRead {
        Item item;
        cudaEvent_t ready = nullptr;
    };
    std::deque<DeferredRead> deferred_reads;
    void issue_reads();
    void wait_reads_of(const Texture* t) {  // the queue's stream waits for t's readback in flight
        for (const DeferredRead& dr : deferred_reads)
            for (const auto& u : dr.item.textures)
                if (u.get() == t) {
                    issue_reads();
                    goto issued;
                }
    issued:
        auto f = read_fence.find(t);
        if (f != read_fence.end()) cuda_check(cudaStreamWaitEvent(stream, f->second->ev, 0), "read fence");
    }
    void wait_all_reads() {
        issue_reads();
        for (auto& f : read_fence) cuda_check(cudaStreamWaitEvent(stream, f.second->ev, 0), "read fence");
    }
    void finish_reads(uint64_t before);
    // worker lookahead (worker_main): the planner, whether it holds the next group, and the
    // non-submission items queued before that group
    Planner* la_planner = nullptr;
    bool la_ahead = false;
    std::vector<std::vector<Item>> la_between;
    void lookahead();

    std::mutex obj_mu;
    uint64_t next_handle = 1;
    std::unordered_map<uint64_t, std::shared_ptr<Object>> objects;
    ResidentCounter resident = std::make_shared<std::atomic<uint64_t>>(0);
    // HBM a submission group may use for transient memory: the budget less the resident resources
    uint64_t transient_budget() const {
        const uint64_t budget = cfg.hbm_budget_bytes ? cfg.hbm_budget_bytes : (80ull << 30);
        const uint64_t res = resident->load();
        return budget > res ? budget - res : 0;
    }

    std::mutex q_mu;
    std::condition_variable q_cv, done_cv;
    std::deque<Item> queue;
    bool stopping = false;
    uint64_t next_submission = 0;
    uint64_t completed_submissions = 0;  // submissions with index < this are done
    std::map<uint64_t, SubmissionRecord> records;
    bool lost = false;
    std::string lost_msg;
    std::thread worker;

    // worker-owned scratch
    std::atomic<uint64_t> scratch_bytes{0};  // the arena below (read by gbr_device_memory)
    DevBuf records_buf, ovf_buf, tiles_buf, bins_buf, meta_buf, flush_buf, slow_buf, strip_buf, upload_buf, hint_buf,
        split_buf;
    // coalesced small writes: double-buffered pinned staging, each free again once its event (the
    // upload copy from it) has completed
    struct PinnedStage {
        uint8_t* ptr = nullptr;
        size_t size = 0;
        cudaEvent_t done = nullptr;
    } pinned_stage[2], meta_stage[2];
    int pinned_next = 0, meta_next = 0;
    uint32_t ovf_capacity = 4096;
    uint64_t bin_capacity = 1u << 22;
    // chunk work items the visibility raster may split heavy tiles into (0: 32 MiB of key arrays);
    // GBR_VIS_SPLIT_ITEMS sets it at device creation
    uint32_t split_cap_override = 0;
    uint32_t split_chunk = VIS_SPLIT_CHUNK;  // records per chunk; GBR_VIS_SPLIT_CHUNK sets it

    // autotuner: per batch signature, each candidate tile shape is timed once, then the fastest
    // is kept (all shapes give bit-identical results, only the time differs)
    bool autotune = false;
    struct TuneEntry {
        int tried = 0, best = 0;
        float ms[8] = {};
    };
    std::map<uint64_t, TuneEntry> tuner;
    uint64_t tuner_signature(const Batch& b) const;
    int tuner_pick(const Batch& b, int* t, int* w);
    void tuner_record(const Batch& b, int cand, float ms);

    // CUDA graphs of whole launch sequences, keyed by their launch parameters
    struct GraphEntry {
        cudaGraphExec_t exec = nullptr;
        std::vector<cudaEvent_t> events;
        uint64_t last_use = 0;
    };
    std::map<std::string, GraphEntry> graphs;
    uint64_t graph_clock = 0;

    std::vector<Batch> plan_batches(const std::vector<PassCmd>& passes, uint64_t* draws, uint64_t* prims_in,
                                    uint32_t item);
    bool merge_batch(Batch& into, Batch& b);
    std::vector<Batch> split_batch(const Batch& m);
    RunResult run_batches(std::vector<Batch>& batches, size_t from, GroupRun& run);

    template <class T>
    std::shared_ptr<T> get(uint64_t h, const char* what) {
        std::lock_guard<std::mutex> lk(obj_mu);
        auto it = objects.find(h);
        if (it == objects.end()) fail(GBR_ERR_INVALID_ARGUMENT, "invalid %s handle %llu", what, (unsigned long long)h);
        auto p = std::dynamic_pointer_cast<T>(it->second);
        if (!p) fail(GBR_ERR_INVALID_ARGUMENT, "handle %llu is not a %s", (unsigned long long)h, what);
        return p;
    }
    uint64_t add(std::shared_ptr<Object> o) {
        std::lock_guard<std::mutex> lk(obj_mu);
        uint64_t h = next_handle++;
        objects[h] = std::move(o);
        return h;
    }
    void remove(uint64_t h) {
        std::lock_guard<std::mutex> lk(obj_mu);
        objects.erase(h);
    }
    // Writes only need to be applied before whatever is queued after them, so they do not wake
    // the worker: the next submission, read, poll or device destruction does, and the worker then
    // takes the whole run of writes at once (and coalesces the small ones).
    void enqueue(Item&& it) {
        std::lock_guard<std::mutex> lk(q_mu);
        if (lost) fail(GBR_ERR_DEVICE_LOST, "device lost: %s", lost_msg.c_str());
        const bool lazy = it.kind == Item::WRITE_BUFFER || it.kind == Item::WRITE_TEXTURE;
        queue.push_back(std::move(it));
        if (!lazy || queue.size() >= kLazyWakeItems) q_cv.notify_all();
    }
    // Queues writes back to back under one lock (they wake the worker as single writes do).
    void enqueue_all(std::vector<Item>& items) {
        if (items.empty()) return;
        std::lock_guard<std::mutex> lk(q_mu);
        if (lost) fail(GBR_ERR_DEVICE_LOST, "device lost: %s", lost_msg.c_str());
        for (Item& it : items) queue.push_back(std::move(it));
        if (queue.size() >= kLazyWakeItems) q_cv.notify_all();
    }
    void worker_main();
    std::vector<Item> pop_group_locked();
    void execute(Item& it);
    void execute_writes(std::vector<Item>& items);
    PlannedGroup plan_group(std::vector<Item>&& items);
    void run_group(PlannedGroup& g);
    void note_failure(const Failure& f);
};

std::mutex g_dev_mu;
std::unordered_map<uint64_t, std::shared_ptr<Device>> g_devices;
uint64_t g_next_device = 1;

std::shared_ptr<Device> get_device(gbr_device d) {
    std::lock_guard<std::mutex> lk(g_dev_mu);
    auto it = g_devices.find(d);
    if (it == g_devices.end()) fail(GBR_ERR_INVALID_ARGUMENT, "invalid device handle");
    return it->second;
}

// ---------------------------------------------------------------- batch planning
struct Batch {
    std::vector<DrawDesc> draws;
    std::vector<TargetDesc> targets;
    std::vector<uint32_t> target_item;       // submission (index in its group) of each target
    std::vector<const Texture*> writes, reads;  // attachments written, textures sampled
    uint32_t strip_entries = 0;              // strip-table entries of the restart draws
    std::vector<uint64_t> target_frags;      // kTargetCounters counters per target (after the run)
    uint32_t total_prims = 0, total_tiles = 0, nvar = 0;
    uint32_t item = 0;         // the submission of a single-submission batch
    bool single_item = true;
    bool lines = false;        // one line / point draw, drawn by k_lines_points
    std::shared_ptr<JitKernels> jit;  // the WGSL module whose kernels run this batch (or none)
    std::shared_ptr<CopyCmd> copy;    // a copy or clear between passes (no draws, no targets)
};

// A submission group planned on the host, ready for the device.
struct PlannedGroup {
    std::vector<Item> items;
    std::vector<SubmissionRecord> recs;
    std::vector<Batch> batches;
    Failure failure{GBR_OK, ""};  // a failure of the whole group while planning
};

// The worker's planning helper: one thread that plans the group handed to start() and hands the
// result back at finish().
class Planner {
  public:
    explicit Planner(Device* d) : dev_(d), thread_([this] { loop(); }) {}
    ~Planner() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        thread_.join();
    }
    void start(std::vector<Item>&& items) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            in_ = std::move(items);
            have_in_ = true;
            have_out_ = false;
        }
        cv_.notify_all();
    }
    PlannedGroup finish() {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return have_out_; });
        have_out_ = false;
        return std::move(out_);
    }

  private:
    void loop() {
        cudaSetDevice(dev_->ordinal);
        for (;;) {
            std::vector<Item> items;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || have_in_; });
                if (stop_) return;
                items = std::move(in_);
                have_in_ = false;
            }
            PlannedGroup g = dev_->plan_group(std::move(items));
            {
                std::lock_guard<std::mutex> lk(mu_);
                out_ = std::move(g);
                have_out_ = true;
            }
            cv_.notify_all();
        }
    }
    Device* dev_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::vector<Item> in_;
    PlannedGroup out_;
    bool have_in_ = false, have_out_ = false, stop_ = false;
    std::thread thread_;
};

// The FastVs shapes of a batch's draws (bit per shape): one setup launch each.
uint32_t fvs_mask(const Batch& b) {
    uint32_t m = 0;
    for (const DrawDesc& d : b.draws) m |= 1u << d.fast_vs;
    return m;
}

// The setup kernels' work list per FastVs shape (BatchParams::shape_groups): for each shape f,
// its draws with primitives as pairs (draw, first 32-primitive group), groups numbered over the
// shape's draws in batch order and aligned at each draw's first primitive, then (~0, the shape's
// group count); off[f] .. off[f + 1] are the shape's pairs.
void shape_group_table(const Batch& b, std::vector<uint32_t>& table, uint32_t off[8]) {
    table.clear();
    for (uint32_t f = 0; f < 7; ++f) {
        off[f] = (uint32_t)(table.size() / 2);
        uint32_t groups = 0;
        for (uint32_t k = 0; k < (uint32_t)b.draws.size(); ++k) {
            const DrawDesc& d = b.draws[k];
            const uint64_t n = (uint64_t)d.prims_per_instance * d.instance_count;
            if (d.fast_vs != f || n == 0) continue;
            table.push_back(k);
            table.push_back(groups);
            groups += (uint32_t)((n + 31) / 32);
        }
        if (table.size() / 2 > off[f]) {
            table.push_back(~0u);
            table.push_back(groups);
        }
    }
    off[7] = (uint32_t)(table.size() / 2);
}

// Visibility raster (kind 3): every target has colour and depth, and every draw writes depth
// with one batch-wide Less / LessEqual / Greater / GreaterEqual, does not blend and runs a
// fragment stage that never discards.  Returns the compare function, or 0.
uint32_t visibility_compare(const Batch& b) {
    if (b.draws.empty()) return 0;
    for (const TargetDesc& t : b.targets)
        if (!t.color || !t.depth) return 0;
    const uint32_t cmp = b.draws[0].depth_compare;
    if (cmp != GBR_COMPARE_LESS && cmp != GBR_COMPARE_LESS_EQUAL && cmp != GBR_COMPARE_GREATER &&
        cmp != GBR_COMPARE_GREATER_EQUAL)
        return 0;
    for (const DrawDesc& d : b.draws)
        if (!d.depth_test || !d.depth_write || d.depth_compare != cmp || d.blend_enabled || !d.has_fragment ||
            d.program == PROG_MESH_COLOR_DISCARD || d.may_discard || d.early_depth != EARLY_DEPTH_NONE)
            return 0;
    return cmp;
}

// Which raster kernel runs a batch (kernels.h): 3 = the visibility raster (above) when allowed;
// 1 = a vec4f colour passed straight to an Rgba16Float target with SrcAlpha/OneMinusSrcAlpha
// (alpha One/OneMinusSrcAlpha) blending and no depth test; 2 = the textured Lambert program into
// Rgba8 with a depth test, no blending, parity profile.  Every draw of the batch must qualify;
// otherwise 0, the generic ordered kernel.
int fragment_kind(const Batch& b, bool allow_visibility) {
    if (allow_visibility && visibility_compare(b)) return 3;
    if (b.jit) return 0;  // a WGSL module carries the generic and the visibility raster only
    if (b.draws.empty() || b.targets.size() != 1 || !b.targets[0].color) return 0;
    const uint32_t fmt = b.targets[0].color_format;
    bool k1 = fmt == GBR_TEXTURE_FORMAT_RGBA16_FLOAT, k2 = fmt == GBR_TEXTURE_FORMAT_RGBA8_UNORM ||
                                                          fmt == GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB;
    for (const DrawDesc& d : b.draws) {
        const bool over = d.blend_enabled && d.blend_color[0] == GBR_BLEND_SRC_ALPHA &&
                          d.blend_color[1] == GBR_BLEND_ONE_MINUS_SRC_ALPHA && d.blend_color[2] == GBR_BLEND_OP_ADD &&
                          d.blend_alpha[0] == GBR_BLEND_ONE && d.blend_alpha[1] == GBR_BLEND_ONE_MINUS_SRC_ALPHA &&
                          d.blend_alpha[2] == GBR_BLEND_OP_ADD;
        k1 = k1 && over && d.write_mask == 0xF && !d.depth_test && d.has_fragment &&
             (d.program == PROG_QUAD_COLOR || d.program == PROG_CLIP_PASSTHROUGH || d.program == PROG_COLORED_TRIANGLE);
        k2 = k2 && !d.blend_enabled && d.write_mask == 0xF && d.depth_test && d.has_fragment &&
             d.program == PROG_MESH_TEX_LAMBERT && d.profile == GBR_PROFILE_PARITY;
    }
    return k1 ? 1 : k2 ? 2 : 0;
}

// Tile shapes (side, warps per tile) the autotuner tries, all compiled into kernels.cu: for the
// ordered kernels, and for the visibility raster.  The first is the shape used before any
// measurement.  The tuner times each batch's whole launch sequence (setup, binning and raster:
// the tile side changes the binning cost as well), one candidate per submission of a batch shape.
const int kTuneCands[][2] = {{16, 8}, {32, 8}, {32, 4}, {16, 4}, {16, 2}};
const int kTuneCandsVis[][2] = {{32, 8}, {16, 4}, {32, 4}, {16, 2}, {16, 1}};
constexpr int kNumTuneCands = 5;

uint64_t log2_bucket(uint64_t v) {
    uint64_t r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}

// Batches with the same fragment kernel, order of magnitude of primitives, of pixels and of
// targets share a tuning decision.
uint64_t Device::tuner_signature(const Batch& b) const {
    uint64_t pixels = 0;
    for (const TargetDesc& t : b.targets) pixels += (uint64_t)t.width * t.height;
    return ((uint64_t)fragment_kind(b, cfg.raster_order == GBR_RASTER_AUTO) << 48) |
           (log2_bucket(b.total_prims + 1) << 32) |
           (log2_bucket(pixels + 1) << 16) | log2_bucket(b.targets.size());
}
int Device::tuner_pick(const Batch& b, int* t, int* w) {
    TuneEntry& e = tuner[tuner_signature(b)];
    const auto& cands = fragment_kind(b, cfg.raster_order == GBR_RASTER_AUTO) == 3 ? kTuneCandsVis : kTuneCands;
    const int c = e.tried < kNumTuneCands ? e.tried : e.best;
    *t = cands[c][0];
    *w = cands[c][1];
    return e.tried < kNumTuneCands ? e.tried : -1;
}
void Device::tuner_record(const Batch& b, int cand, float ms) {
    TuneEntry& e = tuner[tuner_signature(b)];
    if (cand != e.tried || cand >= kNumTuneCands) return;  // a second batch of the same signature
    e.ms[cand] = ms;
    e.tried = cand + 1;
    if (e.tried == kNumTuneCands) {
        e.best = 0;
        for (int c = 1; c < kNumTuneCands; ++c)
            if (e.ms[c] < e.ms[e.best]) e.best = c;
    }
}

uint32_t ilog2(uint32_t v) {
    uint32_t r = 0;
    while ((1u << r) < v) ++r;
    return r;
}

TargetDesc make_target(const PassCmd& p, bool first_in_pass, uint32_t tile, uint32_t profile) {
    TargetDesc t{};
    t.width = p.width;
    t.height = p.height;
    if (p.color) {
        const gbr_color_attachment& ca = p.begin.color_attachments[0];
        t.color = p.color->ptr;
        t.color_format = p.color->desc.format;
        t.color_bpp = p.color->bpp;
        t.slice_offset = (uint32_t)((uint64_t)ca.depth_slice * p.width * p.height * p.color->bpp);
        t.color_load = first_in_pass && ca.load_op == GBR_LOAD_OP_CLEAR ? 1u : 0u;
        for (int k = 0; k < 4; ++k) t.clear[k] = (float)ca.clear_value[k];  // wgpu_color_to_vec4
        uint32_t f = t.color_format;
        if (profile == GBR_PROFILE_PARITY && (f == GBR_TEXTURE_FORMAT_RGBA16_FLOAT || f == GBR_TEXTURE_FORMAT_RGBA32_FLOAT))
            fail(GBR_ERR_UNSUPPORTED, "Unsupported texture format for colour writes (texture.rs:407)");
        // the reference writes Srgb formats as Unorm (texture.rs:389-398); the extension profile
        // encodes linear -> sRGB on write and decodes for blending
        if (profile == GBR_PROFILE_EXTENSION && f == GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB)
            t.color_format = TFMT_RGBA8_SRGB_ENCODE;
        if (profile == GBR_PROFILE_EXTENSION && f == GBR_TEXTURE_FORMAT_BGRA8_UNORM_SRGB)
            t.color_format = TFMT_BGRA8_SRGB_ENCODE;
    }
    if (p.depth) {
        const gbr_depth_attachment& da = p.begin.depth_attachment;
        t.depth = reinterpret_cast<float*>(p.depth->ptr);
        t.depth_load = !da.has_depth_ops ? 2u : (first_in_pass && da.depth_load_op == GBR_LOAD_OP_CLEAR ? 1u : 0u);
        t.depth_clear = da.depth_clear_value;
    }
    t.tiles_x = (p.width + tile - 1) / tile;
    t.tiles_y = (p.height + tile - 1) / tile;
    return t;
}

// Primitive slots of `count` stream positions (primitive.rs:248-264, 324-358): lists take whole
// groups, strips one per position after the first (or two); with primitive restart a slot can stay
// empty.
uint32_t primitive_slots(uint32_t topology, uint32_t count) {
    switch (topology) {
        case GBR_TOPOLOGY_POINT_LIST: return count;
        case GBR_TOPOLOGY_LINE_LIST: return count / 2;
        case GBR_TOPOLOGY_LINE_STRIP: return count >= 2 ? count - 1 : 0;
        case GBR_TOPOLOGY_TRIANGLE_LIST: return count / 3;
        default: return count >= 3 ? count - 2 : 0;
    }
}

DrawDesc make_draw(const DrawCmd& dc, uint32_t profile, bool has_depth_attachment) {
    DrawDesc d{};
    const Pipeline& pl = *dc.pipeline;
    const gbr_render_pipeline_desc& pd = pl.desc;
    const ProgramInfo& prog = *pl.prog;
    const gbr_primitive_state& ps = pd.primitive;
    if (ps.polygon_mode != GBR_POLYGON_FILL) fail(GBR_ERR_UNSUPPORTED, "Unsupported polygon mode (state.rs:475-477)");
    if (ps.topology > GBR_TOPOLOGY_TRIANGLE_STRIP) fail(GBR_ERR_INVALID_ARGUMENT, "topology");
    if (dc.indexed && ps.strip_index_format != GBR_INDEX_NONE) {
        if (ps.topology != GBR_TOPOLOGY_TRIANGLE_STRIP && ps.topology != GBR_TOPOLOGY_LINE_STRIP)
            fail(GBR_ERR_VALIDATION, "List can't be separated");
        if (ps.strip_index_format != dc.index_format)
            fail(GBR_ERR_VALIDATION, "strip_index_format does not match the index format");
        d.strip_restart = 1;  // separators split the strip (index.rs:90-106, primitive.rs:428-487)
    }
    if (prog.perspective && profile != GBR_PROFILE_EXTENSION)
        fail(GBR_ERR_UNSUPPORTED, "perspective interpolation is todo!() in the reference (fragment.rs:343-345)");
    d.topology = ps.topology;
    d.index_format = dc.indexed ? dc.index_format : 0;
    d.first = dc.start;
    d.count = dc.end > dc.start ? dc.end - dc.start : 0;
    d.base_vertex = dc.base_vertex;
    d.instance_start = dc.inst_start;
    d.instance_count = dc.inst_end > dc.inst_start ? dc.inst_end - dc.inst_start : 0;
    d.prims_per_instance = primitive_slots(ps.topology, d.count);
    if (dc.indexed) {
        if (!dc.index.buf) fail(GBR_ERR_VALIDATION, "No index buffer bound");
        d.index_data = dc.index.buf->ptr + dc.index.offset;
        d.index_bytes = dc.index.size;
        uint32_t isz = dc.index_format == GBR_INDEX_UINT16 ? 2 : 4;
        if (dc.index.offset % isz) fail(GBR_ERR_VALIDATION, "index buffer offset is not aligned");
    }
    for (uint32_t b = 0; b < pd.vertex_buffer_count; ++b) {
        const gbr_vertex_buffer_layout& L = pd.vertex_buffers[b];
        const Slice& s = dc.vb[b];
        if (!s.buf) fail(GBR_ERR_VALIDATION, "Buffer %u not bound (vertex.rs:268-272)", b);
        d.vb_data[b] = s.buf->ptr + s.offset;
        d.vb_size[b] = s.size;
        d.vb_stride_vertex[b] = L.step_mode == GBR_STEP_VERTEX ? (uint32_t)L.array_stride : 0;
        d.vb_stride_instance[b] = L.step_mode == GBR_STEP_INSTANCE ? (uint32_t)L.array_stride : 0;
    }
    for (int l = 0; l < 16; ++l) d.attr[l] = pl.attr[l];
    for (int g = 0; g < GBR_MAX_BIND_GROUPS; ++g) {
        const BindGroup* bg = dc.groups[g].get();
        if (!bg) continue;
        for (uint32_t e = 0; e < bg->desc.entry_count; ++e) {
            const gbr_bind_group_entry& en = bg->desc.entries[e];
            if (en.binding >= 8) continue;
            auto* obj = bg->refs[e].get();
            if (en.kind == GBR_BINDING_BUFFER) {
                auto* b = static_cast<Buffer*>(obj);
                uint64_t size = en.size ? en.size : b->size - en.offset;
                d.uniform[g][en.binding] = b->ptr + en.offset;
                d.uniform_size[g][en.binding] = size;
            } else if (en.kind == GBR_BINDING_TEXTURE_VIEW && g == prog.tex_group && (int)en.binding == prog.tex_binding) {
                auto* t = static_cast<Texture*>(obj);
                d.tex.data = t->ptr;
                d.tex.width = t->desc.size.width;
                d.tex.height = t->desc.size.height;
                d.tex.format = t->desc.format;
                d.tex.mip_count = t->mips_stored;
                for (uint32_t m = 0; m < t->mips_stored && m < 16; ++m) d.tex.mip_offset[m] = t->mip_offset[m];
            } else if (en.kind == GBR_BINDING_SAMPLER && g == prog.samp_group && (int)en.binding == prog.samp_binding) {
                auto* s = static_cast<Sampler*>(obj);
                d.samp.address_u = s->desc.address_mode_u;
                d.samp.address_v = s->desc.address_mode_v;
                d.samp.mag_filter = s->desc.mag_filter;
                d.samp.min_filter = s->desc.min_filter;
                d.samp.mip_filter = s->desc.mipmap_filter;
                d.samp.lod_min = s->desc.lod_min_clamp;
                d.samp.lod_max = s->desc.lod_max_clamp;
            }
        }
    }
    if (prog.uniform_min && (!d.uniform[0][0] || d.uniform_size[0][0] < prog.uniform_min))
        fail(GBR_ERR_VALIDATION, "No such binding resource: uniform @group(0) @binding(0)");
    for (int g = 0; g < 4; ++g)
        for (int b = 0; b < 8; ++b)
            if (prog.uniform_req[g][b] && (!d.uniform[g][b] || d.uniform_size[g][b] < prog.uniform_req[g][b]))
                fail(GBR_ERR_VALIDATION, "No such binding resource: uniform @group(%d) @binding(%d) of %u bytes", g, b,
                     prog.uniform_req[g][b]);
    if (prog.uses_texture) {
        if (!d.tex.data)
            fail(GBR_ERR_VALIDATION, "No such binding resource: texture @group(%d) @binding(%d)", prog.tex_group,
                 prog.tex_binding);
        if (d.tex.format != GBR_TEXTURE_FORMAT_RGBA8_UNORM && d.tex.format != GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB)
            fail(GBR_ERR_UNSUPPORTED, "sampling this texture format is todo!() (texture.rs:186)");
        if (d.samp.address_u == GBR_ADDRESS_CLAMP_TO_BORDER || d.samp.address_v == GBR_ADDRESS_CLAMP_TO_BORDER)
            fail(GBR_ERR_UNSUPPORTED, "ClampToBorder is todo!() (binding.rs:160)");
        bool have_sampler = false;
        const int gi = prog.samp_group;
        if (gi >= 0 && gi < GBR_MAX_BIND_GROUPS && dc.groups[gi])
            for (uint32_t e = 0; e < dc.groups[gi]->desc.entry_count; ++e)
                if (dc.groups[gi]->desc.entries[e].kind == GBR_BINDING_SAMPLER &&
                    (int)dc.groups[gi]->desc.entries[e].binding == prog.samp_binding)
                    have_sampler = true;
        if (!have_sampler)
            fail(GBR_ERR_VALIDATION, "No such binding resource: sampler @group(%d) @binding(%d)", prog.samp_group,
                 prog.samp_binding);
    }
    d.program = prog.id;
    d.has_fragment = pd.has_fragment;
    d.num_varyings = prog.num_varyings;
    d.interp = prog.perspective ? INTERP_PERSPECTIVE : INTERP_LINEAR;
    d.may_discard = prog.may_discard ? 1u : 0u;
    d.flat_mask = prog.flat_mask;
    d.early_depth = prog.early_depth;
    d.profile = profile;
    // extension-profile sampling needs the (u, v) derivatives: the native textured program's uv
    // are varyings 3 and 4 (lod_var = 1 + the index of u)
    d.lod_var = profile == GBR_PROFILE_EXTENSION && prog.id == PROG_MESH_TEX_LAMBERT ? 4u : 0u;
    d.cull_mode = ps.cull_mode;
    d.front_face = ps.front_face;
    // ToRaster::new (raster.rs:130-143): translation = offset + 0.5 size, scaling = 0.5 size, y *= -1
    volatile float vx = dc.viewport[0], vy = dc.viewport[1], vw = dc.viewport[2], vh = dc.viewport[3];
    d.vp_tx = vx + 0.5f * vw;
    d.vp_ty = vy + 0.5f * vh;
    d.vp_sx = 0.5f * vw;
    d.vp_sy = (0.5f * vh) * -1.0f;
    d.sc_x0 = dc.scissor[0];
    d.sc_y0 = dc.scissor[1];
    d.sc_x1 = dc.scissor[0] + dc.scissor[2];
    d.sc_y1 = dc.scissor[1] + dc.scissor[3];
    d.depth_test = (pd.has_depth_stencil && has_depth_attachment) ? 1u : 0u;
    d.depth_compare = pd.depth_stencil.depth_compare;
    d.depth_write = pd.depth_stencil.depth_write_enabled;
    d.write_mask = 0xF;
    if (profile == GBR_PROFILE_EXTENSION && pd.has_fragment && pd.color_target_count > 0) {
        const gbr_color_target_state& ct = pd.color_targets[0];
        d.blend_enabled = ct.has_blend;
        d.blend_color[0] = ct.color.src_factor;
        d.blend_color[1] = ct.color.dst_factor;
        d.blend_color[2] = ct.color.operation;
        d.blend_alpha[0] = ct.alpha.src_factor;
        d.blend_alpha[1] = ct.alpha.dst_factor;
        d.blend_alpha[2] = ct.alpha.operation;
        d.write_mask = ct.write_mask & 0xF;
    }
    for (int k = 0; k < 4; ++k) d.blend_constant[k] = (float)dc.blend_constant[k];
    d.fast_vs = fast_vs_kind(d);
    d.fast_vcount = fast_vs_vcount(d);
    d.fast_packed = fast_vs_packed(d);
    return d;
}

// ---------------------------------------------------------------- worker
uint64_t submission_estimate(const Item& it);
constexpr size_t kMaxGroup = 256;  // submissions merged into one launch at most
constexpr size_t kLookaheadItems = 8192;  // queue items the worker looks past for the next submission (a frame's writes can be hundreds)
constexpr size_t kMaxCoalescedWrites = 4096;           // small buffer writes uploaded together at most
constexpr uint64_t kMaxCoalescedBytes = 16ull << 20;  // and their bytes

// The next group of queue items (q_mu held): one item, a run of small buffer writes, or a
// submission with the submissions queued behind it that the HBM budget admits to its launch.
std::vector<Item> Device::pop_group_locked() {
    std::vector<Item> group;
    {
        {
            group.push_back(std::move(queue.front()));
            queue.pop_front();
            // continuous batching: the submissions queued behind this one join its launch while
            // their expected transient memory fits the HBM budget (the rest wait for the next)
            // a run of buffer writes (per-draw uniforms, meshes and the like) is placed by one
            // scatter kernel, still in queue order: the host-side bytes go up as one copy, the
            // device-staged ones are copied from their staging
            // (a write overlapping an earlier one of the run ends it: the scatter kernel places
            // segments concurrently, and the later bytes must win)
            if (group[0].kind == Item::WRITE_BUFFER) {
                auto host_bytes = [](const Item& it) { return it.staged ? uint64_t(0) : (uint64_t)it.data.size(); };
                uint64_t bytes = host_bytes(group[0]);
                std::map<uint64_t, uint64_t> spans;  // destination [begin, end) of the run's writes
                auto span_of = [](const Item& it) {
                    const uint64_t b = reinterpret_cast<uint64_t>(it.buffer->ptr) + it.offset;
                    return std::make_pair(b, b + (it.staged ? it.staged_size : (uint64_t)it.data.size()));
                };
                spans.insert(span_of(group[0]));
                while (!queue.empty() && queue.front().kind == Item::WRITE_BUFFER &&
                       group.size() < kMaxCoalescedWrites && bytes + host_bytes(queue.front()) <= kMaxCoalescedBytes) {
                    const auto sp = span_of(queue.front());
                    auto next = spans.lower_bound(sp.first);
                    if (next != spans.end() && next->first < sp.second) break;
                    if (next != spans.begin() && std::prev(next)->second > sp.first) break;
                    spans.insert(sp);
                    bytes += host_bytes(queue.front());
                    group.push_back(std::move(queue.front()));
                    queue.pop_front();
                }
            }
            if (group[0].kind == Item::SUBMIT && cfg.batch_submissions) {
                // the first submission always runs (it fails with OUT_OF_MEMORY if it cannot fit)
                const uint64_t budget = transient_budget();
                uint64_t est = GBR_ADMISSION_GROUP_BYTES + submission_estimate(group[0]);
                while (!queue.empty() && queue.front().kind == Item::SUBMIT && group.size() < kMaxGroup) {
                    const uint64_t e = submission_estimate(queue.front());
                    if (est + e > budget) break;
                    est += e;
                    group.push_back(std::move(queue.front()));
                    queue.pop_front();
                }
            }
        }
    }
    return group;
}

void Device::worker_main() {
    cudaSetDevice(ordinal);
    // Host planning of the next queued submission group runs on this helper thread while the
    // worker's current group is on the device (planning reads only host-side objects).
    Planner planner(this);
    for (;;) {
        std::vector<Item> group;
        {
            std::unique_lock<std::mutex> lk(q_mu);
            if (queue.empty() && (!pending_reads.empty() || !deferred_reads.empty())) {  // idle: the readbacks complete
                lk.unlock();
                finish_reads(UINT64_MAX);
                continue;
            }
            q_cv.wait(lk, [&] { return stopping || !queue.empty(); });
            if (queue.empty() && stopping) return;
            group = pop_group_locked();
        }
        if (group[0].kind != Item::SUBMIT) {
            if (group.size() > 1) execute_writes(group);
            else execute(group[0]);
            continue;
        }
        PlannedGroup cur = plan_group(std::move(group));
        la_planner = &planner;
        for (;;) {
            // look ahead: the next queued submission group is planned while this one runs, also
            // past writes, reads and cache flushes queued before it (planning reads only host-side
            // objects, which those do not change); they run, in queue order, after this group.
            // The queue is looked at now and again just before the worker waits for the launch.
            la_ahead = false;
            la_between.clear();
            lookahead();
            run_group(cur);
            for (std::vector<Item>& g : la_between) {
                if (g.size() > 1) execute_writes(g);
                else execute(g[0]);
            }
            la_between.clear();
            if (!la_ahead) break;
            cur = planner.finish();
        }
        la_planner = nullptr;
    }
}

// Hands the next queued submission group (and the writes, reads and flushes queued before it) to
// the planner, once per group the worker runs (la_ahead).
void Device::lookahead() {
    if (!la_planner || la_ahead) return;
    std::lock_guard<std::mutex> lk(q_mu);
    size_t k = 0;
    while (k < queue.size() && k < kLookaheadItems && queue[k].kind != Item::SUBMIT) ++k;
    if (k < queue.size() && queue[k].kind == Item::SUBMIT) {
        while (queue.front().kind != Item::SUBMIT) la_between.push_back(pop_group_locked());
        la_planner->start(pop_group_locked());
        la_ahead = true;
    }
}

// Coalesced buffer writes: the host-side bytes copied into one pinned block (16-byte aligned
// offsets, the segment table after them) and uploaded into device scratch with one copy; one
// scatter kernel then places every write, from that scratch or from the write's device staging,
// cut into pieces of kScatterPiece bytes so that many blocks share a large write.
constexpr uint64_t kScatterPiece = 64u << 10;
void Device::execute_writes(std::vector<Item>& items) {
    try {
        if (lost) fail(GBR_ERR_DEVICE_LOST, "device lost: %s", lost_msg.c_str());
        auto size_of = [](const Item& it) { return it.staged ? it.staged_size : (uint64_t)it.data.size(); };
        uint64_t data_bytes = 0, nseg = 0;
        for (const Item& it : items) {
            if (!it.staged) data_bytes += (it.data.size() + 15) & ~uint64_t(15);
            nseg += (size_of(it) + kScatterPiece - 1) / kScatterPiece;
        }
        if (nseg > UINT32_MAX) fail(GBR_ERR_UNSUPPORTED, "too many write segments");
        const uint64_t total = data_bytes + nseg * 3 * sizeof(uint64_t);
        PinnedStage& ps = pinned_stage[pinned_next];
        pinned_next ^= 1;
        if (ps.done) cuda_check(cudaEventSynchronize(ps.done), "pinned staging reuse");
        else cuda_check(cudaEventCreateWithFlags(&ps.done, cudaEventDisableTiming), "cudaEventCreate");
        if (ps.size < total) {
            if (ps.ptr) cudaFreeHost(ps.ptr);
            ps.ptr = nullptr;
            ps.size = 0;
            const size_t want = std::max<size_t>(total, 1u << 20);
            cuda_check(cudaHostAlloc(reinterpret_cast<void**>(&ps.ptr), want, cudaHostAllocDefault), "cudaHostAlloc");
            ps.size = want;
        }
        upload_buf.ensure(total, &scratch_bytes);
        const uint64_t dev_stage = reinterpret_cast<uint64_t>(upload_buf.ptr);
        uint64_t* desc = reinterpret_cast<uint64_t*>(ps.ptr + data_bytes);
        uint64_t off = 0, s = 0;
        for (const Item& it : items) {
            const uint64_t size = size_of(it);
            uint64_t src = reinterpret_cast<uint64_t>(it.staged);
            if (!it.staged) {
                std::memcpy(ps.ptr + off, it.data.data(), size);
                src = dev_stage + off;
                off += (size + 15) & ~uint64_t(15);
            }
            const uint64_t dst = reinterpret_cast<uint64_t>(it.buffer->ptr + it.offset);
            for (uint64_t p = 0; p < size; p += kScatterPiece, ++s) {
                desc[3 * s] = dst + p;
                desc[3 * s + 1] = src + p;
                desc[3 * s + 2] = std::min(kScatterPiece, size - p);
            }
        }
        cuda_check(cudaMemcpyAsync(upload_buf.ptr, ps.ptr, total, cudaMemcpyHostToDevice, stream), "coalesced writes");
        cuda_check(cudaEventRecord(ps.done, stream), "cudaEventRecord");
        cuda_check(launch_scatter_writes(reinterpret_cast<const uint64_t*>(dev_stage + data_bytes), (uint32_t)nseg, stream),
                   "scatter writes");
        for (Item& it : items)  // stream-ordered after the kernel that reads them
            if (it.staged) {
                cuda_check(cudaFreeAsync(it.staged, stream), "write_buffer staging");
                it.staged = nullptr;
            }
    } catch (const Failure& f) {
        note_failure(f);
    }
}

void Device::execute(Item& it) {
    Failure err{GBR_OK, ""};
    bool deferred = false;  // an asynchronous readback: completed later, by finish_reads
    try {
        if (lost) fail(GBR_ERR_DEVICE_LOST, "device lost: %s", lost_msg.c_str());
        switch (it.kind) {
            case Item::WRITE_BUFFER:
                if (it.staged) {
                    cuda_check(cudaMemcpyAsync(it.buffer->ptr + it.offset, it.staged, it.staged_size,
                                               cudaMemcpyDeviceToDevice, stream),
                               "write_buffer");
                    cuda_check(cudaFreeAsync(it.staged, stream), "write_buffer staging");
                    it.staged = nullptr;
                } else {
                    cuda_check(cudaMemcpyAsync(it.buffer->ptr + it.offset, it.data.data(), it.data.size(),
                                               cudaMemcpyHostToDevice, stream),
                               "write_buffer");
                }
                break;
            case Item::WRITE_TEXTURE: {
                Texture& t = *it.texture;
                wait_reads_of(&t);
                uint32_t w = t.mip_w(it.mip), h = t.mip_h(it.mip), layers = t.layers();
                uint64_t row = (uint64_t)w * t.bpp;
                const uint64_t src_size = it.staged ? it.staged_size : it.data.size();
                uint64_t src_row = it.layout.bytes_per_row ? it.layout.bytes_per_row : src_size;
                uint64_t rows_per_image = it.layout.rows_per_image ? it.layout.rows_per_image : h;
                uint8_t* dst = t.ptr + t.mip_offset[it.mip];
                const uint8_t* src = it.staged ? static_cast<const uint8_t*>(it.staged) : it.data.data();
                for (uint32_t z = 0; z < layers; ++z)
                    cuda_check(cudaMemcpy2DAsync(dst + (uint64_t)z * h * row, row,
                                                 src + it.layout.offset + z * rows_per_image * src_row, src_row, row,
                                                 h, it.staged ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                                 stream),
                               "write_texture");
                if (it.staged) {
                    cuda_check(cudaFreeAsync(it.staged, stream), "write_texture staging");
                    it.staged = nullptr;
                }
                break;
            }
            case Item::READ_BUFFER:
                cuda_check(cudaMemcpyAsync(it.dst, it.buffer->ptr + it.offset, it.size, cudaMemcpyDeviceToHost, stream),
                           "buffer_read");
                cuda_check(cudaStreamSynchronize(stream), "buffer_read sync");
                break;
            case Item::READ_TEXTURE:
                cuda_check(cudaMemcpyAsync(it.dst, it.texture->ptr + it.texture->mip_offset[it.mip],
                                           it.texture->mip_bytes(it.mip), cudaMemcpyDeviceToHost, stream),
                           "texture_read");
                cuda_check(cudaStreamSynchronize(stream), "texture_read sync");
                break;
            case Item::READ_TEXTURES: {
                if (it.indexed) {
                    // asynchronous: its place in the queue's stream marked now, its copies (copy
                    // engines, rb_stream) issued by issue_reads
                    DeferredRead dr;
                    cuda_check(cudaEventCreateWithFlags(&dr.ready, cudaEventDisableTiming), "cudaEventCreate");
                    const cudaError_t e = cudaEventRecord(dr.ready, stream);
                    if (e != cudaSuccess) cudaEventDestroy(dr.ready);
                    cuda_check(e, "readback ordering");
                    dr.item.kind = it.kind;
                    dr.item.index = it.index;
                    dr.item.t_submit = it.t_submit;
                    dr.item.textures = std::move(it.textures);
                    dr.item.mips = std::move(it.mips);
                    dr.item.dsts = std::move(it.dsts);
                    deferred_reads.push_back(std::move(dr));
                    deferred = true;
                    break;
                }
                // Destinations the device can address (pinned host memory, as the attributes report
                // it) are written by one copy kernel over all SMs, which moves the bytes over the
                // CPU-GPU link faster than one copy-engine transfer per texture; any other
                // destination (pageable, unaligned) takes cudaMemcpyAsync.
                CopyOutJobs jobs{};
                for (size_t k = 0; k < it.textures.size(); ++k) {
                    const Texture& t = *it.textures[k];
                    const uint8_t* src = t.ptr + t.mip_offset[it.mips[k]];
                    const uint64_t n = t.mip_bytes(it.mips[k]);
                    // both ends of the destination mapped, at the same distance on the device side
                    cudaPointerAttributes pa{}, pe{};
                    void* dev_dst = nullptr;
                    const uint8_t* last = static_cast<const uint8_t*>(it.dsts[k]) + (n ? n - 1 : 0);
                    if (cudaPointerGetAttributes(&pa, it.dsts[k]) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
                        pa.devicePointer != nullptr && cudaPointerGetAttributes(&pe, last) == cudaSuccess &&
                        pe.type == cudaMemoryTypeHost &&
                        static_cast<const uint8_t*>(pe.devicePointer) == static_cast<const uint8_t*>(pa.devicePointer) + (n ? n - 1 : 0))
                        dev_dst = pa.devicePointer;
                    else
                        cudaGetLastError();  // clear a failed query: the copy below takes over
                    if (dev_dst && ((reinterpret_cast<uintptr_t>(dev_dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
                        jobs.src[jobs.n] = src;
                        jobs.dst[jobs.n] = static_cast<uint8_t*>(dev_dst);
                        jobs.bytes[jobs.n] = n;
                        if (++jobs.n == kCopyOutMax) {
                            cuda_check(launch_copy_out(jobs, num_sms, stream), "textures_read");
                            jobs.n = 0;
                        }
                    } else {
                        cuda_check(cudaMemcpyAsync(it.dsts[k], src, n, cudaMemcpyDeviceToHost, stream), "textures_read");
                    }
                }
                cuda_check(launch_copy_out(jobs, num_sms, stream), "textures_read");
                cuda_check(cudaStreamSynchronize(stream), "textures_read sync");
                break;
            }
            case Item::FLUSH:
                flush_buf.ensure(256ull << 20, &scratch_bytes);
                cuda_check(cudaMemsetAsync(flush_buf.ptr, (int)(it.offset & 0xFF), flush_buf.size, stream), "flush");
                break;
            case Item::SUBMIT: break;  // submissions run through execute_group
        }
    } catch (const Failure& f) {
        err = f;
        note_failure(f);
    }
    if (it.done) it.done->set_value(err);
    if (it.indexed && !deferred) {  // an asynchronous readback that failed before its copies: done now
        std::lock_guard<std::mutex> lk(q_mu);
        SubmissionRecord rec;
        rec.status = err.status;
        rec.error = err.msg;
        rec.stats.submission_index = it.index;
        rec.stats.submit_to_fence_ms = ms_between(it.t_submit, Clock::now());
        records[it.index] = rec;
        completed_submissions = std::max(completed_submissions, it.index + 1);
        while (records.size() > kKeptRecords) records.erase(records.begin());
        done_cv.notify_all();
    }
}

// Issues the copies of the deferred readbacks, in queue order: each on rb_stream after its
// `ready` mark, then its `done` event, which becomes the fence of its textures.  A readback whose
// copies cannot be issued completes at once with the error.
void Device::issue_reads() {
    while (!deferred_reads.empty()) {
        DeferredRead dr = std::move(deferred_reads.front());
        deferred_reads.pop_front();
        Item& it = dr.item;
        auto done = std::make_shared<ReadFence>();
        cudaError_t e = cudaStreamWaitEvent(rb_stream, dr.ready, 0);
        cudaEventDestroy(dr.ready);  // released once the wait is satisfied
        for (size_t k = 0; e == cudaSuccess && k < it.textures.size(); ++k) {
            const Texture& t = *it.textures[k];
            e = cudaMemcpyAsync(it.dsts[k], t.ptr + t.mip_offset[it.mips[k]], t.mip_bytes(it.mips[k]),
                                cudaMemcpyDeviceToHost, rb_stream);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done->ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(done->ev, rb_stream);
        if (e != cudaSuccess) {
            note_failure(Failure{GBR_ERR_CUDA, cudaGetErrorString(e)});
            std::lock_guard<std::mutex> lk(q_mu);
            SubmissionRecord rec;
            rec.status = GBR_ERR_CUDA;
            rec.error = cudaGetErrorString(e);
            rec.stats.submission_index = it.index;
            records[it.index] = rec;
            completed_submissions = std::max(completed_submissions, it.index + 1);
            done_cv.notify_all();
            continue;
        }
        for (const auto& t : it.textures) read_fence[t.get()] = done;
        pending_reads.push_back(PendingRead{it.index, done, std::move(it.textures), it.t_submit});
    }
}

// Completes the asynchronous readbacks with index < before, in order: waits for each one's
// copies, records it like a submission and drops the fences that still point at it.
void Device::finish_reads(uint64_t before) {
    issue_reads();
    while (!pending_reads.empty() && pending_reads.front().index < before) {
        PendingRead pr = std::move(pending_reads.front());
        pending_reads.pop_front();
        const cudaError_t e = cudaEventSynchronize(pr.done->ev);
        for (const auto& t : pr.keep) {
            auto f = read_fence.find(t.get());
            if (f != read_fence.end() && f->second == pr.done) read_fence.erase(f);
        }
        if (e != cudaSuccess) note_failure(Failure{GBR_ERR_CUDA, cudaGetErrorString(e)});
        std::lock_guard<std::mutex> lk(q_mu);
        SubmissionRecord rec;
        rec.status = e == cudaSuccess ? GBR_OK : GBR_ERR_CUDA;
        if (e != cudaSuccess) rec.error = cudaGetErrorString(e);
        rec.stats.submission_index = pr.index;
        rec.stats.submit_to_fence_ms = ms_between(pr.t_submit, Clock::now());
        records[pr.index] = rec;
        completed_submissions = std::max(completed_submissions, pr.index + 1);
        while (records.size() > kKeptRecords) records.erase(records.begin());
        done_cv.notify_all();
    }
}

void Device::note_failure(const Failure& f) {
    cudaError_t ce = cudaGetLastError();
    if (f.status == GBR_ERR_CUDA || f.status == GBR_ERR_DEVICE_LOST || ce != cudaSuccess) {
        std::lock_guard<std::mutex> lk(q_mu);
        lost = true;
        if (lost_msg.empty()) lost_msg = f.msg;
    }
}

// Transient device memory a submission is expected to need (records, bins, tile arrays):
// what admission counts against the HBM budget.
uint64_t submission_estimate(const Item& it) {
    uint64_t prims = 0, pixels = 0;
    for (const PassCmd& p : it.passes) {
        pixels += (uint64_t)p.width * p.height;
        for (const DrawCmd& dc : p.draws) {
            const uint64_t cnt = dc.end > dc.start ? dc.end - dc.start : 0;
            prims += (cnt / 3 + 2) * (dc.inst_end > dc.inst_start ? dc.inst_end - dc.inst_start : 0);
        }
    }
    return prims * GBR_ADMISSION_BYTES_PER_PRIMITIVE + pixels / 16 + 4096;
}

// A run of submissions executed together (one, unless the config merges queued submissions).
// Each is planned on its own, so a submission that fails validation fails alone; submissions
// that plan to a single batch are merged into one launch batch while no pass of one writes a
// texture another reads or writes; the group's batches are launched back to back and every
// submission gets its own record (fragments counted per target on the device).
// Host planning of a submission group (no device work): each submission planned on its own (a
// validation failure fails only it), single-batch submissions merged while hazard-free.
PlannedGroup Device::plan_group(std::vector<Item>&& items) {
    PlannedGroup g;
    g.items = std::move(items);
    const size_t n = g.items.size();
    g.recs.resize(n);
    auto& recs = g.recs;
    auto& batches = g.batches;
    auto fail_item = [&](size_t i, gbr_status st, const std::string& msg) {
        if (recs[i].status == GBR_OK) {
            recs[i].status = st;
            recs[i].error = msg;
        }
    };
    try {
        bool open = false;  // the last batch accepts another single-batch submission
        for (size_t i = 0; i < n; ++i) {
            recs[i].stats.batched_with = (uint32_t)n;
            std::vector<Batch> own;
            try {
                uint64_t draws = 0, prims = 0;
                own = plan_batches(g.items[i].passes, &draws, &prims, (uint32_t)i);
                recs[i].stats.draws = draws;
                recs[i].stats.primitives_in = prims;
            } catch (const Failure& f) {
                fail_item(i, f.status, f.msg);
                continue;
            }
            const bool single = own.size() == 1;
            if (single && open && merge_batch(batches.back(), own[0])) continue;
            for (Batch& b : own) batches.push_back(std::move(b));
            open = single && cfg.batch_submissions && cfg.launch_mode == GBR_LAUNCH_BATCHED;
        }
    } catch (const Failure& f) {
        g.failure = f;
    }
    return g;
}

// The group's batches on the device (retries included), then every submission's record.
void Device::run_group(PlannedGroup& g) {
    std::vector<Item>& items = g.items;
    const size_t n = items.size();
    std::vector<SubmissionRecord>& recs = g.recs;
    std::vector<Batch>& batches = g.batches;
    const auto t_start = Clock::now();
    for (size_t i = 0; i < n; ++i) recs[i].stats.queue_wait_ms = ms_between(items[i].t_submit, t_start);
    auto fail_item = [&](size_t i, gbr_status st, const std::string& msg) {
        if (recs[i].status == GBR_OK) {
            recs[i].status = st;
            recs[i].error = msg;
        }
    };
    GroupRun run;
    try {
        if (lost) fail(GBR_ERR_DEVICE_LOST, "device lost: %s", lost_msg.c_str());
        if (g.failure.status != GBR_OK) throw g.failure;
        // textures the group writes wait for their readbacks in flight (copies: all of them)
        if (!read_fence.empty() || !deferred_reads.empty())
            for (const Batch& b : batches) {
                if (b.copy) wait_all_reads();
                for (const Texture* t : b.writes) wait_reads_of(t);
            }
        size_t from = 0;
        while (from < batches.size()) {
            const RunResult r = run_batches(batches, from, run);
            if (r.bad == batches.size()) break;
            Batch& bad = batches[r.bad];
            std::vector<uint32_t> its;
            for (uint32_t ti : bad.target_item)
                if (std::find(its.begin(), its.end(), ti) == its.end()) its.push_back(ti);
            if (its.size() > 1) {
                // a merged batch failed: run its submissions' parts separately to find the culprit
                std::vector<Batch> parts = split_batch(bad);
                batches.erase(batches.begin() + (ptrdiff_t)r.bad);
                batches.insert(batches.begin() + (ptrdiff_t)r.bad, std::make_move_iterator(parts.begin()),
                               std::make_move_iterator(parts.end()));
                from = r.bad;
                continue;
            }
            const uint32_t culprit = its.empty() ? bad.item : its[0];
            fail_item(culprit, GBR_ERR_VALIDATION, r.msg);
            // the failed submission's later batches do not run
            size_t k = r.bad + 1;
            while (k < batches.size() && batches[k].item == culprit && batches[k].single_item) batches.erase(batches.begin() + (ptrdiff_t)k);
            from = r.bad + 1;
        }
    } catch (const Failure& f) {
        note_failure(f);
        for (size_t i = 0; i < n; ++i) fail_item(i, f.status, f.msg);
    }
    // per-submission fragment counts from the per-target counters
    std::vector<uint64_t> frags(n, 0), fs_runs(n, 0), tex_runs(n, 0);
    for (const Batch& b : batches)
        for (size_t t = 0; t < b.target_item.size() && (t + 1) * kTargetCounters <= b.target_frags.size(); ++t) {
            frags[b.target_item[t]] += b.target_frags[t * kTargetCounters];
            fs_runs[b.target_item[t]] += b.target_frags[t * kTargetCounters + 1];
            tex_runs[b.target_item[t]] += b.target_frags[t * kTargetCounters + 2];
        }
    float group_ms = 0.0f;
    if (run.ev && run.started) cudaEventElapsedTime(&group_ms, run.ev->start, run.ev->end);
    // readbacks queued before these submissions complete first (completion is in queue order)
    if (!pending_reads.empty() || !deferred_reads.empty()) {
        uint64_t first = UINT64_MAX;
        for (size_t i = 0; i < n; ++i) first = std::min(first, items[i].index);
        finish_reads(first);
    }
    std::lock_guard<std::mutex> lk(q_mu);
    for (size_t i = 0; i < n; ++i) {
        SubmissionRecord& rec = recs[i];
        rec.stats.submission_index = items[i].index;
        rec.stats.submit_to_fence_ms = ms_between(items[i].t_submit, Clock::now());
        rec.stats.fragments_shaded = rec.status == GBR_OK ? frags[i] : 0;
        rec.stats.fs_invocations = rec.status == GBR_OK ? fs_runs[i] : 0;
        rec.stats.texture_fs_invocations = rec.status == GBR_OK ? tex_runs[i] : 0;
        rec.stats.kernel_launches = run.launches;
        rec.stats.gpu_ms = group_ms;
        rec.stats.raster_ms = run.raster_ms;
        rec.stats.generic_setup_prims = (uint32_t)std::min<uint64_t>(run.slow_prims, 0xFFFFFFFFu);
        rec.stats.split_tile_chunks = (uint32_t)std::min<uint64_t>(run.split_chunks, 0xFFFFFFFFu);
        rec.stats.tile_shape = run.tile_shape;
        rec.ev = run.started ? run.ev : nullptr;
        records[items[i].index] = rec;
        completed_submissions = std::max(completed_submissions, items[i].index + 1);
    }
    while (records.size() > kKeptRecords) records.erase(records.begin());
    done_cv.notify_all();
}

// Appends single-submission batch `b` to batch `into` when no pass of one touches a texture the
// other writes and the primitive ids still fit; returns false (nothing changed) otherwise.
bool Device::merge_batch(Batch& into, Batch& b) {
    auto has = [](const std::vector<const Texture*>& v, const Texture* t) {
        return t && std::find(v.begin(), v.end(), t) != v.end();
    };
    for (const Texture* t : b.writes)
        if (has(into.writes, t) || has(into.reads, t)) return false;
    for (const Texture* t : b.reads)
        if (has(into.writes, t)) return false;
    const uint64_t kMaxPrims = (1ull << (32 - SUBTRI_BITS)) - 1;
    if ((uint64_t)into.total_prims + b.total_prims > kMaxPrims) return false;
    if (into.jit && b.jit && into.jit != b.jit) return false;
    if (into.copy || b.copy) return false;
    if (into.lines || b.lines) return false;
    if (!into.jit) into.jit = b.jit;
    const uint32_t tbase = (uint32_t)into.targets.size();
    for (DrawDesc d : b.draws) {
        d.prim_base += into.total_prims;
        d.target += tbase;
        d.strip_table += into.strip_entries;
        into.draws.push_back(d);
    }
    into.strip_entries += b.strip_entries;
    into.targets.insert(into.targets.end(), b.targets.begin(), b.targets.end());
    into.target_item.insert(into.target_item.end(), b.target_item.begin(), b.target_item.end());
    into.writes.insert(into.writes.end(), b.writes.begin(), b.writes.end());
    into.reads.insert(into.reads.end(), b.reads.begin(), b.reads.end());
    into.total_prims += b.total_prims;
    into.nvar = std::max(into.nvar, b.nvar);
    into.single_item = false;
    return true;
}

// The per-submission batches a merged batch was made of.
std::vector<Batch> Device::split_batch(const Batch& m) {
    std::vector<Batch> out;
    std::vector<int> item_batch;
    std::vector<uint32_t> new_target(m.targets.size());
    for (size_t t = 0; t < m.targets.size(); ++t) {
        const uint32_t it = m.target_item[t];
        size_t k = 0;
        while (k < out.size() && out[k].item != it) ++k;
        if (k == out.size()) {
            out.emplace_back();
            out.back().item = it;
            out.back().single_item = true;
            out.back().jit = m.jit;
        }
        new_target[t] = (uint32_t)out[k].targets.size();
        out[k].targets.push_back(m.targets[t]);
        out[k].target_item.push_back(it);
    }
    for (const DrawDesc& d0 : m.draws) {
        const uint32_t it = m.target_item[d0.target];
        size_t k = 0;
        while (out[k].item != it) ++k;
        DrawDesc d = d0;
        const uint64_t np = (uint64_t)d.prims_per_instance * d.instance_count;
        d.prim_base = out[k].total_prims;
        d.target = new_target[d0.target];
        if (d.strip_restart) {
            d.strip_table = out[k].strip_entries;
            out[k].strip_entries += d.count;
        }
        out[k].total_prims += (uint32_t)np;
        out[k].nvar = std::max(out[k].nvar, d.num_varyings);
        out[k].draws.push_back(d);
    }
    return out;
}

// Splits a list of render passes into launch batches.
//  PER_DRAW  one batch per draw (the pass's load ops apply to its first draw);
//  PER_PASS  one batch per pass;
//  BATCHED   consecutive passes share a batch until one would touch a texture an earlier pass of
//            the batch writes (as an attachment) or reads (as a bound texture), or write one it
//            reads — so no batch contains a dependency between its passes.
std::vector<Batch> Device::plan_batches(const std::vector<PassCmd>& passes, uint64_t* draws, uint64_t* prims_in,
                                        uint32_t item) {
    const uint32_t profile = cfg.profile;
    std::vector<Batch> batches;
    bool open = false;
    auto has = [](const std::vector<const Texture*>& v, const Texture* t) {
        return t && std::find(v.begin(), v.end(), t) != v.end();
    };
    auto new_batch = [&]() -> Batch& {
        batches.emplace_back();
        batches.back().item = item;
        batches.back().single_item = true;
        return batches.back();
    };
    for (const PassCmd& p : passes) {
        if (p.copy) {  // ordered between the passes around it: closes the open batch
            open = false;
            new_batch().copy = p.copy;
            continue;
        }
        if (p.width == 0 || p.height == 0) continue;
        std::vector<const Texture*> p_write, p_read;
        if (p.color) p_write.push_back(p.color.get());
        if (p.depth) p_write.push_back(p.depth.get());
        for (const DrawCmd& dc : p.draws)
            for (const auto& g : dc.groups)
                if (g)
                    for (const auto& ref : g->refs)
                        if (auto* t = dynamic_cast<const Texture*>(ref.get())) p_read.push_back(t);
        uint64_t p_prims = 0;
        for (const DrawCmd& dc : p.draws) {
            const auto& ps = dc.pipeline->desc.primitive;
            uint32_t cnt = dc.end > dc.start ? dc.end - dc.start : 0;
            uint32_t ppi = primitive_slots(ps.topology, cnt);
            p_prims += (uint64_t)ppi * (dc.inst_end > dc.inst_start ? dc.inst_end - dc.inst_start : 0);
        }
        const uint64_t kMaxPrims = (1ull << (32 - SUBTRI_BITS)) - 1;
        // the WGSL modules the pass's draws run: one batch runs at most one
        std::shared_ptr<JitKernels> p_jit;
        bool several_jit = false, has_lines = false;
        for (const DrawCmd& dc : p.draws) {
            if (dc.pipeline->jit) {
                if (p_jit && p_jit != dc.pipeline->jit) several_jit = true;
                p_jit = dc.pipeline->jit;
            }
            has_lines = has_lines || dc.pipeline->desc.primitive.topology < GBR_TOPOLOGY_TRIANGLE_LIST;
        }
        // a pass with line or point draws goes draw by draw (each line/point draw is a batch of
        // its own, drawn in primitive order)
        if ((cfg.launch_mode == GBR_LAUNCH_PER_DRAW || several_jit || has_lines) && !p.draws.empty()) {
            open = false;
            bool first = true;
            for (const DrawCmd& dc : p.draws) {
                ++*draws;
                Batch& b = new_batch();
                b.targets.push_back(make_target(p, first, tile, profile));
                b.target_item.push_back(item);
                b.writes = p_write;
                b.reads = p_read;
                b.jit = dc.pipeline->jit;
                b.lines = dc.pipeline->desc.primitive.topology < GBR_TOPOLOGY_TRIANGLE_LIST;
                first = false;
                DrawDesc d = make_draw(dc, profile, (bool)p.depth);
                d.raster_rule = cfg.raster_rule;
                uint64_t np = (uint64_t)d.prims_per_instance * d.instance_count;
                *prims_in += np;
                if (np > kMaxPrims) fail(GBR_ERR_UNSUPPORTED, "too many primitives in one draw");
                b.total_prims = (uint32_t)np;
                b.nvar = d.num_varyings;
                if (d.strip_restart) {
                    d.strip_table = 0;
                    b.strip_entries = d.count;
                }
                if (np) b.draws.push_back(d);
            }
            continue;
        }
        bool conflict = !open || cfg.launch_mode == GBR_LAUNCH_PER_PASS;
        if (!conflict) {
            const Batch& cur = batches.back();
            for (const Texture* t : p_write) conflict = conflict || has(cur.writes, t) || has(cur.reads, t);
            for (const Texture* t : p_read) conflict = conflict || has(cur.writes, t);
            if ((uint64_t)cur.total_prims + p_prims > kMaxPrims) conflict = true;
            if (p_jit && cur.jit && p_jit != cur.jit) conflict = true;
        }
        if (conflict) {
            new_batch();
            open = true;
        }
        Batch& b = batches.back();
        if (p_jit) b.jit = p_jit;
        const uint32_t ti = (uint32_t)b.targets.size();
        b.targets.push_back(make_target(p, true, tile, profile));
        b.target_item.push_back(item);
        for (const DrawCmd& dc : p.draws) {
            ++*draws;
            DrawDesc d = make_draw(dc, profile, (bool)p.depth);
            d.raster_rule = cfg.raster_rule;
            d.prim_base = b.total_prims;
            d.target = ti;
            uint64_t np = (uint64_t)d.prims_per_instance * d.instance_count;
            *prims_in += np;
            if ((uint64_t)b.total_prims + np > kMaxPrims) fail(GBR_ERR_UNSUPPORTED, "too many primitives in one pass");
            b.total_prims += (uint32_t)np;
            b.nvar = std::max(b.nvar, d.num_varyings);
            if (d.strip_restart && np) {
                d.strip_table = b.strip_entries;
                b.strip_entries += d.count;
            }
            if (np) b.draws.push_back(d);
        }
        b.writes.insert(b.writes.end(), p_write.begin(), p_write.end());
        b.reads.insert(b.reads.end(), p_read.begin(), p_read.end());
    }
    return batches;
}

// Launches batches[from..] back to back: each batch's tile shape (fixed by the config, or by
// the autotuner), tile layout, descriptors and per-target fragment counters; re-runs from a
// batch that ran out of scratch space after growing it.  Returns the first batch that failed
// validation on the device (batches before it completed), or batches.size().
// Stream-ordered execution of a copy or clear (extension profile).  Textures store mip m at
// mip_offset[m], its layers back to back, rows tightly packed.
void execute_copy(const CopyCmd& c, cudaStream_t s) {
    auto texel = [](const Texture& t, uint32_t mip, uint32_t x, uint32_t y, uint32_t z) {
        const uint64_t row = (uint64_t)t.mip_w(mip) * t.bpp;
        return t.ptr + t.mip_offset[mip] + ((uint64_t)z * t.mip_h(mip) + y) * row + (uint64_t)x * t.bpp;
    };
    switch (c.op) {
        case GBR_OP_COPY_BUFFER_TO_BUFFER:
            cuda_check(cudaMemcpyAsync(c.buf2->ptr + c.off2, c.buf->ptr + c.off, c.size, cudaMemcpyDeviceToDevice, s),
                       "copy_buffer_to_buffer");
            break;
        case GBR_OP_COPY_BUFFER_TO_TEXTURE:
        case GBR_OP_COPY_TEXTURE_TO_BUFFER: {
            const Texture& t = *c.tex;
            const uint64_t width = (uint64_t)c.ext.width * t.bpp;
            const uint64_t bpr = c.layout.bytes_per_row ? c.layout.bytes_per_row : width;
            const uint64_t rpi = c.layout.rows_per_image ? c.layout.rows_per_image : c.ext.height;
            const uint64_t trow = (uint64_t)t.mip_w(c.mip) * t.bpp;
            for (uint32_t z = 0; z < c.ext.depth_or_array_layers; ++z) {
                uint8_t* tp = texel(t, c.mip, c.ox, c.oy, c.oz + z);
                uint8_t* bp = c.buf->ptr + c.layout.offset + z * rpi * bpr;
                if (c.op == GBR_OP_COPY_BUFFER_TO_TEXTURE)
                    cuda_check(cudaMemcpy2DAsync(tp, trow, bp, bpr, width, c.ext.height, cudaMemcpyDeviceToDevice, s),
                               "copy_buffer_to_texture");
                else
                    cuda_check(cudaMemcpy2DAsync(bp, bpr, tp, trow, width, c.ext.height, cudaMemcpyDeviceToDevice, s),
                               "copy_texture_to_buffer");
            }
            break;
        }
        case GBR_OP_COPY_TEXTURE_TO_TEXTURE: {
            const Texture &a = *c.tex, &b = *c.tex2;
            const uint64_t width = (uint64_t)c.ext.width * a.bpp;
            for (uint32_t z = 0; z < c.ext.depth_or_array_layers; ++z)
                cuda_check(cudaMemcpy2DAsync(texel(b, c.mip2, c.ox2, c.oy2, c.oz2 + z), (uint64_t)b.mip_w(c.mip2) * b.bpp,
                                             texel(a, c.mip, c.ox, c.oy, c.oz + z), (uint64_t)a.mip_w(c.mip) * a.bpp,
                                             width, c.ext.height, cudaMemcpyDeviceToDevice, s),
                           "copy_texture_to_texture");
            break;
        }
        case GBR_OP_CLEAR_BUFFER:
            cuda_check(cudaMemsetAsync(c.buf->ptr + c.off, 0, c.size, s), "clear_buffer");
            break;
        case GBR_OP_CLEAR_TEXTURE: {
            const Texture& t = *c.tex;
            for (uint32_t m = c.mip; m < c.mip + c.mip_count; ++m) {
                const uint64_t layer = (uint64_t)t.mip_w(m) * t.mip_h(m) * t.bpp;
                cuda_check(cudaMemsetAsync(t.ptr + t.mip_offset[m] + c.oz * layer, 0, c.layer_count * layer, s),
                           "clear_texture");
            }
            break;
        }
        default: fail(GBR_ERR_INVALID_ARGUMENT, "copy opcode %u", c.op);
    }
}

RunResult Device::run_batches(std::vector<Batch>& batches, size_t from, GroupRun& run) {
    const size_t nb = batches.size();
    std::vector<int> btile(nb, tile), bwarps(nb, warps), tuning(nb, -1);
    for (size_t i = from; i < nb; ++i) {
        Batch& b = batches[i];
        int t = tile, w = warps;
        if (b.jit) {  // a WGSL module is compiled at one tile shape per raster kernel
            const bool vis = fragment_kind(b, cfg.raster_order == GBR_RASTER_AUTO) == 3;
            t = vis ? b.jit->vis_tile : b.jit->ord_tile;
            w = vis ? b.jit->vis_warps : b.jit->ord_warps;
        } else if (autotune) {
            tuning[i] = tuner_pick(b, &t, &w);
        }
        btile[i] = t;
        bwarps[i] = w;
        uint32_t base = 0;
        for (TargetDesc& td : b.targets) {
            td.tiles_x = (td.width + t - 1) / t;
            td.tiles_y = (td.height + t - 1) / t;
            td.tile_base = base;
            base += td.tiles_x * td.tiles_y;
        }
        b.total_tiles = base;
    }

    // metadata layout: [abort flag][statuses][work counters][fragment counters]
    //                  [draw/target descriptors (+ raster states) per batch]
    auto align = [](size_t v) { return (v + 255) & ~size_t(255); };
    size_t n_targets = 0;
    std::vector<size_t> counter_first(nb, 0);
    for (size_t i = from; i < nb; ++i) {
        counter_first[i] = n_targets;
        n_targets += batches[i].targets.size();
    }
    const size_t off_status = 256, off_work = align(off_status + nb * sizeof(BatchStatus));
    const size_t off_counters = align(off_work + nb * sizeof(uint32_t) * 4);
    const size_t off_desc = align(off_counters + n_targets * kTargetCounters * sizeof(unsigned long long));
    std::vector<size_t> desc_off(nb, 0), states_off(nb, 0);
    std::vector<int> kinds(nb, 0);
    std::vector<std::vector<uint32_t>> shape_tables(nb);
    struct SgOff {
        uint32_t v[8];
    };
    std::vector<SgOff> sg_offs(nb);
    auto shape_table_at = [](const Batch& b) {  // offset of the shape table in the batch's descriptors
        return (b.draws.size() * (sizeof(DrawDesc) + sizeof(uint32_t)) + b.targets.size() * sizeof(TargetDesc) + 7) &
               ~size_t(7);
    };
    size_t cur = off_desc;
    for (size_t i = from; i < nb; ++i) {
        kinds[i] = fragment_kind(batches[i], cfg.raster_order == GBR_RASTER_AUTO);
        desc_off[i] = cur;
        // descriptors, targets, the draws' first primitives as one contiguous table, then the
        // setup kernels' per-shape group table (8-byte aligned)
        shape_group_table(batches[i], shape_tables[i], sg_offs[i].v);
        cur = align(cur + shape_table_at(batches[i]) + shape_tables[i].size() * sizeof(uint32_t));
        if (kinds[i] == 3) {
            states_off[i] = cur;
            cur = align(cur + batches[i].draws.size() * raster_state_bytes());
        }
    }
    const uint64_t budget = cfg.hbm_budget_bytes ? cfg.hbm_budget_bytes : (80ull << 30);
    meta_buf.ensure(cur, &scratch_bytes);
    uint8_t* meta = static_cast<uint8_t*>(meta_buf.ptr);
    // the descriptors are built in pinned host memory (two buffers in turn, each reused once its
    // upload has completed), so their upload is an asynchronous DMA
    PinnedStage& hm = meta_stage[meta_next];
    meta_next ^= 1;
    if (hm.done) cuda_check(cudaEventSynchronize(hm.done), "descriptor staging reuse");
    else cuda_check(cudaEventCreateWithFlags(&hm.done, cudaEventDisableTiming), "cudaEventCreate");
    if (hm.size < cur) {
        if (hm.ptr) cudaFreeHost(hm.ptr);
        hm.ptr = nullptr;
        hm.size = 0;
        const size_t want = std::max<size_t>(cur, 1u << 20);
        cuda_check(cudaHostAlloc(reinterpret_cast<void**>(&hm.ptr), want, cudaHostAllocDefault), "cudaHostAlloc");
        hm.size = want;
    }
    uint8_t* const host_meta = hm.ptr;
    // the abort flag, statuses, work counters and fragment counters start at zero; the descriptor
    // regions below are written whole (the gaps between them are never read, and the raster
    // states are built on the device)
    std::memset(host_meta, 0, off_desc);
    for (size_t i = from; i < nb; ++i) {
        uint8_t* p = host_meta + desc_off[i];
        std::memcpy(p, batches[i].draws.data(), batches[i].draws.size() * sizeof(DrawDesc));
        TargetDesc* tp = reinterpret_cast<TargetDesc*>(p + batches[i].draws.size() * sizeof(DrawDesc));
        for (size_t t = 0; t < batches[i].targets.size(); ++t) {
            TargetDesc td = batches[i].targets[t];
            td.frag_count = reinterpret_cast<unsigned long long*>(meta + off_counters) + (counter_first[i] + t) * kTargetCounters;
            std::memcpy(tp + t, &td, sizeof td);
        }
        uint8_t* bases = p + batches[i].draws.size() * sizeof(DrawDesc) + batches[i].targets.size() * sizeof(TargetDesc);
        for (size_t k = 0; k < batches[i].draws.size(); ++k)
            std::memcpy(bases + k * sizeof(uint32_t), &batches[i].draws[k].prim_base, sizeof(uint32_t));
        if (!shape_tables[i].empty())
            std::memcpy(p + shape_table_at(batches[i]), shape_tables[i].data(), shape_tables[i].size() * sizeof(uint32_t));
    }
    cuda_check(cudaMemcpyAsync(meta, host_meta, cur, cudaMemcpyHostToDevice, stream), "upload descriptors");
    cuda_check(cudaEventRecord(hm.done, stream), "cudaEventRecord");

    if (!run.ev) {
        run.ev = std::make_shared<EventPair>();
        cuda_check(cudaEventCreate(&run.ev->start), "event");
        cuda_check(cudaEventCreate(&run.ev->end), "event");
    }
    size_t first_batch = from;
    std::vector<BatchStatus> st(nb);
    std::vector<unsigned long long> counters(n_targets * kTargetCounters);
    std::vector<cudaEvent_t> rev;  // raster kernel events (time_kernels)
    struct EventGuard {
        std::vector<cudaEvent_t>* v;
        ~EventGuard() {
            for (cudaEvent_t e : *v) cudaEventDestroy(e);
        }
    } rev_guard{&rev};
    const bool any_tuning = std::any_of(tuning.begin(), tuning.end(), [](int v) { return v >= 0; });
    if (cfg.time_kernels || any_tuning) {
        rev.resize(2 * nb);
        for (auto& e : rev) cuda_check(cudaEventCreate(&e), "event");
    }
    // the whole launch sequence of each batch the tuner times (tile shapes change binning too)
    std::vector<cudaEvent_t> tev;
    EventGuard tev_guard{&tev};
    if (any_tuning) {
        tev.resize(2 * nb);
        for (auto& e : tev) cuda_check(cudaEventCreate(&e), "event");
    }
    for (int attempt = 0; attempt < 12; ++attempt) {
        // scratch for the remaining batches
        uint32_t max_prims = 0, max_tiles = 0, max_stride = 0, max_strip = 0;
        for (size_t i = first_batch; i < nb; ++i) {
            max_strip = std::max(max_strip, batches[i].strip_entries);
            uint32_t stride = (uint32_t)((sizeof(TriRecord) + 3 * batches[i].nvar * sizeof(float) + 15) & ~size_t(15));
            max_stride = std::max(max_stride, stride);
            max_prims = std::max(max_prims, batches[i].total_prims);
            max_tiles = std::max(max_tiles, batches[i].total_tiles);
        }
        records_buf.ensure((size_t)std::max(1u, max_prims) * max_stride, &scratch_bytes);
        slow_buf.ensure((size_t)std::max(1u, max_prims) * sizeof(uint32_t), &scratch_bytes);
        hint_buf.ensure((size_t)std::max(1u, max_prims) * sizeof(uint32_t), &scratch_bytes);
        if (max_strip) strip_buf.ensure((size_t)max_strip * sizeof(uint32_t), &scratch_bytes);
        ovf_buf.ensure((size_t)ovf_capacity * max_stride, &scratch_bytes);
        tiles_buf.ensure((size_t)(max_tiles + 1) * 3 * sizeof(uint32_t) + 64, &scratch_bytes);
        bins_buf.ensure((size_t)bin_capacity * sizeof(uint32_t), &scratch_bytes);
        // visibility raster, split tiles: per-tile marker, heavy list, item table, the chunks' key
        // arrays (32 MiB of them at the largest tile of the batches)
        uint32_t vis_npix = 0;
        for (size_t i = first_batch; i < nb; ++i)
            if (kinds[i] == 3) vis_npix = std::max(vis_npix, (uint32_t)(btile[i] * btile[i]));
        uint32_t split_items = vis_npix ? std::max(64u, (uint32_t)((32u << 20) / (vis_npix * 8u))) : 0u;
        if (vis_npix && split_cap_override) split_items = split_cap_override;
        const uint32_t split_heavy = split_items / 2;  // a split tile has two chunks or more
        const size_t split_off_heavy = align((size_t)max_tiles * sizeof(uint32_t));
        const size_t split_off_items = align(split_off_heavy + (size_t)split_heavy * 16);
        const size_t split_off_keys = align(split_off_items + (size_t)split_items * sizeof(uint32_t));
        if (vis_npix)
            split_buf.ensure(split_off_keys + (size_t)split_items * vis_npix * sizeof(unsigned long long), &scratch_bytes);
        if (scratch_bytes.load() + resident->load() > budget)
            fail(GBR_ERR_OUT_OF_MEMORY, "resident resources and transient memory exceed the HBM budget");
        if (!run.started) {
            cuda_check(cudaEventRecord(run.ev->start, stream), "event");
            run.started = true;
        }
        // The launch sequence of the remaining batches; replayed from a CUDA graph when the
        // config asks for graphs and the same parameters were launched before.
        std::vector<BatchParams> params(nb);
        std::vector<cudaEvent_t>* revp = &rev;
        auto enqueue = [&]() {
            cuda_check(cudaMemsetAsync(meta, 0, 4, stream), "abort flag");
            for (size_t i = first_batch; i < nb; ++i) {
                const Batch& b = batches[i];
                BatchParams& bp = params[i];
                bp = BatchParams{};
                bp.draws = reinterpret_cast<const DrawDesc*>(meta + desc_off[i]);
                bp.targets =
                    reinterpret_cast<const TargetDesc*>(meta + desc_off[i] + b.draws.size() * sizeof(DrawDesc));
                bp.draw_base = reinterpret_cast<const uint32_t*>(meta + desc_off[i] + b.draws.size() * sizeof(DrawDesc) +
                                                                 b.targets.size() * sizeof(TargetDesc));
                bp.num_draws = (uint32_t)b.draws.size();
                bp.num_targets = (uint32_t)b.targets.size();
                bp.total_prims = b.total_prims;
                bp.total_tiles = b.total_tiles;
                bp.tile_size = btile[i];
                bp.tile_shift = ilog2(btile[i]);
                bp.record_stride = (uint32_t)((sizeof(TriRecord) + 3 * b.nvar * sizeof(float) + 15) & ~size_t(15));
                bp.num_varyings = b.nvar;
                bp.records = static_cast<uint8_t*>(records_buf.ptr);
                bp.slow_prims = static_cast<uint32_t*>(slow_buf.ptr);
                bp.tile_hint = static_cast<uint32_t*>(hint_buf.ptr);
            bp.strip_info = b.strip_entries ? static_cast<uint32_t*>(strip_buf.ptr) : nullptr;
                bp.ovf_records = static_cast<uint8_t*>(ovf_buf.ptr);
                bp.ovf_capacity = ovf_capacity;
                bp.bin_capacity = (uint32_t)std::min<uint64_t>(bin_capacity, 0xFFFFFFFFull);
                uint32_t* tiles = static_cast<uint32_t*>(tiles_buf.ptr);
                bp.tile_count = tiles;
                bp.tile_offset = tiles + (max_tiles + 1);
                bp.tile_cursor = tiles + 2 * (max_tiles + 1);
                bp.bins = static_cast<uint32_t*>(bins_buf.ptr);
                bp.work_counter = reinterpret_cast<uint32_t*>(meta + off_work) + i * 4;
                bp.status = reinterpret_cast<BatchStatus*>(meta + off_status) + i;
                bp.abort_flag = reinterpret_cast<uint32_t*>(meta);
                bp.raster_rule = cfg.raster_rule;
                bp.fvs_mask = b.jit ? 0u : fvs_mask(b);
                bp.shape_groups = reinterpret_cast<const uint32_t*>(meta + desc_off[i] + shape_table_at(b));
                std::memcpy(bp.sg_off, sg_offs[i].v, sizeof bp.sg_off);
                if (kinds[i] == 3) {
                    bp.states = meta + states_off[i];
                    bp.vis_compare = visibility_compare(b);
                    uint8_t* sb = static_cast<uint8_t*>(split_buf.ptr);
                    bp.split_tile = reinterpret_cast<uint32_t*>(sb);
                    bp.split_heavy = reinterpret_cast<uint32_t*>(sb + split_off_heavy);
                    bp.split_item = reinterpret_cast<uint32_t*>(sb + split_off_items);
                    bp.split_keys = reinterpret_cast<unsigned long long*>(sb + split_off_keys);
                    bp.split_cap_heavy = split_heavy;
                    bp.split_cap_items = split_items;
                    bp.split_chunk = split_chunk;
                }
                cudaEvent_t* ev = revp->empty() ? nullptr : &(*revp)[2 * i];
                if (b.copy) {
                    cuda_check(cudaMemsetAsync(bp.status, 0, sizeof(BatchStatus), stream), "status");
                    if (ev) cuda_check(cudaEventRecord(ev[0], stream), "event");
                    execute_copy(*b.copy, stream);
                    if (ev) cuda_check(cudaEventRecord(ev[1], stream), "event");
                    continue;
                }
                const bool timed = !tev.empty() && tuning[i] >= 0;
                if (timed) cuda_check(cudaEventRecord(tev[2 * i], stream), "event");
                if (b.lines)
                    cuda_check(b.jit ? launch_lines_jit(*b.jit, bp, num_sms, stream, &run.launches, ev)
                                     : launch_lines(bp, num_sms, stream, &run.launches, ev),
                               "launch");
                else if (b.jit)
                    cuda_check(launch_batch_jit(*b.jit, bp, num_sms, stream, &run.launches, ev, kinds[i]), "launch");
                else
                    cuda_check(launch_batch(bp, btile[i], bwarps[i], num_sms, stream, &run.launches, ev, kinds[i]),
                               "launch");
                if (timed) cuda_check(cudaEventRecord(tev[2 * i + 1], stream), "event");
            }
        };
        bool any_copy = false;  // a captured graph would keep a copy's addresses: no graphs then
        for (size_t i = from; i < nb; ++i) any_copy = any_copy || (bool)batches[i].copy;
        if (cfg.use_graphs && attempt == 0 && !any_tuning && !any_copy) {
            // key: every launch parameter of the sequence (descriptors are re-uploaded each time)
            std::string key;
            auto put = [&](const void* p, size_t len) { key.append(static_cast<const char*>(p), len); };
            put(&from, sizeof from);
            for (size_t i = from; i < nb; ++i) {
                put(&btile[i], sizeof(int));
                put(&bwarps[i], sizeof(int));
                put(&kinds[i], sizeof(int));
                put(&batches[i].total_prims, sizeof(uint32_t));
                put(&batches[i].total_tiles, sizeof(uint32_t));
                put(&batches[i].nvar, sizeof(uint32_t));
                const uint32_t fm = fvs_mask(batches[i]);
                put(&fm, sizeof fm);
                const void* jp = batches[i].jit.get();
                put(&jp, sizeof jp);
                const size_t nd = batches[i].draws.size(), nt = batches[i].targets.size();
                put(&nd, sizeof nd);
                put(&nt, sizeof nt);
                put(sg_offs[i].v, sizeof sg_offs[i].v);  // the setup launches' shape ranges
                put(&desc_off[i], sizeof desc_off[i]);
            }
            const void* ptrs[9] = {records_buf.ptr, ovf_buf.ptr, tiles_buf.ptr, bins_buf.ptr, meta_buf.ptr, slow_buf.ptr,
                                   strip_buf.ptr, hint_buf.ptr, split_buf.ptr};
            put(ptrs, sizeof ptrs);
            put(&ovf_capacity, sizeof ovf_capacity);
            put(&bin_capacity, sizeof bin_capacity);
            key.push_back(rev.empty() ? 0 : 1);
            GraphEntry& g = graphs[key];
            g.last_use = ++graph_clock;
            if (!g.exec) {
                if (!rev.empty() && g.events.empty()) {
                    g.events.resize(rev.size());
                    for (auto& e : g.events) cuda_check(cudaEventCreate(&e), "event");
                }
                revp = &g.events;
                cudaGraph_t graph = nullptr;
                cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
                try {
                    enqueue();
                } catch (...) {
                    cudaStreamEndCapture(stream, &graph);
                    if (graph) cudaGraphDestroy(graph);
                    throw;
                }
                cuda_check(cudaStreamEndCapture(stream, &graph), "end capture");
                cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
                cudaGraphDestroy(graph);
                cuda_check(ie, "cudaGraphInstantiate");
                // keep the 32 most recently used graphs
                while (graphs.size() > 32) {
                    auto victim = graphs.begin();
                    for (auto gi = graphs.begin(); gi != graphs.end(); ++gi)
                        if (gi->second.last_use < victim->second.last_use) victim = gi;
                    if (victim->second.exec) cudaGraphExecDestroy(victim->second.exec);
                    for (cudaEvent_t e : victim->second.events) cudaEventDestroy(e);
                    graphs.erase(victim);
                }
            } else {
                revp = &g.events;
                for (size_t i = first_batch; i < nb; ++i)
                    run.launches += batches[i].lines ? 2u : (batches[i].strip_entries ? 1u : 0u) +
                                    (batches[i].jit ? 2u + (batches[i].total_prims ? 3u : 0u) + (kinds[i] == 3 ? 1u : 0u)
                                                    : batch_kernel_launches(batches[i].total_prims, btile[i], bwarps[i],
                                                                            kinds[i], fvs_mask(batches[i])));
            }
            cuda_check(cudaGraphLaunch(graphs[key].exec, stream), "cudaGraphLaunch");
        } else {
            enqueue();
        }
        // readbacks queued before this launch: their copies issued while it runs (ahead of this
        // launch's own status readback, which waits for the launch)
        issue_reads();
        lookahead();  // a submission queued since this group started is planned while it runs
        cuda_check(cudaEventRecord(run.ev->end, stream), "event");
        cuda_check(cudaMemcpyAsync(st.data(), meta + off_status, nb * sizeof(BatchStatus), cudaMemcpyDeviceToHost,
                                   stream),
                   "status readback");
        if (n_targets)
            cuda_check(cudaMemcpyAsync(counters.data(), meta + off_counters,
                                       n_targets * kTargetCounters * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                       stream),
                       "counter readback");
        cuda_check(cudaStreamSynchronize(stream), "submission");
        // first failing batch
        size_t bad = nb;
        for (size_t i = first_batch; i < nb; ++i)
            if (st[i].error) {
                bad = i;
                break;
            }
        for (size_t i = first_batch; i < bad; ++i) {
            Batch& b = batches[i];
            b.target_frags.assign(counters.begin() + (ptrdiff_t)(counter_first[i] * kTargetCounters),
                                  counters.begin() + (ptrdiff_t)((counter_first[i] + b.targets.size()) * kTargetCounters));
            run.slow_prims += st[i].slow_count;
            run.split_chunks += st[i].split_items;
            if (!b.copy && !b.lines && (!run.tile_shape || b.total_prims > run.tile_shape_prims)) {
                run.tile_shape = (uint32_t)btile[i] << 8 | (uint32_t)bwarps[i];
                run.tile_shape_prims = b.total_prims;
            }
            if (!revp->empty()) {
                float ms = 0.0f;
                if (cudaEventElapsedTime(&ms, (*revp)[2 * i], (*revp)[2 * i + 1]) == cudaSuccess) run.raster_ms += ms;
            }
            if (!tev.empty() && tuning[i] >= 0 && !b.copy) {
                float ms = 0.0f;
                if (cudaEventElapsedTime(&ms, tev[2 * i], tev[2 * i + 1]) == cudaSuccess) tuner_record(b, tuning[i], ms);
            }
        }
        if (bad == nb) return RunResult{nb, 0, {}};
        const BatchStatus& s = st[bad];
        if (s.error == ERR_OVERFLOW_RECORDS) {
            ovf_capacity = std::max<uint32_t>(ovf_capacity * 2, s.ovf_used + 1024);
        } else if (s.error == ERR_OVERFLOW_BINS) {
            bin_capacity = std::max<uint64_t>(bin_capacity * 2, s.bin_entries + (s.bin_entries >> 2));
        } else {
            static const char* names[] = {"none", "clip position w=0 (primitive.rs:177 / raster.rs:146)",
                                          "index out of range of the index buffer",
                                          "vertex attribute read out of range of the vertex buffer",
                                          "index + base_vertex overflows u32 (index.rs:55-57)", "", "",
                                          "scanline coordinate does not fit u32 (scanline.rs:156-170)",
                                          "unsupported"};
            char msg[256];
            std::snprintf(msg, sizeof msg, "%s (primitive %u)", s.error < 9 ? names[s.error] : "device error",
                          s.error_detail);
            return RunResult{bad, s.error, msg};
        }
        // counters of the batches that re-run start from zero
        if (n_targets > counter_first[bad])
            cuda_check(cudaMemsetAsync(reinterpret_cast<unsigned long long*>(meta + off_counters) +
                                           counter_first[bad] * kTargetCounters,
                                       0, (n_targets - counter_first[bad]) * kTargetCounters * sizeof(unsigned long long),
                                       stream),
                       "counters");
        first_batch = bad;
        if (attempt == 11) fail(GBR_ERR_OUT_OF_MEMORY, "scratch growth did not converge");
    }
    return RunResult{nb, 0, {}};
}

// ---------------------------------------------------------------- command decoding
template <class T>
const T* payload(const gbr_cmd_header& h, const uint8_t* body) {
    if (h.payload_bytes < sizeof(T)) fail(GBR_ERR_INVALID_ARGUMENT, "command %u payload too short", h.opcode);
    return reinterpret_cast<const T*>(body);
}

// A texture region of a copy: mip level stored, origin + extent inside it.
void check_region(const Texture& t, uint32_t mip, uint32_t x, uint32_t y, uint32_t z, const gbr_extent3d& e) {
    if (mip >= t.mips_stored) fail(GBR_ERR_VALIDATION, "copy: mip level %u not stored", mip);
    if ((uint64_t)x + e.width > t.mip_w(mip) || (uint64_t)y + e.height > t.mip_h(mip) ||
        (uint64_t)z + e.depth_or_array_layers > t.layers())
        fail(GBR_ERR_VALIDATION, "copy: texture region out of range");
}

CopyCmd decode_copy(Device& dev, const gbr_cmd_header& h, const uint8_t* b) {
    static const char* const kNames[] = {"copy_buffer_to_buffer", "copy_buffer_to_texture", "copy_texture_to_buffer",
                                         "copy_texture_to_texture", "clear_buffer", "clear_texture"};
    static const char* const kLines[] = {"37-46", "48-55", "57-64", "66-73", "108-115", "100-106"};
    const uint32_t k = h.opcode - GBR_OP_COPY_BUFFER_TO_BUFFER;
    if (dev.cfg.profile != GBR_PROFILE_EXTENSION)
        fail(GBR_ERR_UNSUPPORTED, "%s is todo!() (command.rs:%s)", kNames[k], kLines[k]);
    CopyCmd c;
    c.op = h.opcode;
    switch (h.opcode) {
        case GBR_OP_COPY_BUFFER_TO_BUFFER: {
            auto* p = payload<gbr_cmd_copy_buffer_to_buffer>(h, b);
            c.buf = dev.get<Buffer>(p->source, "buffer");
            c.buf2 = dev.get<Buffer>(p->destination, "buffer");
            c.off = p->source_offset;
            c.off2 = p->destination_offset;
            c.size = p->size == UINT64_MAX ? c.buf->size - std::min(c.off, c.buf->size) : p->size;
            if (c.buf == c.buf2) fail(GBR_ERR_VALIDATION, "copy_buffer_to_buffer: source and destination are the same buffer");
            if (c.off % 4 || c.off2 % 4 || c.size % 4) fail(GBR_ERR_VALIDATION, "copy_buffer_to_buffer: alignment");
            if (!range_fits(c.off, c.size, c.buf->size) || !range_fits(c.off2, c.size, c.buf2->size))
                fail(GBR_ERR_VALIDATION, "copy_buffer_to_buffer: range out of bounds");
            break;
        }
        case GBR_OP_COPY_BUFFER_TO_TEXTURE:
        case GBR_OP_COPY_TEXTURE_TO_BUFFER: {
            auto* p = payload<gbr_cmd_copy_buffer_texture>(h, b);
            c.buf = dev.get<Buffer>(p->buffer, "buffer");
            c.tex = dev.get<Texture>(p->texture.texture, "texture");
            c.layout = p->layout;
            c.mip = p->texture.mip_level;
            c.ox = p->texture.origin_x;
            c.oy = p->texture.origin_y;
            c.oz = p->texture.origin_z;
            c.ext = p->size;
            check_region(*c.tex, c.mip, c.ox, c.oy, c.oz, c.ext);
            const uint64_t width = (uint64_t)c.ext.width * c.tex->bpp;
            const uint64_t bpr = c.layout.bytes_per_row ? c.layout.bytes_per_row : width;
            const uint64_t rpi = c.layout.rows_per_image ? c.layout.rows_per_image : c.ext.height;
            if ((c.ext.height > 1 || c.ext.depth_or_array_layers > 1) && (c.layout.bytes_per_row % 256 || !c.layout.bytes_per_row))
                fail(GBR_ERR_VALIDATION, "%s: bytes_per_row must be a multiple of 256", kNames[k]);
            if (bpr < width || rpi < c.ext.height) fail(GBR_ERR_VALIDATION, "%s: layout smaller than the copy", kNames[k]);
            if (c.layout.offset % c.tex->bpp) fail(GBR_ERR_VALIDATION, "%s: offset not a multiple of the texel size", kNames[k]);
            if (c.ext.width && c.ext.height && c.ext.depth_or_array_layers) {
                const uint64_t need = span_end(c.layout.offset, (uint64_t)(c.ext.depth_or_array_layers - 1) * rpi +
                                                                    (c.ext.height - 1), bpr, width);
                if (need > c.buf->size) fail(GBR_ERR_VALIDATION, "%s: buffer range out of bounds", kNames[k]);
            }
            break;
        }
        case GBR_OP_COPY_TEXTURE_TO_TEXTURE: {
            auto* p = payload<gbr_cmd_copy_texture_to_texture>(h, b);
            c.tex = dev.get<Texture>(p->source.texture, "texture");
            c.tex2 = dev.get<Texture>(p->destination.texture, "texture");
            c.mip = p->source.mip_level;
            c.ox = p->source.origin_x;
            c.oy = p->source.origin_y;
            c.oz = p->source.origin_z;
            c.mip2 = p->destination.mip_level;
            c.ox2 = p->destination.origin_x;
            c.oy2 = p->destination.origin_y;
            c.oz2 = p->destination.origin_z;
            c.ext = p->size;
            if (c.tex->desc.format != c.tex2->desc.format) fail(GBR_ERR_VALIDATION, "copy_texture_to_texture: formats differ");
            check_region(*c.tex, c.mip, c.ox, c.oy, c.oz, c.ext);
            check_region(*c.tex2, c.mip2, c.ox2, c.oy2, c.oz2, c.ext);
            if (c.tex == c.tex2 && c.mip == c.mip2 &&
                c.oz < c.oz2 + c.ext.depth_or_array_layers && c.oz2 < c.oz + c.ext.depth_or_array_layers)
                fail(GBR_ERR_VALIDATION, "copy_texture_to_texture: source and destination overlap");
            break;
        }
        case GBR_OP_CLEAR_BUFFER: {
            auto* p = payload<gbr_cmd_clear_buffer>(h, b);
            c.buf = dev.get<Buffer>(p->buffer, "buffer");
            c.off = p->offset;
            c.size = p->size == UINT64_MAX ? c.buf->size - std::min(c.off, c.buf->size) : p->size;
            if (c.off % 4 || c.size % 4) fail(GBR_ERR_VALIDATION, "clear_buffer: alignment");
            if (!range_fits(c.off, c.size, c.buf->size)) fail(GBR_ERR_VALIDATION, "clear_buffer: range out of bounds");
            break;
        }
        case GBR_OP_CLEAR_TEXTURE: {
            auto* p = payload<gbr_cmd_clear_texture>(h, b);
            c.tex = dev.get<Texture>(p->texture, "texture");
            c.mip = p->base_mip_level;
            c.oz = p->base_array_layer;
            if (c.mip >= c.tex->mips_stored || c.oz >= c.tex->layers())
                fail(GBR_ERR_VALIDATION, "clear_texture: subresource range out of range");
            c.mip_count = p->mip_level_count ? p->mip_level_count : c.tex->mips_stored - c.mip;
            c.layer_count = p->array_layer_count ? p->array_layer_count : c.tex->layers() - c.oz;
            if ((uint64_t)c.mip + c.mip_count > c.tex->mips_stored || (uint64_t)c.oz + c.layer_count > c.tex->layers())
                fail(GBR_ERR_VALIDATION, "clear_texture: subresource range out of range");
            break;
        }
    }
    return c;
}

std::vector<PassCmd> decode(Device& dev, const uint8_t* data, uint64_t len) {
    std::vector<PassCmd> passes;
    uint64_t off = 0;
    PassCmd* cur = nullptr;
    DrawCmd st;  // current render-pass state (state.rs:57-74)
    while (off < len) {
        if (len - off < sizeof(gbr_cmd_header)) fail(GBR_ERR_INVALID_ARGUMENT, "truncated command header");
        gbr_cmd_header h;
        std::memcpy(&h, data + off, sizeof h);
        off += sizeof h;
        uint64_t padded = (h.payload_bytes + 7ull) & ~7ull;
        if (len - off < padded) fail(GBR_ERR_INVALID_ARGUMENT, "truncated command payload");
        std::vector<uint8_t> tmp(data + off, data + off + h.payload_bytes);
        const uint8_t* b = tmp.data();
        off += padded;
        if (h.opcode == GBR_OP_BEGIN_RENDER_PASS) {
            if (cur) fail(GBR_ERR_INVALID_ARGUMENT, "nested render pass");
            passes.emplace_back();
            cur = &passes.back();
            std::memcpy(&cur->begin, payload<gbr_cmd_begin_render_pass>(h, b), sizeof cur->begin);
            // State::new (state.rs:77-133): all attachments must have the same size
            bool have = false;
            auto size_of = [&](const Texture& t) {
                if (!have) {
                    cur->width = t.desc.size.width;
                    cur->height = t.desc.size.height;
                    have = true;
                } else if (cur->width != t.desc.size.width || cur->height != t.desc.size.height) {
                    fail(GBR_ERR_VALIDATION, "All render attachments must be the same size");
                }
            };
            if (cur->begin.color_attachment_count > GBR_MAX_COLOR_TARGETS) fail(GBR_ERR_VALIDATION, "too many attachments");
            for (uint32_t a = 0; a < cur->begin.color_attachment_count; ++a) {
                uint64_t v = cur->begin.color_attachments[a].view;
                if (!v) continue;
                if (a > 0) fail(GBR_ERR_UNSUPPORTED, "more than one colour attachment");
                cur->color = dev.get<Texture>(v, "texture");
                size_of(*cur->color);
                if (cur->begin.color_attachments[a].depth_slice >= cur->color->layers())
                    fail(GBR_ERR_VALIDATION, "depth_slice out of range");
            }
            if (cur->begin.has_depth_attachment && cur->begin.depth_attachment.view) {
                cur->depth = dev.get<Texture>(cur->begin.depth_attachment.view, "texture");
                if (cur->depth->desc.format != GBR_TEXTURE_FORMAT_DEPTH32_FLOAT)
                    fail(GBR_ERR_UNSUPPORTED, "depth attachment format");
                size_of(*cur->depth);
            }
            st = DrawCmd();
            st.viewport[2] = (float)cur->width;
            st.viewport[3] = (float)cur->height;
            st.viewport[5] = 1.0f;
            st.scissor[2] = cur->width;
            st.scissor[3] = cur->height;
            continue;
        }
        if (h.opcode == GBR_OP_END_RENDER_PASS) {
            if (!cur) fail(GBR_ERR_INVALID_ARGUMENT, "end without begin");
            cur = nullptr;
            continue;
        }
        if (h.opcode >= GBR_OP_COPY_BUFFER_TO_BUFFER && h.opcode <= GBR_OP_CLEAR_TEXTURE) {
            if (cur) fail(GBR_ERR_INVALID_ARGUMENT, "command %u inside a render pass", h.opcode);
            passes.emplace_back();
            passes.back().copy = std::make_shared<CopyCmd>(decode_copy(dev, h, b));
            continue;
        }
        if (!cur) fail(GBR_ERR_INVALID_ARGUMENT, "command %u outside a render pass", h.opcode);
        switch (h.opcode) {
            case GBR_OP_SET_PIPELINE:
                st.pipeline = dev.get<Pipeline>(payload<gbr_cmd_set_pipeline>(h, b)->pipeline, "pipeline");
                break;
            case GBR_OP_SET_BIND_GROUP: {
                auto* p = payload<gbr_cmd_set_bind_group>(h, b);
                if (p->index >= GBR_MAX_BIND_GROUPS) fail(GBR_ERR_VALIDATION, "bind group index");
                st.groups[p->index] = p->bind_group ? dev.get<BindGroup>(p->bind_group, "bind group") : nullptr;
                break;
            }
            case GBR_OP_SET_INDEX_BUFFER: {
                auto* p = payload<gbr_cmd_set_index_buffer>(h, b);
                auto buf = dev.get<Buffer>(p->buffer, "buffer");
                uint64_t size = p->size ? p->size : buf->size - std::min(p->offset, buf->size);
                if (!range_fits(p->offset, size, buf->size)) fail(GBR_ERR_VALIDATION, "index buffer slice out of range");
                st.index = {buf, p->offset, size};
                st.index_format = p->index_format;
                break;
            }
            case GBR_OP_SET_VERTEX_BUFFER: {
                auto* p = payload<gbr_cmd_set_vertex_buffer>(h, b);
                if (p->slot >= GBR_MAX_VERTEX_BUFFERS) fail(GBR_ERR_VALIDATION, "vertex buffer slot");
                if (p->offset % 4) fail(GBR_ERR_VALIDATION, "vertex buffer offset must be a multiple of 4");
                auto buf = dev.get<Buffer>(p->buffer, "buffer");
                uint64_t size = p->size ? p->size : buf->size - std::min(p->offset, buf->size);
                if (!range_fits(p->offset, size, buf->size)) fail(GBR_ERR_VALIDATION, "vertex buffer slice out of range");
                st.vb[p->slot] = {buf, p->offset, size};
                break;
            }
            case GBR_OP_SET_VIEWPORT: {
                auto* p = payload<gbr_cmd_set_viewport>(h, b);
                st.viewport[0] = p->x;
                st.viewport[1] = p->y;
                st.viewport[2] = p->width;
                st.viewport[3] = p->height;
                st.viewport[4] = p->min_depth;
                st.viewport[5] = p->max_depth;
                break;
            }
            case GBR_OP_SET_SCISSOR_RECT: {
                auto* p = payload<gbr_cmd_set_scissor_rect>(h, b);
                if ((uint64_t)p->x + p->width > cur->width || (uint64_t)p->y + p->height > cur->height)
                    fail(GBR_ERR_VALIDATION, "scissor rect exceeds the render target");
                st.scissor[0] = p->x;
                st.scissor[1] = p->y;
                st.scissor[2] = p->width;
                st.scissor[3] = p->height;
                break;
            }
            case GBR_OP_SET_BLEND_CONSTANT: {
                auto* p = payload<gbr_cmd_set_blend_constant>(h, b);
                for (int k = 0; k < 4; ++k) st.blend_constant[k] = p->color[k];
                break;
            }
            case GBR_OP_SET_STENCIL_REFERENCE: break;
            case GBR_OP_DRAW:
            case GBR_OP_DRAW_INDEXED: {
                if (!st.pipeline) fail(GBR_ERR_VALIDATION, "No pipeline bound");
                DrawCmd dc = st;
                if (h.opcode == GBR_OP_DRAW) {
                    auto* p = payload<gbr_cmd_draw>(h, b);
                    dc.indexed = false;
                    dc.start = p->vertex_start;
                    dc.end = p->vertex_end;
                    dc.base_vertex = 0;
                    dc.inst_start = p->instance_start;
                    dc.inst_end = p->instance_end;
                } else {
                    auto* p = payload<gbr_cmd_draw_indexed>(h, b);
                    if (!st.index.buf) fail(GBR_ERR_VALIDATION, "No index buffer bound");
                    dc.indexed = true;
                    dc.start = p->index_start;
                    dc.end = p->index_end;
                    dc.base_vertex = p->base_vertex;
                    dc.inst_start = p->instance_start;
                    dc.inst_end = p->instance_end;
                }
                cur->draws.push_back(dc);
                break;
            }
            default: fail(GBR_ERR_INVALID_ARGUMENT, "unknown opcode %u", h.opcode);
        }
    }
    if (cur) fail(GBR_ERR_INVALID_ARGUMENT, "render pass not ended");
    return passes;
}

}  // namespace

// Sets the text that gbr_last_error() returns on this thread (used by entry points defined in
// other translation units).
void set_thread_error(const char* msg) { g_last_error = msg ? msg : ""; }

}  // namespace gbr

using namespace gbr;

#define GBR_TRY(...)                      \
    try {                                 \
        __VA_ARGS__;                      \
        return GBR_OK;                    \
    } catch (const Failure& f) {          \
        g_last_error = f.msg;             \
        return f.status;                  \
    } catch (const std::exception& e) {   \
        g_last_error = e.what();          \
        return GBR_ERR_OUT_OF_MEMORY;     \
    }

extern "C" {

GBR_API size_t gbr_last_error(char* buf, size_t len) {
    if (buf && len) {
        size_t n = std::min(len - 1, g_last_error.size());
        std::memcpy(buf, g_last_error.data(), n);
        buf[n] = 0;
    }
    return g_last_error.size();
}
GBR_API uint32_t gbr_abi_version(void) { return GBR_ABI_VERSION; }

GBR_API gbr_status gbr_device_create(const gbr_device_config* cfg, gbr_device* out) {
    GBR_TRY({
        if (!cfg || !out) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        if (cfg->abi_version != GBR_ABI_VERSION) fail(GBR_ERR_INVALID_ARGUMENT, "ABI version mismatch");
        auto d = std::make_shared<Device>();
        d->cfg = *cfg;
        d->ordinal = (int)cfg->device_ordinal;
        int n = 0;
        cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (d->ordinal >= n) fail(GBR_ERR_INVALID_ARGUMENT, "no CUDA device %d", d->ordinal);
        cuda_check(cudaSetDevice(d->ordinal), "cudaSetDevice");
        cuda_check(cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, d->ordinal), "attribute");
        d->tile = cfg->tile_size ? (int)cfg->tile_size : 16;
        d->warps = cfg->warps_per_tile ? (int)cfg->warps_per_tile : (d->tile == 8 ? 2 : 8);
        if (!raster_config_supported(d->tile, d->warps))
            fail(GBR_ERR_INVALID_ARGUMENT, "unsupported tile size / warps per tile %d/%d", d->tile, d->warps);
        if (cfg->bin_capacity) d->bin_capacity = cfg->bin_capacity;
        if (const char* e = std::getenv("GBR_VIS_SPLIT_ITEMS")) d->split_cap_override = (uint32_t)std::strtoul(e, nullptr, 10);
        if (const char* e = std::getenv("GBR_VIS_SPLIT_CHUNK"))
            d->split_chunk = std::max<uint32_t>(32u, (uint32_t)std::strtoul(e, nullptr, 10));
        d->autotune = cfg->tile_size == 0 && cfg->warps_per_tile == 0;
        if (cfg->launch_mode > GBR_LAUNCH_PER_PASS) fail(GBR_ERR_INVALID_ARGUMENT, "launch_mode");
        if (cfg->raster_order > GBR_RASTER_ORDERED) fail(GBR_ERR_INVALID_ARGUMENT, "raster_order");
        if (cfg->raster_rule > GBR_RASTER_RULE_EDGE) fail(GBR_ERR_INVALID_ARGUMENT, "raster_rule");
        if (cfg->raster_rule == GBR_RASTER_RULE_EDGE && cfg->profile != GBR_PROFILE_EXTENSION)
            fail(GBR_ERR_INVALID_ARGUMENT, "the edge-function raster rule belongs to the extension profile");
        cuda_check(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        cuda_check(cudaStreamCreateWithFlags(&d->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        cuda_check(cudaStreamCreateWithFlags(&d->rb_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        {
            cudaMemPoolProps props{};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = d->ordinal;
            cuda_check(cudaMemPoolCreate(&d->staging_pool, &props), "cudaMemPoolCreate");
            uint64_t keep = 1ull << 30;  // staging kept for reuse up to 1 GiB
            cuda_check(cudaMemPoolSetAttribute(d->staging_pool, cudaMemPoolAttrReleaseThreshold, &keep),
                       "cudaMemPoolSetAttribute");
        }
        Device* raw = d.get();
        d->worker = std::thread([raw] { raw->worker_main(); });
        std::lock_guard<std::mutex> lk(g_dev_mu);
        uint64_t h = g_next_device++;
        g_devices[h] = d;
        *out = h;
    })
}

GBR_API gbr_status gbr_device_destroy(gbr_device dh) {
    GBR_TRY({
        std::shared_ptr<Device> d;
        {
            std::lock_guard<std::mutex> lk(g_dev_mu);
            auto it = g_devices.find(dh);
            if (it == g_devices.end()) fail(GBR_ERR_INVALID_ARGUMENT, "invalid device handle");
            d = it->second;
            g_devices.erase(it);
        }
        {
            std::lock_guard<std::mutex> lk(d->q_mu);
            d->stopping = true;
            d->q_cv.notify_all();
        }
        if (d->worker.joinable()) d->worker.join();
        cudaSetDevice(d->ordinal);
        cudaStreamSynchronize(d->stream);
        d->records.clear();  // their events go with them
        for (auto& g : d->graphs) {
            if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
            for (cudaEvent_t e : g.second.events) cudaEventDestroy(e);
        }
        d->graphs.clear();
        d->objects.clear();
        d->records_buf.release();
        d->slow_buf.release();
        d->hint_buf.release();
        d->split_buf.release();
        d->strip_buf.release();
        d->ovf_buf.release();
        d->tiles_buf.release();
        d->bins_buf.release();
        d->meta_buf.release();
        d->flush_buf.release();
        cudaStreamSynchronize(d->stream);
        d->upload_buf.release();
        for (auto* stages : {d->pinned_stage, d->meta_stage})
            for (int k = 0; k < 2; ++k) {
                auto& ps = stages[k];
                if (ps.ptr) cudaFreeHost(ps.ptr);
                if (ps.done) cudaEventDestroy(ps.done);
                ps.ptr = nullptr;
                ps.done = nullptr;
            }
        cudaStreamSynchronize(d->rb_stream);
        d->read_fence.clear();
        d->pending_reads.clear();
        for (auto& dr : d->deferred_reads) cudaEventDestroy(dr.ready);
        d->deferred_reads.clear();
        cudaStreamDestroy(d->stream);
        cudaStreamDestroy(d->copy_stream);
        cudaStreamDestroy(d->rb_stream);
        if (d->staging_pool) cudaMemPoolDestroy(d->staging_pool);
    })
}

GBR_API gbr_status gbr_device_limits(gbr_device dh, gbr_limits* out) {
    GBR_TRY({
        get_device(dh);
        out->max_texture_dimension_2d = 16384;
        out->max_bind_groups = GBR_MAX_BIND_GROUPS;
        out->max_vertex_buffers = GBR_MAX_VERTEX_BUFFERS;
        out->max_vertex_attributes = GBR_MAX_VERTEX_ATTRIBUTES;
        out->max_color_attachments = 1;
        out->max_inter_stage_components = MAX_VARYING_FLOATS;
        out->max_buffer_size = 1ull << 36;
    })
}

GBR_API gbr_status gbr_buffer_create(gbr_device dh, uint64_t size, uint32_t usage, gbr_buffer* out) {
    GBR_TRY({
        (void)usage;
        auto d = get_device(dh);
        cuda_check(cudaSetDevice(d->ordinal), "cudaSetDevice");
        auto b = std::make_shared<Buffer>();
        b->size = size;
        cuda_check(cudaMalloc(&b->ptr, std::max<uint64_t>(size, 16)), "cudaMalloc(buffer)");
        b->allocated = std::max<uint64_t>(size, 16);
        b->resident = d->resident;
        d->resident->fetch_add(b->allocated);
        cuda_check(cudaMemset(b->ptr, 0, std::max<uint64_t>(size, 16)), "cudaMemset(buffer)");
        *out = d->add(b);
    })
}
GBR_API gbr_status gbr_buffer_destroy(gbr_device dh, gbr_buffer b) {
    GBR_TRY({
        auto d = get_device(dh);
        d->get<Buffer>(b, "buffer");
        d->remove(b);
    })
}
// The caller's bytes on the device, copied now (the queue applies them later, in order); null
// for small writes (a host copy costs less than a synchronised transfer) or when the staging
// pool has no room, and the item then keeps a host copy instead.
constexpr uint64_t kStageMinBytes = 256u << 10;
void* stage_on_device(Device* d, const void* src, uint64_t n) {
    if (n < kStageMinBytes) return nullptr;
    std::lock_guard<std::mutex> lk(d->copy_mu);
    void* p = nullptr;
    if (cudaMallocFromPoolAsync(&p, n, d->staging_pool, d->copy_stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    cuda_check(cudaMemcpyAsync(p, src, n, cudaMemcpyHostToDevice, d->copy_stream), "write staging");
    cuda_check(cudaStreamSynchronize(d->copy_stream), "write staging sync");
    return p;
}

GBR_API gbr_status gbr_queue_write_buffer(gbr_device dh, gbr_buffer b, uint64_t offset, const void* data, uint64_t size) {
    GBR_TRY({
        auto d = get_device(dh);
        Item it;
        it.kind = Item::WRITE_BUFFER;
        it.buffer = d->get<Buffer>(b, "buffer");
        if (!range_fits(offset, size, it.buffer->size)) fail(GBR_ERR_VALIDATION, "write_buffer out of range");
        if (!size) return GBR_OK;
        it.offset = offset;
        it.staged = stage_on_device(d.get(), data, size);
        it.staged_size = size;
        if (!it.staged) it.data.assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + size);
        d->enqueue(std::move(it));
    })
}
GBR_API gbr_status gbr_queue_write_buffers(gbr_device dh, uint32_t count, const gbr_buffer_write* writes) {
    GBR_TRY({
        auto d = get_device(dh);
        if (count && !writes) fail(GBR_ERR_INVALID_ARGUMENT, "null write array");
        std::vector<Item> items;
        items.reserve(count);
        for (uint32_t k = 0; k < count; ++k) {  // validate everything before queuing anything
            const gbr_buffer_write& w = writes[k];
            Item it;
            it.kind = Item::WRITE_BUFFER;
            it.buffer = d->get<Buffer>(w.buffer, "buffer");
            if (!range_fits(w.offset, w.size, it.buffer->size)) fail(GBR_ERR_VALIDATION, "write_buffer out of range (entry %u)", k);
            if (w.size && !w.data) fail(GBR_ERR_INVALID_ARGUMENT, "null data (entry %u)", k);
            it.offset = w.offset;
            it.staged_size = w.size;
            if (w.size) items.push_back(std::move(it));
        }
        size_t j = 0;
        for (uint32_t k = 0; k < count; ++k) {
            const gbr_buffer_write& w = writes[k];
            if (!w.size) continue;
            Item& it = items[j++];
            it.staged = stage_on_device(d.get(), w.data, w.size);
            if (!it.staged) it.data.assign(static_cast<const uint8_t*>(w.data), static_cast<const uint8_t*>(w.data) + w.size);
        }
        d->enqueue_all(items);
    })
}
GBR_API gbr_status gbr_buffer_read(gbr_device dh, gbr_buffer b, uint64_t offset, void* dst, uint64_t size) {
    GBR_TRY({
        auto d = get_device(dh);
        Item it;
        it.kind = Item::READ_BUFFER;
        it.buffer = d->get<Buffer>(b, "buffer");
        if (!range_fits(offset, size, it.buffer->size)) fail(GBR_ERR_VALIDATION, "buffer read out of range");
        it.offset = offset;
        it.dst = dst;
        it.size = size;
        std::promise<Failure> done;
        auto fut = done.get_future();
        it.done = &done;
        d->enqueue(std::move(it));
        Failure f = fut.get();
        if (f.status != GBR_OK) throw f;
    })
}

GBR_API gbr_status gbr_texture_create(gbr_device dh, const gbr_texture_desc* desc, gbr_texture* out) {
    GBR_TRY({
        auto d = get_device(dh);
        if (!desc) fail(GBR_ERR_INVALID_ARGUMENT, "null descriptor");
        uint32_t bpp = bytes_per_texel(desc->format);
        if (!bpp) fail(GBR_ERR_UNSUPPORTED, "Unsupported texture format: %u", desc->format);
        if (!desc->size.width || !desc->size.height) fail(GBR_ERR_VALIDATION, "zero-sized texture");
        cuda_check(cudaSetDevice(d->ordinal), "cudaSetDevice");
        auto t = std::make_shared<Texture>();
        t->desc = *desc;
        t->bpp = bpp;
        uint32_t mips = desc->mip_level_count ? desc->mip_level_count : 1;
        // the reference stores mip 0 only (texture.rs:34-43); the extension profile keeps the chain
        t->mips_stored = d->cfg.profile == GBR_PROFILE_EXTENSION ? std::min(mips, 16u) : 1;
        uint64_t off = 0;
        for (uint32_t m = 0; m < t->mips_stored; ++m) {
            t->mip_offset[m] = off;
            off += (t->mip_bytes(m) + 255) & ~uint64_t(255);
        }
        t->bytes = off;
        cuda_check(cudaMalloc(&t->ptr, off), "cudaMalloc(texture)");
        t->resident = d->resident;
        d->resident->fetch_add(off);
        cuda_check(cudaMemset(t->ptr, 0, off), "cudaMemset(texture)");
        *out = d->add(t);
    })
}
GBR_API gbr_status gbr_texture_destroy(gbr_device dh, gbr_texture t) {
    GBR_TRY({
        auto d = get_device(dh);
        d->get<Texture>(t, "texture");
        d->remove(t);
    })
}
GBR_API gbr_status gbr_queue_write_texture(gbr_device dh, gbr_texture th, uint32_t mip, const void* data,
                                           uint64_t data_size, const gbr_texel_copy_buffer_layout* layout,
                                           gbr_extent3d size) {
    GBR_TRY({
        (void)size;  // the reference copies the whole texture (the extent is shadowed, device.rs:388)
        auto d = get_device(dh);
        Item it;
        it.kind = Item::WRITE_TEXTURE;
        it.texture = d->get<Texture>(th, "texture");
        const Texture& t = *it.texture;
        if (mip >= t.mips_stored) fail(GBR_ERR_UNSUPPORTED, "write_texture to mip_level %u (device.rs:378-380)", mip);
        it.mip = mip;
        it.layout = *layout;
        uint64_t row = (uint64_t)t.mip_w(mip) * t.bpp;
        uint64_t src_row = layout->bytes_per_row ? layout->bytes_per_row : data_size;
        uint64_t rows_per_image = layout->rows_per_image ? layout->rows_per_image : t.mip_h(mip);
        if (src_row < row) fail(GBR_ERR_VALIDATION, "bytes_per_row smaller than a texel row");
        uint64_t need = span_end(layout->offset, span_end(0, (uint64_t)(t.layers() - 1), rows_per_image, t.mip_h(mip) - 1),
                                 src_row, row);
        if (need > data_size) fail(GBR_ERR_VALIDATION, "write_texture source out of range");
        it.staged = stage_on_device(d.get(), data, data_size);
        it.staged_size = data_size;
        if (!it.staged)
            it.data.assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + data_size);
        d->enqueue(std::move(it));
    })
}
GBR_API gbr_status gbr_texture_read(gbr_device dh, gbr_texture th, uint32_t mip, void* dst, uint64_t size) {
    GBR_TRY({
        auto d = get_device(dh);
        Item it;
        it.kind = Item::READ_TEXTURE;
        it.texture = d->get<Texture>(th, "texture");
        if (mip >= it.texture->mips_stored) fail(GBR_ERR_VALIDATION, "mip level not stored");
        if (size < it.texture->mip_bytes(mip)) fail(GBR_ERR_VALIDATION, "destination too small");
        it.mip = mip;
        it.dst = dst;
        std::promise<Failure> done;
        auto fut = done.get_future();
        it.done = &done;
        d->enqueue(std::move(it));
        Failure f = fut.get();
        if (f.status != GBR_OK) throw f;
    })
}
GBR_API gbr_status gbr_textures_read(gbr_device dh, uint32_t count, const gbr_texture* textures, const uint32_t* mips,
                                     void* const* dsts, const uint64_t* sizes) {
    GBR_TRY({
        auto d = get_device(dh);
        if (count && (!textures || !mips || !dsts || !sizes)) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        Item it;
        it.kind = Item::READ_TEXTURES;
        for (uint32_t k = 0; k < count; ++k) {
            auto t = d->get<Texture>(textures[k], "texture");
            if (mips[k] >= t->mips_stored) fail(GBR_ERR_VALIDATION, "mip level not stored");
            if (sizes[k] < t->mip_bytes(mips[k])) fail(GBR_ERR_VALIDATION, "destination too small");
            if (!dsts[k]) fail(GBR_ERR_INVALID_ARGUMENT, "null destination");
            it.textures.push_back(std::move(t));
            it.mips.push_back(mips[k]);
            it.dsts.push_back(dsts[k]);
        }
        if (!count) return GBR_OK;
        std::promise<Failure> done;
        auto fut = done.get_future();
        it.done = &done;
        d->enqueue(std::move(it));
        Failure f = fut.get();
        if (f.status != GBR_OK) throw f;
    })
}

GBR_API gbr_status gbr_queue_read_textures(gbr_device dh, uint32_t count, const gbr_texture* textures,
                                           const uint32_t* mips, void* const* dsts, const uint64_t* sizes,
                                           uint64_t* out_index) {
    GBR_TRY({
        auto d = get_device(dh);
        if (count && (!textures || !mips || !dsts || !sizes)) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        Item it;
        it.kind = Item::READ_TEXTURES;
        it.t_submit = Clock::now();
        for (uint32_t k = 0; k < count; ++k) {
            auto t = d->get<Texture>(textures[k], "texture");
            if (mips[k] >= t->mips_stored) fail(GBR_ERR_VALIDATION, "mip level not stored");
            if (sizes[k] < t->mip_bytes(mips[k])) fail(GBR_ERR_VALIDATION, "destination too small");
            if (!dsts[k]) fail(GBR_ERR_INVALID_ARGUMENT, "null destination");
            it.textures.push_back(std::move(t));
            it.mips.push_back(mips[k]);
            it.dsts.push_back(dsts[k]);
        }
        it.indexed = true;
        {
            std::lock_guard<std::mutex> lk(d->q_mu);
            if (d->lost) fail(GBR_ERR_DEVICE_LOST, "device lost: %s", d->lost_msg.c_str());
            it.index = d->next_submission++;
            if (out_index) *out_index = it.index;
            d->queue.push_back(std::move(it));
            d->q_cv.notify_all();
        }
    })
}

GBR_API gbr_status gbr_sampler_create(gbr_device dh, const gbr_sampler_desc* desc, gbr_sampler* out) {
    GBR_TRY({
        auto d = get_device(dh);
        auto s = std::make_shared<Sampler>();
        s->desc = *desc;
        *out = d->add(s);
    })
}
GBR_API gbr_status gbr_sampler_destroy(gbr_device dh, gbr_sampler s) {
    GBR_TRY({
        auto d = get_device(dh);
        d->get<Sampler>(s, "sampler");
        d->remove(s);
    })
}

GBR_API gbr_status gbr_shader_module_create_native(gbr_device dh, const char* name, gbr_shader_module* out) {
    GBR_TRY({
        auto d = get_device(dh);
        const ProgramInfo* p = name ? find_program(name) : nullptr;
        if (!p) fail(GBR_ERR_SHADER, "unknown native program '%s'", name ? name : "(null)");
        auto m = std::make_shared<ShaderModule>();
        m->prog = p;
        *out = d->add(m);
    })
}
GBR_API gbr_status gbr_shader_module_create(gbr_device dh, const char* wgsl, uint64_t len, gbr_shader_module* out) {
    GBR_TRY({
        auto d = get_device(dh);
        if (!wgsl || !out) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        auto m = std::make_shared<ShaderModule>();
        m->wgsl = parse_wgsl(wgsl, len);
        if (wgsl::entry_points(*m->wgsl).empty()) fail(GBR_ERR_SHADER, "the module has no entry point");
        *out = d->add(m);
    })
}

GBR_API gbr_status gbr_wgsl_translate(const char* wgsl, uint64_t len, const char* vertex_entry, const char* fragment_entry,
                                      char* out, uint64_t capacity, uint64_t* needed) {
    GBR_TRY({
        if (!wgsl) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        auto m = parse_wgsl(wgsl, len);
        const wgsl::ProgramCode pc = emit_wgsl(*m, vertex_entry ? vertex_entry : "", fragment_entry ? m.get() : nullptr,
                                               fragment_entry ? fragment_entry : "");
        if (needed) *needed = pc.cuda.size() + 1;
        if (out && capacity) {
            const size_t k = std::min<size_t>(capacity - 1, pc.cuda.size());
            std::memcpy(out, pc.cuda.data(), k);
            out[k] = 0;
        }
    })
}

GBR_API gbr_status gbr_wgsl_compile_check(const char* wgsl, uint64_t len, const char* vertex_entry,
                                          const char* fragment_entry, char* log, uint64_t capacity) {
    GBR_TRY({
        if (!wgsl) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        auto m = parse_wgsl(wgsl, len);
        const wgsl::ProgramCode pc = emit_wgsl(*m, vertex_entry ? vertex_entry : "", fragment_entry ? m.get() : nullptr,
                                               fragment_entry ? fragment_entry : "");
        std::vector<char> cubin;
        std::vector<std::string> names;
        std::string lg;
        const bool ok = jit_compile_cubin(pc.cuda, false, &cubin, &names, &lg);
        if (log && capacity) {
            const size_t k = std::min<size_t>(capacity - 1, lg.size());
            std::memcpy(log, lg.data(), k);
            log[k] = 0;
        }
        if (!ok) fail(GBR_ERR_SHADER, "NVRTC: %s", lg.substr(0, 400).c_str());
    })
}
GBR_API gbr_status gbr_shader_module_destroy(gbr_device dh, gbr_shader_module m) {
    GBR_TRY({
        auto d = get_device(dh);
        d->get<ShaderModule>(m, "shader module");
        d->remove(m);
    })
}

GBR_API gbr_status gbr_render_pipeline_create(gbr_device dh, const gbr_render_pipeline_desc* desc,
                                              gbr_render_pipeline* out) {
    GBR_TRY({
        auto d = get_device(dh);
        if (!desc) fail(GBR_ERR_INVALID_ARGUMENT, "null descriptor");
        auto pl = std::make_shared<Pipeline>();
        pl->desc = *desc;
        pl->desc.vertex_constants = pl->desc.fragment_constants = nullptr;  // the caller's, read below only
        pl->desc.vertex_constant_count = pl->desc.fragment_constant_count = 0;
        auto vs = d->get<ShaderModule>(desc->vertex_module, "shader module");
        pl->prog = vs->prog;
        if (vs->wgsl) {
            // WGSL: emit the vertex (+ fragment) program and compile it with the kernels
            std::shared_ptr<ShaderModule> fs;
            if (desc->has_fragment) {
                fs = d->get<ShaderModule>(desc->fragment_module, "shader module");
                if (!fs->wgsl) fail(GBR_ERR_UNSUPPORTED, "a WGSL vertex stage needs a WGSL fragment stage");
            }
            auto entry = [](const char* name, const wgsl::Module& m, int stage) {
                std::string e(name, strnlen(name, GBR_MAX_ENTRY_POINT_NAME));
                if (!e.empty()) return e;
                std::string only;
                int count = 0;
                for (const auto& ep : wgsl::entry_points(m))
                    if (ep.second == stage) {
                        only = ep.first;
                        ++count;
                    }
                if (count != 1) fail(GBR_ERR_VALIDATION, "an entry point name is required (%d candidates)", count);
                return only;
            };
            // PipelineCompilationOptions::constants of each stage (shader.rs:52-74)
            auto constants = [](const gbr_pipeline_constant* c, uint32_t n) {
                wgsl::Constants m;
                if (n && !c) fail(GBR_ERR_INVALID_ARGUMENT, "null pipeline constants");
                for (uint32_t i = 0; i < n; ++i) {
                    if (!c[i].key) fail(GBR_ERR_INVALID_ARGUMENT, "pipeline constant %u has no key", i);
                    m[c[i].key] = c[i].value;
                }
                return m;
            };
            const wgsl::Constants vconsts = constants(desc->vertex_constants, desc->vertex_constant_count);
            const wgsl::Constants fconsts = constants(desc->fragment_constants, desc->fragment_constant_count);
            const wgsl::ProgramCode pc =
                emit_wgsl(*vs->wgsl, entry(desc->vertex_entry_point, *vs->wgsl, 0), fs ? fs->wgsl.get() : nullptr,
                          fs ? entry(desc->fragment_entry_point, *fs->wgsl, 1) : std::string(), vconsts, fconsts);
            ProgramInfo& pi = pl->own;
            pi.name = "wgsl";
            pi.id = PROG_JIT;
            pi.jit = true;
            pi.num_inputs = pc.num_inputs;
            for (int i = 0; i < pc.num_inputs; ++i) {
                pi.input_loc[i] = pc.input_loc[i];
                pi.input_comps[i] = pc.input_comps[i];
                pi.input_kind[i] = pc.input_kind[i];
            }
            pi.num_varyings = pc.num_varyings;
            pi.perspective = pc.perspective;
            pi.uniform_min = 0;
            std::memcpy(pi.uniform_req, pc.uniform_size, sizeof pi.uniform_req);
            pi.uses_texture = pc.tex_group >= 0;
            if (pi.uses_texture) {
                pi.tex_group = pc.tex_group;
                pi.tex_binding = pc.tex_binding;
                pi.samp_group = pc.samp_group;
                pi.samp_binding = pc.samp_binding;
            }
            pi.may_discard = pc.may_discard;
            pi.flat_mask = pc.flat_mask;
            pi.early_depth = pc.early_depth;
            std::string err;
            pl->jit = jit_module(pc.cuda, d->cfg.raster_rule == GBR_RASTER_RULE_EDGE, &err);
            if (!pl->jit) fail(GBR_ERR_SHADER, "%s", err.c_str());
            pl->prog = &pl->own;
        } else if (desc->has_fragment) {
            auto fs = d->get<ShaderModule>(desc->fragment_module, "shader module");
            if (fs->prog != vs->prog)
                fail(GBR_ERR_UNSUPPORTED, "native programs pair their own vertex and fragment stages");
        }
        if (desc->vertex_buffer_count > GBR_MAX_VERTEX_BUFFERS) fail(GBR_ERR_VALIDATION, "too many vertex buffers");
        for (auto& a : pl->attr) a = AttrDesc{-1, 0, 0, 0};
        // VertexState::new (vertex.rs:50-94): location -> (buffer, offset, format); duplicates panic
        for (uint32_t b = 0; b < desc->vertex_buffer_count; ++b) {
            const gbr_vertex_buffer_layout& L = desc->vertex_buffers[b];
            if (L.array_stride % 4) fail(GBR_ERR_VALIDATION, "array_stride must be a multiple of 4");
            for (uint32_t a = 0; a < L.attribute_count && a < GBR_MAX_VERTEX_ATTRIBUTES; ++a) {
                const gbr_vertex_attribute& at = L.attributes[a];
                if (at.shader_location >= 16) fail(GBR_ERR_VALIDATION, "shader location out of range");
                if (pl->attr[at.shader_location].buffer >= 0)
                    fail(GBR_ERR_VALIDATION, "Duplicate vertex attribute at location %u", at.shader_location);
                uint32_t align = at.format == GBR_VERTEX_FORMAT_UNORM8X4 ? 1u
                                 : (at.format == GBR_VERTEX_FORMAT_FLOAT16X2 || at.format == GBR_VERTEX_FORMAT_FLOAT16X4) ? 2u
                                                                                                                       : 4u;
                if (at.offset % align) fail(GBR_ERR_VALIDATION, "attribute offset must be a multiple of %u", align);
                pl->attr[at.shader_location] = AttrDesc{(int32_t)b, at.format, (uint32_t)at.offset, 0};
            }
        }
        const ProgramInfo& p = *pl->prog;
        for (int i = 0; i < p.num_inputs; ++i) {
            const AttrDesc& a = pl->attr[p.input_loc[i]];
            if (a.buffer < 0) fail(GBR_ERR_VALIDATION, "No vertex attribute at location %d", p.input_loc[i]);
            uint32_t fsz = vertex_format_bytes(a.format);
            bool ext_conv = d->cfg.profile == GBR_PROFILE_EXTENSION && p.input_comps[i] == 4 &&
                            (a.format == GBR_VERTEX_FORMAT_FLOAT16X4 || a.format == GBR_VERTEX_FORMAT_UNORM8X4);
            if (!ext_conv && fsz != (uint32_t)p.input_comps[i] * 4u)
                fail(GBR_ERR_VALIDATION, "vertex format size %u does not match the shader input (vertex.rs:150-154)", fsz);
        }
        if (desc->has_depth_stencil && desc->depth_stencil.format != GBR_TEXTURE_FORMAT_DEPTH32_FLOAT)
            fail(GBR_ERR_UNSUPPORTED, "depth format");
        *out = d->add(pl);
    })
}
GBR_API gbr_status gbr_render_pipeline_eval_vertices(gbr_device dh, gbr_render_pipeline ph, uint32_t first_vertex,
                                                     uint32_t count, float* out, uint32_t* errors) {
    GBR_TRY({
        auto d = get_device(dh);
        auto pl = d->get<Pipeline>(ph, "pipeline");
        if (!pl->jit) fail(GBR_ERR_UNSUPPORTED, "only WGSL pipelines can be evaluated");
        if (!out || !errors || !count) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        // evaluated without bindings: a program that reads a uniform buffer cannot run here
        for (int g = 0; g < 4; ++g)
            for (int b = 0; b < 8; ++b)
                if (pl->prog->uniform_req[g][b]) fail(GBR_ERR_UNSUPPORTED, "the vertex stage reads uniform buffers");
        cudaSetDevice(d->ordinal);
        DrawDesc dd{};
        dd.program = PROG_JIT;
        for (int l = 0; l < 16; ++l) dd.attr[l] = AttrDesc{-1, 0, 0, 0};
        dd.num_varyings = pl->prog->num_varyings;
        dd.profile = d->cfg.profile;
        dd.instance_count = 1;
        const size_t per = 4 + MAX_VARYING_FLOATS;
        void *p_d = nullptr, *p_out = nullptr, *p_err = nullptr;
        cudaStream_t s = nullptr;
        auto cleanup = [&] {
            if (s) cudaStreamDestroy(s);
            cudaFree(p_d);
            cudaFree(p_out);
            cudaFree(p_err);
        };
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMalloc(&p_d, sizeof dd);
        if (e == cudaSuccess) e = cudaMalloc(&p_out, (size_t)count * per * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&p_err, (size_t)count * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemcpyAsync(p_d, &dd, sizeof dd, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = jit_eval_vertices(*pl->jit, static_cast<const DrawDesc*>(p_d), first_vertex, count,
                                  static_cast<float*>(p_out), static_cast<uint32_t*>(p_err), s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(out, p_out, (size_t)count * per * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(errors, p_err, (size_t)count * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cleanup();
        cuda_check(e, "eval vertices");
    })
}

GBR_API gbr_status gbr_render_pipeline_destroy(gbr_device dh, gbr_render_pipeline p) {
    GBR_TRY({
        auto d = get_device(dh);
        d->get<Pipeline>(p, "pipeline");
        d->remove(p);
    })
}

GBR_API gbr_status gbr_bind_group_create(gbr_device dh, const gbr_bind_group_desc* desc, gbr_bind_group* out) {
    GBR_TRY({
        auto d = get_device(dh);
        if (!desc || desc->entry_count > GBR_MAX_BIND_GROUP_ENTRIES) fail(GBR_ERR_INVALID_ARGUMENT, "bad descriptor");
        auto g = std::make_shared<BindGroup>();
        g->desc = *desc;
        for (uint32_t e = 0; e < desc->entry_count; ++e) {
            const gbr_bind_group_entry& en = desc->entries[e];
            if (en.kind == GBR_BINDING_BUFFER) {
                auto b = d->get<Buffer>(en.resource, "buffer");
                if (en.offset > b->size || (en.size && !range_fits(en.offset, en.size, b->size)))
                    fail(GBR_ERR_VALIDATION, "bind group buffer range out of bounds");
                if (en.offset % 16) fail(GBR_ERR_VALIDATION, "uniform binding offset must be a multiple of 16");
                g->refs.push_back(b);
            } else if (en.kind == GBR_BINDING_SAMPLER) {
                g->refs.push_back(d->get<Sampler>(en.resource, "sampler"));
            } else if (en.kind == GBR_BINDING_TEXTURE_VIEW) {
                g->refs.push_back(d->get<Texture>(en.resource, "texture"));
            } else {
                fail(GBR_ERR_INVALID_ARGUMENT, "binding kind");
            }
        }
        *out = d->add(g);
    })
}
GBR_API gbr_status gbr_bind_group_destroy(gbr_device dh, gbr_bind_group g) {
    GBR_TRY({
        auto d = get_device(dh);
        d->get<BindGroup>(g, "bind group");
        d->remove(g);
    })
}

GBR_API gbr_status gbr_queue_submit(gbr_device dh, const void* cmds, uint64_t len, uint64_t* out_index) {
    GBR_TRY({
        auto d = get_device(dh);
        Item it;
        it.kind = Item::SUBMIT;
        it.t_submit = Clock::now();
        it.passes = decode(*d, static_cast<const uint8_t*>(cmds), cmds ? len : 0);
        {
            std::lock_guard<std::mutex> lk(d->q_mu);
            if (d->lost) fail(GBR_ERR_DEVICE_LOST, "device lost: %s", d->lost_msg.c_str());
            it.index = d->next_submission++;
            if (out_index) *out_index = it.index;
            d->queue.push_back(std::move(it));
            d->q_cv.notify_all();
        }
    })
}

GBR_API gbr_status gbr_device_poll(gbr_device dh, uint32_t wait, uint32_t has_index, uint64_t index,
                                   uint64_t timeout_ns, uint32_t* out_status) {
    GBR_TRY({
        {  // queued writes run now (they do not wake the worker themselves)
            auto dq = get_device(dh);
            std::lock_guard<std::mutex> lk(dq->q_mu);
            if (!dq->queue.empty()) dq->q_cv.notify_all();
        }
        auto d = get_device(dh);
        std::unique_lock<std::mutex> lk(d->q_mu);
        if (!wait) {
            if (out_status) *out_status = GBR_POLL_POLL;
            return GBR_OK;
        }
        auto deadline = timeout_ns == UINT64_MAX ? Clock::time_point::max()
                                                 : Clock::now() + std::chrono::nanoseconds(timeout_ns);
        if (has_index && index >= d->next_submission) fail(GBR_ERR_INVALID_ARGUMENT, "unknown submission index");
        const bool empty = d->completed_submissions == d->next_submission;
        uint64_t target = has_index ? index + 1 : d->completed_submissions + 1;
        while (!empty && d->completed_submissions < target) {
            if (deadline == Clock::time_point::max()) {
                d->done_cv.wait(lk);
            } else if (d->done_cv.wait_until(lk, deadline) == std::cv_status::timeout &&
                       d->completed_submissions < target) {
                fail(GBR_ERR_TIMEOUT, "poll timed out");
            }
        }
        if (out_status) *out_status = empty ? GBR_POLL_QUEUE_EMPTY : GBR_POLL_WAIT_SUCCEEDED;
        if (has_index) {
            auto it = d->records.find(index);
            if (it != d->records.end() && it->second.status != GBR_OK) fail(it->second.status, "%s", it->second.error.c_str());
        }
    })
}

GBR_API gbr_status gbr_submission_stats_get(gbr_device dh, uint64_t index, gbr_submission_stats* out) {
    GBR_TRY({
        auto d = get_device(dh);
        std::lock_guard<std::mutex> lk(d->q_mu);
        auto it = d->records.find(index);
        if (it == d->records.end()) fail(GBR_ERR_INVALID_ARGUMENT, "unknown or unfinished submission");
        *out = it->second.stats;
    })
}

GBR_API gbr_status gbr_device_elapsed_ms(gbr_device dh, uint64_t first, uint64_t last, double* out_ms) {
    GBR_TRY({
        auto d = get_device(dh);
        std::lock_guard<std::mutex> lk(d->q_mu);
        auto a = d->records.find(first), b = d->records.find(last);
        if (a == d->records.end() || b == d->records.end() || !a->second.ev || !b->second.ev)
            fail(GBR_ERR_INVALID_ARGUMENT, "no device timing for these submissions");
        float ms = 0.0f;
        cuda_check(cudaEventElapsedTime(&ms, a->second.ev->start, b->second.ev->end), "cudaEventElapsedTime");
        *out_ms = ms;
    })
}

GBR_API gbr_status gbr_device_memory(gbr_device dh, uint64_t* resident_bytes, uint64_t* transient_bytes) {
    GBR_TRY({
        auto d = get_device(dh);
        if (resident_bytes) *resident_bytes = d->resident->load();
        if (transient_bytes) *transient_bytes = d->scratch_bytes.load();
    })
}

GBR_API gbr_status gbr_device_flush_caches(gbr_device dh) {
    GBR_TRY({
        auto d = get_device(dh);
        Item it;
        it.kind = Item::FLUSH;
        static uint64_t salt = 0;
        it.offset = ++salt;
        d->enqueue(std::move(it));
    })
}

}  // extern "C"
