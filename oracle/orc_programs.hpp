// TEST INFRASTRUCTURE — the oracle (see orc_core.hpp).
//
// orc_programs.hpp — hand-written C++ restatements of the WGSL shader programs used by the
// parity tests and the benchmark workloads, executed with naga-cranelift's arithmetic:
// one IEEE binary32 operation per WGSL operator, no contraction, left-to-right evaluation,
// `mat4x4f * vec4f` as the column sum ((v0*c0 + v1*c1) + v2*c2) + v3*c3
// (naga-cranelift/src/expression/binary.rs:273-325).  The WGSL text of every program lives in
// wgpu-cpu_gb300/shaders/*.wgsl.
#pragma once

#include <cstdint>
#include <cstring>
#include <iterator>
#include <string>
#include <vector>

#include "orc_core.hpp"

namespace orc {

enum Interp { INTERP_LINEAR = 0, INTERP_PERSPECTIVE = 1, INTERP_FLAT = 2 };
enum ScalarKind { SK_F32 = 0, SK_U32 = 1, SK_I32 = 2 };

struct TextureView;  // defined in orc_device.cpp
struct SamplerState;

struct VsIn {
    uint32_t vertex_index, instance_index;
    float attr[16][4];  // vertex attributes by shader location, already decoded to f32 lanes
};
struct VsOut {
    V4 position;
    float var[8][4];  // inter-stage variables by location
};
struct FsIn {
    V4 position;
    bool front_facing;
    uint32_t primitive_index, sample_index, sample_mask;
    float var[8][4];
    float dvar_dx[8][4], dvar_dy[8][4];  // screen-space derivatives of linear inputs (extension sampling)
};
struct FsOut {
    bool killed;
    V4 color[4];
};

// Resources a program may read.  Uniform buffers are raw bytes; textures are sampled through
// the callback, which implements binding.rs:93-164 (and the extension sampler).
struct ProgramBindings {
    const uint8_t* uniform[4][8];
    uint64_t uniform_size[4][8];
    const TextureView* texture[4][8];
    const SamplerState* sampler[4][8];
    // grad = (du/dx, dv/dx, du/dy, dv/dy) of the coordinate; read by extension-profile sampling
    V4 (*sample)(const TextureView*, const SamplerState*, float u, float v, const float grad[4], const void* ctx);
    const void* sample_ctx;
};

struct ProgramInput {
    int location;
    int components;
    int kind;  // ScalarKind
};
struct ProgramVarying {
    int location;
    int components;
    int interp;  // Interp
};
struct ProgramBinding {
    int group, binding;
    int kind;  // 0 uniform buffer, 1 texture, 2 sampler
    uint64_t min_size;
};

struct Program {
    const char* name;
    int num_inputs;
    ProgramInput inputs[4];
    int num_varyings;
    ProgramVarying varyings[4];
    int num_outputs;  // colour outputs at @location(0..n)
    int num_bindings;
    ProgramBinding bindings[4];
    bool (*vs)(const VsIn&, const ProgramBindings&, VsOut&);
    void (*fs)(const FsIn&, const ProgramBindings&, FsOut&);
    // @early_depth_test of the fragment entry point (naga::EarlyDepthTest, read by
    // fragment.rs:83-86): 0 = none, 1 = Force, 2 = Allow
    int early_depth = 0;
};

static inline float ld_f32(const uint8_t* p, size_t off) {
    float f;
    std::memcpy(&f, p + off, 4);
    return f;
}

// mat4x4f (column-major, 16 floats at `m`) * vec4f, column-sum order.
static inline V4 mat4_mul_vec4(const uint8_t* m, V4 v) {
    float vv[4] = {v.x, v.y, v.z, v.w};
    float r[4];
    for (int lane = 0; lane < 4; ++lane) {
        float sum = vv[0] * ld_f32(m, (0 * 4 + lane) * 4);
        sum = sum + vv[1] * ld_f32(m, (1 * 4 + lane) * 4);
        sum = sum + vv[2] * ld_f32(m, (2 * 4 + lane) * 4);
        sum = sum + vv[3] * ld_f32(m, (3 * 4 + lane) * 4);
        r[lane] = sum;
    }
    return {r[0], r[1], r[2], r[3]};
}

// ---- colored_triangle: procedural triangle from vertex_index (the reference's
// wgpu-cpu-tests colored_triangle shader).
static bool vs_colored_triangle(const VsIn& in, const ProgramBindings&, VsOut& out) {
    uint32_t vi = in.vertex_index % 3u;
    float x = (float)((int32_t)vi - 1);
    float y = (float)((int32_t)(vi & 1u) * 2 - 1);
    out.position = {x, y, 0.0f, 1.0f};
    out.var[0][0] = (float)(vi == 0u);
    out.var[0][1] = (float)(vi == 1u);
    out.var[0][2] = (float)(vi == 2u);
    out.var[0][3] = 1.0f;
    return true;
}
static void fs_passthrough_vec4(const FsIn& in, const ProgramBindings&, FsOut& out) {
    out.killed = false;
    out.color[0] = {in.var[0][0], in.var[0][1], in.var[0][2], in.var[0][3]};
}

// ---- mesh_color: position * MVP, per-vertex RGB colour.
static bool vs_mesh_color(const VsIn& in, const ProgramBindings& b, VsOut& out) {
    V4 p = {in.attr[0][0], in.attr[0][1], in.attr[0][2], 1.0f};
    out.position = mat4_mul_vec4(b.uniform[0][0], p);
    out.var[0][0] = in.attr[1][0];
    out.var[0][1] = in.attr[1][1];
    out.var[0][2] = in.attr[1][2];
    return true;
}
static void fs_mesh_color(const FsIn& in, const ProgramBindings&, FsOut& out) {
    out.killed = false;
    out.color[0] = {in.var[0][0], in.var[0][1], in.var[0][2], 1.0f};
}

// ---- mesh_tex_lambert: textured, Lambert term from a light direction in the uniform block
// struct { mvp: mat4x4f, light: vec4f } at @group(0) @binding(0); texture @group(1)
// @binding(0), sampler @group(1) @binding(1).
static bool vs_mesh_tex_lambert(const VsIn& in, const ProgramBindings& b, VsOut& out) {
    V4 p = {in.attr[0][0], in.attr[0][1], in.attr[0][2], 1.0f};
    out.position = mat4_mul_vec4(b.uniform[0][0], p);
    out.var[0][0] = in.attr[1][0];
    out.var[0][1] = in.attr[1][1];
    out.var[0][2] = in.attr[1][2];
    out.var[1][0] = in.attr[2][0];
    out.var[1][1] = in.attr[2][1];
    return true;
}
static void fs_mesh_tex_lambert(const FsIn& in, const ProgramBindings& b, FsOut& out) {
    const float grad[4] = {in.dvar_dx[1][0], in.dvar_dx[1][1], in.dvar_dy[1][0], in.dvar_dy[1][1]};
    V4 t = b.sample(b.texture[1][0], b.sampler[1][1], in.var[1][0], in.var[1][1], grad, b.sample_ctx);
    const uint8_t* u = b.uniform[0][0];
    float lx = ld_f32(u, 64), ly = ld_f32(u, 68), lz = ld_f32(u, 72);
    float d = in.var[0][0] * lx + in.var[0][1] * ly;
    d = d + in.var[0][2] * lz;
    float k = (d > 0.0f) ? d : 0.0f;  // select(0.0, d, d > 0.0)
    out.killed = false;
    out.color[0] = {t.x * k, t.y * k, t.z * k, t.w * k};
}

// ---- quad_color: clip-space position passthrough (w = 1) and a per-vertex RGBA colour.
static bool vs_quad_color(const VsIn& in, const ProgramBindings&, VsOut& out) {
    out.position = {in.attr[0][0], in.attr[0][1], in.attr[0][2], 1.0f};
    for (int k = 0; k < 4; ++k) out.var[0][k] = in.attr[1][k];
    return true;
}

// ---- clip_passthrough: clip-space position (vec4f) and an RGBA colour straight through.
static bool vs_clip_passthrough(const VsIn& in, const ProgramBindings&, VsOut& out) {
    out.position = {in.attr[0][0], in.attr[0][1], in.attr[0][2], in.attr[0][3]};
    for (int k = 0; k < 4; ++k) out.var[0][k] = in.attr[1][k];
    return true;
}

// ---- mesh_color_discard: mesh_color that discards fragments whose red channel is below 0.5
// (exercises `discard` = EntryPointError::Killed, fragment.rs:202-208).
static void fs_mesh_color_discard(const FsIn& in, const ProgramBindings&, FsOut& out) {
    if (in.var[0][0] < 0.5f) {
        out.killed = true;
        return;
    }
    out.killed = false;
    out.color[0] = {in.var[0][0], in.var[0][1], in.var[0][2], 1.0f};
}

// ---- clip_flat_id: @location(0) @interpolate(flat) id: u32 = 0x7fc00000 | (vertex_index &
// 0xffff) (as an f32 a NaN: any arithmetic on the slot would show) and a linear colour; the
// fragment stage returns vec4f(f32(id & 0xffu) / 255.0, colour.x, colour.y, 1.0).
static bool vs_clip_flat_id(const VsIn& in, const ProgramBindings&, VsOut& out) {
    out.position = {in.attr[0][0], in.attr[0][1], in.attr[0][2], in.attr[0][3]};
    const uint32_t id = 0x7fc00000u | (in.vertex_index & 0xffffu);
    std::memcpy(&out.var[0][0], &id, 4);
    for (int k = 0; k < 3; ++k) out.var[1][k] = in.attr[1][k];
    return true;
}
static void fs_clip_flat_id(const FsIn& in, const ProgramBindings&, FsOut& out) {
    uint32_t id;
    std::memcpy(&id, &in.var[0][0], 4);
    out.killed = false;
    out.color[0] = {(float)(id & 0xffu) / 255.0f, in.var[1][0], in.var[1][1], 1.0f};
}
// ---- clip_discard: clip_passthrough that discards fragments whose red channel is below 0.5.
static void fs_clip_discard(const FsIn& in, const ProgramBindings&, FsOut& out) {
    if (in.var[0][0] < 0.5f) {
        out.killed = true;
        return;
    }
    out.killed = false;
    out.color[0] = {in.var[0][0], in.var[0][1], in.var[0][2], in.var[0][3]};
}

static const Program kBasePrograms[] = {
    {"colored_triangle", 0, {}, 1, {{0, 4, INTERP_LINEAR}}, 1, 0, {}, vs_colored_triangle, fs_passthrough_vec4},
    {"mesh_color", 2, {{0, 3, SK_F32}, {1, 3, SK_F32}}, 1, {{0, 3, INTERP_LINEAR}}, 1, 1, {{0, 0, 0, 64}},
     vs_mesh_color, fs_mesh_color},
    {"mesh_color_perspective", 2, {{0, 3, SK_F32}, {1, 3, SK_F32}}, 1, {{0, 3, INTERP_PERSPECTIVE}}, 1, 1,
     {{0, 0, 0, 64}}, vs_mesh_color, fs_mesh_color},
    {"mesh_color_discard", 2, {{0, 3, SK_F32}, {1, 3, SK_F32}}, 1, {{0, 3, INTERP_LINEAR}}, 1, 1,
     {{0, 0, 0, 64}}, vs_mesh_color, fs_mesh_color_discard},
    {"mesh_tex_lambert", 3, {{0, 3, SK_F32}, {1, 3, SK_F32}, {2, 2, SK_F32}}, 2,
     {{0, 3, INTERP_LINEAR}, {1, 2, INTERP_LINEAR}}, 1, 3, {{0, 0, 0, 80}, {1, 0, 1, 0}, {1, 1, 2, 0}},
     vs_mesh_tex_lambert, fs_mesh_tex_lambert},
    {"quad_color", 2, {{0, 3, SK_F32}, {1, 4, SK_F32}}, 1, {{0, 4, INTERP_LINEAR}}, 1, 0, {}, vs_quad_color,
     fs_passthrough_vec4},
    {"clip_passthrough", 2, {{0, 4, SK_F32}, {1, 4, SK_F32}}, 1, {{0, 4, INTERP_LINEAR}}, 1, 0, {},
     vs_clip_passthrough, fs_passthrough_vec4},
    {"clip_flat", 2, {{0, 4, SK_F32}, {1, 4, SK_F32}}, 1, {{0, 4, INTERP_FLAT}}, 1, 0, {}, vs_clip_passthrough,
     fs_passthrough_vec4},
    {"clip_flat_id", 2, {{0, 4, SK_F32}, {1, 4, SK_F32}}, 2, {{0, 1, INTERP_FLAT}, {1, 3, INTERP_LINEAR}}, 1, 0, {},
     vs_clip_flat_id, fs_clip_flat_id},
    {"clip_discard", 2, {{0, 4, SK_F32}, {1, 4, SK_F32}}, 1, {{0, 4, INTERP_LINEAR}}, 1, 0, {}, vs_clip_passthrough,
     fs_clip_discard},
};

// The programs, and the variants whose fragment entry point carries @early_depth_test(force)
// ("<name>@early_force") or @early_depth_test(<conservative>) ("<name>@early_allow").
static inline const std::vector<Program>& programs() {
    static const std::vector<Program> table = [] {
        std::vector<Program> v(std::begin(kBasePrograms), std::end(kBasePrograms));
        static const char* const kEarly[] = {"clip_passthrough", "clip_discard", "clip_flat_id", "mesh_color",
                                             "mesh_color_discard"};
        static std::vector<std::string> names;
        names.reserve(2 * (sizeof kEarly / sizeof kEarly[0]));
        const size_t base = v.size();
        for (const char* n : kEarly)
            for (int mode : {1, 2})
                for (size_t i = 0; i < base; ++i)
                    if (std::strcmp(v[i].name, n) == 0) {
                        names.push_back(std::string(n) + (mode == 1 ? "@early_force" : "@early_allow"));
                        Program q = v[i];
                        q.name = names.back().c_str();
                        q.early_depth = mode;
                        v.push_back(q);
                    }
        return v;
    }();
    return table;
}

static inline const Program* find_program(const char* name) {
    for (const Program& p : programs())
        if (std::strcmp(p.name, name) == 0) return &p;
    return nullptr;
}

}  // namespace orc
