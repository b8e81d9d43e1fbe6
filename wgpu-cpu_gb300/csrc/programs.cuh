// programs.cuh — the library's native shader programs: hand-written CUDA versions of the WGSL
// programs in shaders/*.wgsl, evaluated with naga-cranelift's arithmetic (one rounded IEEE op
// per WGSL operator, left to right; mat4x4f * vec4f as the column sum
// ((v0*c0 + v1*c1) + v2*c2) + v3*c3, naga-cranelift/src/expression/binary.rs:273-325).
//
// Also here: vertex attribute fetch (render_pass/vertex.rs:128-156, 191-195) and the nearest
// texture sampler of render_pass/binding.rs:93-164.
#pragma once

#include "exact.cuh"
#include "gbr_types.h"
#include "sampling.cuh"

namespace gbr {

// gbr_vertex_format sizes (wgpu VertexFormat::size)
__device__ __forceinline__ uint32_t vertex_format_size(uint32_t f) {
    switch (f) {
        case 1: case 5: case 6: case 7: case 9: return 4;  // f32, u32, i32, f16x2, unorm8x4
        case 2: case 8: return 8;                          // f32x2, f16x4
        case 3: return 12;
        case 4: return 16;
        default: return 0;
    }
}

// Fetch `comps` f32 lanes of the attribute at `loc`.  In the parity profile the bytes are copied
// as they are (the reference copies `format.size()` bytes into the shader input; the host
// rejects pipelines whose format size differs from the input's); the extension profile
// converts Float16x4 / Unorm8x4 to f32 as WebGPU does.
__device__ __forceinline__ bool fetch_attr(const DrawDesc& d, int loc, int comps, uint32_t vertex, uint32_t instance,
                                           float out[4], uint32_t* err) {
    const AttrDesc a = d.attr[loc];
    if (a.buffer < 0) {
        *err = ERR_UNSUPPORTED;
        return false;
    }
    const int b = a.buffer;
    const uint64_t start = (uint64_t)instance * d.vb_stride_instance[b] + (uint64_t)vertex * d.vb_stride_vertex[b] +
                           a.offset;
    const uint32_t fsize = vertex_format_size(a.format);
    if (start + fsize > d.vb_size[b]) {
        *err = ERR_VERTEX_OOB;
        return false;
    }
    const uint8_t* p = d.vb_data[b] + start;
    if (a.format == 8 /* f16x4 */ && comps == 4) {
        const uint16_t* h = reinterpret_cast<const uint16_t*>(p);
        for (int k = 0; k < 4; ++k) out[k] = f16_bits_to_f32(__ldg(h + k));
    } else if (a.format == 9 /* unorm8x4 */ && comps == 4) {
        for (int k = 0; k < 4; ++k) out[k] = fdiv((float)__ldg(p + k), 255.0f);
    } else {
        const float* f = reinterpret_cast<const float*>(p);
        for (int k = 0; k < comps; ++k) out[k] = __ldg(f + k);
    }
    return true;
}

__device__ __forceinline__ float ld_uniform(const DrawDesc& d, int group, int binding, uint32_t byte_off) {
    return __ldg(reinterpret_cast<const float*>(d.uniform[group][binding] + byte_off));
}

// mat4x4f (column-major, 16 floats at m) * vec4f, column-sum order.
__device__ __forceinline__ V4 mat4_mul_vec4(const float* m, V4 v) {
    float r[4];
#pragma unroll
    for (int lane = 0; lane < 4; ++lane) {
        float s = fmul(v.x, m[0 * 4 + lane]);
        s = fadd(s, fmul(v.y, m[1 * 4 + lane]));
        s = fadd(s, fmul(v.z, m[2 * 4 + lane]));
        s = fadd(s, fmul(v.w, m[3 * 4 + lane]));
        r[lane] = s;
    }
    return {r[0], r[1], r[2], r[3]};
}

// texel_coordinate (render_pass/binding.rs:150-164)
__device__ __forceinline__ uint32_t texel_coordinate(float x, uint32_t mode, uint32_t size) {
    if (mode == 0) {  // ClampToEdge: f32::clamp keeps NaN
        if (x < 0.0f) x = 0.0f;
        if (x > 1.0f) x = 1.0f;
    } else if (mode == 1) {  // Repeat: rem_euclid(1.0)
        float r = fmodf(x, 1.0f);
        x = (r < 0.0f) ? fadd(r, 1.0f) : r;
    } else {  // MirrorRepeat: rem_euclid(2.0), fold
        float r = fmodf(x, 2.0f);
        r = (r < 0.0f) ? fadd(r, 2.0f) : r;
        x = (r <= 1.0f) ? r : fsub(2.0f, r);
    }
    return rust_f2u32(roundf(fmul(x, (float)(size - 1u))));
}

// image_sample, nearest, mip 0 of an Rgba8 texture, `x as f32 / 255.0` per channel
// (render_pass/binding.rs:93-140, texture.rs:170-188).
__device__ __forceinline__ V4 sample_nearest_rgba8(const TexDesc& t, const SamplerDescDev& s, float u, float v) {
    uint32_t x = texel_coordinate(u, s.address_u, t.width);
    uint32_t y = texel_coordinate(v, s.address_v, t.height);
    uint32_t px = __ldg(reinterpret_cast<const uint32_t*>(t.data) + (size_t)y * t.width + x);
    return {fdiv((float)(px & 0xFFu), 255.0f), fdiv((float)((px >> 8) & 0xFFu), 255.0f),
            fdiv((float)((px >> 16) & 0xFFu), 255.0f), fdiv((float)(px >> 24), 255.0f)};
}

// ---------------------------------------------------------------------------- programs
// Number of f32 inter-stage values per vertex and their interpolation, by program.
__host__ __device__ __forceinline__ uint32_t program_num_varyings(uint32_t prog) {
    switch (prog) {
        case PROG_COLORED_TRIANGLE: return 4;
        case PROG_MESH_COLOR:
        case PROG_MESH_COLOR_PERSPECTIVE:
        case PROG_MESH_COLOR_DISCARD: return 3;
        case PROG_MESH_TEX_LAMBERT: return 5;
        case PROG_QUAD_COLOR:
        case PROG_CLIP_PASSTHROUGH:
        case PROG_CLIP_FLAT:
        case PROG_CLIP_FLAT_ID:
        case PROG_CLIP_DISCARD: return 4;
        default: return 0;
    }
}
__host__ __device__ __forceinline__ uint32_t program_interp(uint32_t prog) {
    return prog == PROG_MESH_COLOR_PERSPECTIVE ? INTERP_PERSPECTIVE : INTERP_LINEAR;
}

#ifdef GBR_JIT
// The WGSL program of a JIT module (emitted by wgsl.cpp, defined later in the same unit).
__device__ bool jit_vs(const DrawDesc& d, uint32_t vertex, uint32_t instance, V4& pos, float* var, uint32_t* err);
__device__ int jit_fs(const DrawDesc& d, const float* var, bool front_facing, uint32_t prim_index, V4 frag, V4& color);
#endif

// Vertex stage: position + varyings.  Returns false with *err set on a fetch error.  `mvp` is a
// copy of the 16 floats at group 0 / binding 0 (the mesh programs' matrix), or null to read them
// from the uniform buffer.
__device__ __forceinline__ bool run_vs(const DrawDesc& d, const float* mvp, uint32_t vertex, uint32_t instance,
                                       V4& pos, float* var, uint32_t* err) {
    float a0[4], a1[4], a2[4];
    const float* m = mvp ? mvp : reinterpret_cast<const float*>(d.uniform[0][0]);
    switch (d.program) {
        case PROG_COLORED_TRIANGLE: {
            uint32_t vi = vertex % 3u;
            float x = (float)((int32_t)vi - 1);
            float y = (float)((int32_t)(vi & 1u) * 2 - 1);
            pos = {x, y, 0.0f, 1.0f};
            var[0] = (float)(vi == 0u);
            var[1] = (float)(vi == 1u);
            var[2] = (float)(vi == 2u);
            var[3] = 1.0f;
            return true;
        }
        case PROG_MESH_COLOR:
        case PROG_MESH_COLOR_PERSPECTIVE:
        case PROG_MESH_COLOR_DISCARD: {
            if (!fetch_attr(d, 0, 3, vertex, instance, a0, err)) return false;
            if (!fetch_attr(d, 1, 3, vertex, instance, a1, err)) return false;
            pos = mat4_mul_vec4(m, V4{a0[0], a0[1], a0[2], 1.0f});
            var[0] = a1[0];
            var[1] = a1[1];
            var[2] = a1[2];
            return true;
        }
        case PROG_MESH_TEX_LAMBERT: {
            if (!fetch_attr(d, 0, 3, vertex, instance, a0, err)) return false;
            if (!fetch_attr(d, 1, 3, vertex, instance, a1, err)) return false;
            if (!fetch_attr(d, 2, 2, vertex, instance, a2, err)) return false;
            pos = mat4_mul_vec4(m, V4{a0[0], a0[1], a0[2], 1.0f});
            var[0] = a1[0];
            var[1] = a1[1];
            var[2] = a1[2];
            var[3] = a2[0];
            var[4] = a2[1];
            return true;
        }
        case PROG_QUAD_COLOR: {
            if (!fetch_attr(d, 0, 3, vertex, instance, a0, err)) return false;
            if (!fetch_attr(d, 1, 4, vertex, instance, a1, err)) return false;
            pos = {a0[0], a0[1], a0[2], 1.0f};
            var[0] = a1[0];
            var[1] = a1[1];
            var[2] = a1[2];
            var[3] = a1[3];
            return true;
        }
        case PROG_CLIP_PASSTHROUGH:
        case PROG_CLIP_FLAT:
        case PROG_CLIP_DISCARD: {
            if (!fetch_attr(d, 0, 4, vertex, instance, a0, err)) return false;
            if (!fetch_attr(d, 1, 4, vertex, instance, a1, err)) return false;
            pos = {a0[0], a0[1], a0[2], a0[3]};
            var[0] = a1[0];
            var[1] = a1[1];
            var[2] = a1[2];
            var[3] = a1[3];
            return true;
        }
        case PROG_CLIP_FLAT_ID: {
            // @location(0) @interpolate(flat) id: u32 = 0x7fc00000 | (vertex_index & 0xffff) — as
            // an f32 a NaN, so any arithmetic on the slot would show; @location(1) colour.xyz linear
            if (!fetch_attr(d, 0, 4, vertex, instance, a0, err)) return false;
            if (!fetch_attr(d, 1, 4, vertex, instance, a1, err)) return false;
            pos = {a0[0], a0[1], a0[2], a0[3]};
            var[0] = __uint_as_float(0x7fc00000u | (vertex & 0xffffu));
            var[1] = a1[0];
            var[2] = a1[1];
            var[3] = a1[2];
            return true;
        }
#ifdef GBR_JIT
        case PROG_JIT: return jit_vs(d, vertex, instance, pos, var, err);
#endif
        default: *err = ERR_UNSUPPORTED; return false;
    }
}

// What the fragment stage and the output merger need of a draw, cached per warp in shared
// memory by the raster kernel (built from the DrawDesc in global memory).
struct RasterState {
    const DrawDesc* dd;  // the draw itself (for programs that read more of it)
    uint32_t draw;  // DrawDesc index this copy was built from
    uint32_t program, nvar, interp;
    uint32_t sc_x0, sc_y0, sc_x1, sc_y1;
    uint32_t depth_test, depth_compare, depth_write;
    uint32_t blend_enabled, write_mask;
    uint32_t blend_over;  // colour SrcAlpha/OneMinusSrcAlpha/Add, alpha One/OneMinusSrcAlpha/Add
    uint32_t blend_color[3], blend_alpha[3];
    float blend_constant[4];
    const uint8_t* tex_data;
    uint32_t tex_w, tex_h, addr_u, addr_v;
    uint32_t tex_ext;  // extension-profile sampling (sample_ext with the record's LOD)
    float uconst[4];  // program constants read from the uniform block (light direction)
    uint32_t flat_mask;    // DrawDesc::flat_mask
    uint32_t early_depth;  // DrawDesc::early_depth
};

__device__ __forceinline__ void build_raster_state(const DrawDesc& d, uint32_t di, RasterState& rs) {
    rs.dd = &d;
    rs.draw = di;
    rs.program = d.program;
    rs.nvar = d.num_varyings;
    rs.interp = d.interp;
    rs.sc_x0 = d.sc_x0;
    rs.sc_y0 = d.sc_y0;
    rs.sc_x1 = d.sc_x1;
    rs.sc_y1 = d.sc_y1;
    rs.depth_test = d.depth_test;
    rs.depth_compare = d.depth_compare;
    rs.depth_write = d.depth_write;
    rs.blend_enabled = d.blend_enabled;
    rs.write_mask = d.write_mask;
    for (int k = 0; k < 3; ++k) {
        rs.blend_color[k] = d.blend_color[k];
        rs.blend_alpha[k] = d.blend_alpha[k];
    }
    for (int k = 0; k < 4; ++k) rs.blend_constant[k] = d.blend_constant[k];
    rs.blend_over = d.blend_color[0] == 4 && d.blend_color[1] == 5 && d.blend_color[2] == 0 && d.blend_alpha[0] == 1 &&
                    d.blend_alpha[1] == 5 && d.blend_alpha[2] == 0;
    rs.tex_data = d.tex.data;
    rs.tex_w = d.tex.width;
    rs.tex_h = d.tex.height;
    rs.addr_u = d.samp.address_u;
    rs.addr_v = d.samp.address_v;
    rs.tex_ext = d.lod_var != 0;
    rs.flat_mask = d.flat_mask;
    rs.early_depth = d.early_depth;
    for (int k = 0; k < 4; ++k) rs.uconst[k] = 0.0f;
    if (d.program == PROG_MESH_TEX_LAMBERT) {
        rs.uconst[0] = ld_uniform(d, 0, 0, 64);
        rs.uconst[1] = ld_uniform(d, 0, 0, 68);
        rs.uconst[2] = ld_uniform(d, 0, 0, 72);
    }
}

// texel_coordinate with Repeat computed as x - trunc(x): for finite x this is exactly
// fmodf(x, 1.0) (the fractional part of a binary32 value is representable and the subtraction
// is exact); the two can differ only in the sign of a zero result, which the following
// `< 0`, multiply, round and saturating cast map to the same texel 0.  Infinite/NaN x give NaN
// either way.
__device__ __forceinline__ uint32_t texel_coordinate_fast(float x, uint32_t mode, uint32_t size) {
    if (mode == 1) {
        float r = fsub(x, truncf(x));
        x = (r < 0.0f) ? fadd(r, 1.0f) : r;
        return rust_f2u32(roundf(fmul(x, (float)(size - 1u))));
    }
    return texel_coordinate(x, mode, size);
}

// Nearest Rgba8 sample with `x as f32 / 255.0` from a table of exactly those 256 quotients.
__device__ __forceinline__ V4 sample_nearest_rgba8_lut(const RasterState& rs, float u, float v, const float* lut) {
    uint32_t x = texel_coordinate_fast(u, rs.addr_u, rs.tex_w);
    uint32_t y = texel_coordinate_fast(v, rs.addr_v, rs.tex_h);
    uint32_t px = __ldg(reinterpret_cast<const uint32_t*>(rs.tex_data) + (size_t)y * rs.tex_w + x);
    return {lut[px & 0xFFu], lut[(px >> 8) & 0xFFu], lut[(px >> 16) & 0xFFu], lut[px >> 24]};
}

// Fragment stage on the cached state.  Returns false when the fragment is discarded.  `lod` is
// the record's texture LOD (extension-profile sampling only).
__device__ __forceinline__ bool run_fs_rs(const RasterState& rs, const float* var, const float* lut, V4& color,
                                          float lod = 0.0f) {
    switch (rs.program) {
        case PROG_COLORED_TRIANGLE:
        case PROG_QUAD_COLOR:
        case PROG_CLIP_PASSTHROUGH:
        case PROG_CLIP_FLAT: color = {var[0], var[1], var[2], var[3]}; return true;
        case PROG_CLIP_FLAT_ID:  // vec4f(f32(id & 0xffu) / 255.0, colour.x, colour.y, 1.0)
            color = {fdiv((float)(__float_as_uint(var[0]) & 0xffu), 255.0f), var[1], var[2], 1.0f};
            return true;
        case PROG_CLIP_DISCARD:
            if (var[0] < 0.5f) return false;
            color = {var[0], var[1], var[2], var[3]};
            return true;
        case PROG_MESH_COLOR:
        case PROG_MESH_COLOR_PERSPECTIVE: color = {var[0], var[1], var[2], 1.0f}; return true;
        case PROG_MESH_COLOR_DISCARD:
            if (var[0] < 0.5f) return false;
            color = {var[0], var[1], var[2], 1.0f};
            return true;
        case PROG_MESH_TEX_LAMBERT: {
            V4 t = rs.tex_ext ? sample_ext(rs.dd->tex, rs.dd->samp, var[3], var[4], lod, lut)
                              : sample_nearest_rgba8_lut(rs, var[3], var[4], lut);
            float dd = fadd(fmul(var[0], rs.uconst[0]), fmul(var[1], rs.uconst[1]));
            dd = fadd(dd, fmul(var[2], rs.uconst[2]));
            float k = (dd > 0.0f) ? dd : 0.0f;  // select(0.0, d, d > 0.0)
            color = {fmul(t.x, k), fmul(t.y, k), fmul(t.z, k), fmul(t.w, k)};
            return true;
        }
        default: return false;
    }
}

}  // namespace gbr
