// raster_lines.cuh — line and point primitives.
//
// The reference draws them with LineRasterizer (render_pass/raster.rs:233-265: Cohen–Sutherland
// clipping, clipper.rs:268-356; Bresenham without the end point, util/bresenham.rs:17-153, whose
// `t` accumulates 1/dx step by step) and PointRasterizer (raster.rs:197-218), fragment by fragment
// in primitive order.  k_lines_points keeps that order exactly: one CTA walks a draw's primitives
// in turn (assembly, vertex stage, clipping, snapping on one thread), and its threads split each
// line's pixels into contiguous runs; a thread replays the integer error term and the f32 `t`
// sum from the line's start to its run (the same additions in the same order), then processes
// its pixels.  A line's pixels are distinct, so only consecutive primitives need ordering — one
// barrier each.  Fragments are tested and written straight in global memory.
#pragma once

#include "raster.cuh"

namespace gbr {

// clip_line (clipper.rs:268-356): false when the line is outside; alphas of the kept part.
__device__ __forceinline__ bool clip_line_dev(V4 pts[2], float alphas_out[2]) {
    float dist[2][6];
    unsigned outcode[2] = {0, 0};
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int p = 0; p < 6; ++p) {
            dist[i][p] = dot4(pts[i], clip_plane(p));
            if (dist[i][p] < 0.0f) outcode[i] |= 1u << p;
        }
    const unsigned o_or = outcode[0] | outcode[1], o_and = outcode[0] & outcode[1];
    if (o_or == 0) {
        alphas_out[0] = 0.0f;
        alphas_out[1] = 1.0f;
        return true;
    }
    if (o_and != 0) return false;
    float alphas[2] = {0.0f, 1.0f};
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        const unsigned bit = 1u << p;
        if (o_or & bit) {
            const float a = dist[0][p], b = dist[1][p];
            const float alpha = fdiv(a, fsub(a, b));
            if (outcode[0] & bit) {
                if (alpha > alphas[0]) alphas[0] = alpha;
            } else {
                if (alpha < alphas[1]) alphas[1] = alpha;
            }
            if (alphas[0] > alphas[1]) return false;
        }
    }
    V4 p0 = pts[0];
    const V4 p1 = pts[1];
    // point 0 is moved first; moving point 1 then reads the moved point 0 (clipper.rs:337-352)
    if (outcode[0] != 0) {
        const float t = alphas[0], omt = fsub(1.0f, t);
        pts[0] = v4_add(v4_mul(p0, omt), v4_mul(p1, t));
        p0 = pts[0];
    }
    if (outcode[1] != 0) {
        const float t = alphas[1], omt = fsub(1.0f, t);
        pts[1] = v4_add(v4_mul(p0, omt), v4_mul(p1, t));
    }
    alphas_out[0] = alphas[0];
    alphas_out[1] = alphas[1];
    return true;
}

// Bresenham's octant maps (util/bresenham.rs:17-76)
__device__ __forceinline__ void oct_to0(int oct, int64_t x, int64_t y, int64_t& ox, int64_t& oy) {
    switch (oct) {
        case 0: ox = x; oy = y; break;
        case 1: ox = y; oy = x; break;
        case 2: ox = y; oy = -x; break;
        case 3: ox = -x; oy = y; break;
        case 4: ox = -x; oy = -y; break;
        case 5: ox = -y; oy = -x; break;
        case 6: ox = -y; oy = x; break;
        default: ox = x; oy = -y; break;
    }
}
__device__ __forceinline__ void oct_from0(int oct, int64_t x, int64_t y, int64_t& ox, int64_t& oy) {
    switch (oct) {
        case 0: ox = x; oy = y; break;
        case 1: ox = y; oy = x; break;
        case 2: ox = -y; oy = x; break;
        case 3: ox = -x; oy = y; break;
        case 4: ox = -x; oy = -y; break;
        case 5: ox = -y; oy = -x; break;
        case 6: ox = y; oy = -x; break;
        default: ox = x; oy = -y; break;
    }
}

struct LinePrim {
    int ok;             // 0 = nothing to rasterise
    int verts;          // 1 (point) or 2 (line)
    uint32_t prim_index;
    V4 frag[2];         // to_raster fragments of the (clipped) end points
    uint32_t fbx[2], fby[2];
    float alpha[2];     // clip alphas of the kept part
    float inv_w[2];     // 1/w of the unclipped vertices
    float var[2][MAX_VARYING_FLOATS];
};

// One fragment of a line or point: interpolation (fragment.rs:319-378), fragment stage, late
// depth test at the first colour output, blend / write mask, colour write — in global memory.
__device__ __forceinline__ void line_fragment(const BatchParams& bp, const DrawDesc& d, const TargetDesc& tg,
                                              const RasterState& rs, const float* lut, const LinePrim& lp, uint32_t x,
                                              uint32_t y, V4 fragment, const float coeff[2], uint32_t& frag_count,
                                              uint32_t& fs_count) {
    ++frag_count;
    const size_t pix = (size_t)y * tg.width + x;
    if (rs.early_depth != EARLY_DEPTH_NONE && rs.depth_test) {  // @early_depth_test (fragment.rs:166-194)
        if (!depth_compare(rs.depth_compare, fragment.z, tg.depth[pix])) return;
        if (rs.depth_write) tg.depth[pix] = fragment.z;
    }
    ++fs_count;
    const uint32_t nvar = rs.nvar;
    float var[MAX_VARYING_FLOATS];
#pragma unroll
    for (uint32_t q = 0; q < MAX_VARYING_FLOATS; ++q) {
        if (q >= nvar) break;
        if (rs.interp == INTERP_PERSPECTIVE) {
            float num = fmul(fmul(lp.var[0][q], coeff[0]), lp.inv_w[0]);
            float den = fmul(coeff[0], lp.inv_w[0]);
            if (lp.verts == 2) {
                num = fadd(num, fmul(fmul(lp.var[1][q], coeff[1]), lp.inv_w[1]));
                den = fadd(den, fmul(coeff[1], lp.inv_w[1]));
            }
            var[q] = fdiv(num, den);
        } else {
            float a = fmul(lp.var[0][q], coeff[0]);
            if (lp.verts == 2) a = fadd(a, fmul(lp.var[1][q], coeff[1]));
            var[q] = a;
        }
        if ((rs.flat_mask >> q) & 1u) var[q] = lp.var[0][q];  // @interpolate(flat): the first vertex
    }
    V4 col;
    bool keep;
#ifdef GBR_JIT
    if (rs.program == PROG_JIT) {
        const int st = jit_fs(d, var, true, lp.prim_index, fragment, col);
        if (st == 2) raise_error(bp.status, ERR_SHADER_TRAP, lp.prim_index);
        keep = st == 1;
    } else
#endif
    {
        // lines and points have no area: zero derivatives, the sampler's minimum LOD
        const float lod = rs.tex_ext ? lod_from_grad(0.0f, 0.0f, 0.0f, 0.0f, rs.dd->tex.width, rs.dd->tex.height,
                                                     rs.dd->samp.lod_min, rs.dd->samp.lod_max)
                                     : 0.0f;
        keep = run_fs_rs(rs, var, lut, col, lod);
    }
    if (!keep) return;  // discard
    if (rs.depth_test && rs.early_depth != EARLY_DEPTH_FORCE) {  // the late test
        const float stored = tg.depth[pix];
        if (!depth_compare(rs.depth_compare, fragment.z, stored)) return;
        if (rs.depth_write) tg.depth[pix] = fragment.z;
    }
    if (!tg.color) return;
    uint8_t* dst = tg.color + tg.slice_offset + pix * tg.color_bpp;
    uint32_t c[4] = {0, 0, 0, 0};
    if (tg.color_bpp == 4) c[0] = *reinterpret_cast<const uint32_t*>(dst);
    else if (tg.color_bpp == 8) { c[0] = reinterpret_cast<const uint32_t*>(dst)[0]; c[1] = reinterpret_cast<const uint32_t*>(dst)[1]; }
    else if (tg.color_bpp == 16) { for (int q = 0; q < 4; ++q) c[q] = reinterpret_cast<const uint32_t*>(dst)[q]; }
    else if (tg.color_bpp == 2) c[0] = *reinterpret_cast<const uint16_t*>(dst);
    else c[0] = *dst;
    if (rs.blend_enabled || rs.write_mask != 0xF) {
        const V4 dv = decode_color(tg.color_format, c);
        if (rs.blend_enabled) {
            V4 o;
            o.x = blend_channel(rs.blend_color, col.x, col.w, dv.x, dv.w, rs.blend_constant[0]);
            o.y = blend_channel(rs.blend_color, col.y, col.w, dv.y, dv.w, rs.blend_constant[1]);
            o.z = blend_channel(rs.blend_color, col.z, col.w, dv.z, dv.w, rs.blend_constant[2]);
            o.w = blend_channel(rs.blend_alpha, col.w, col.w, dv.w, dv.w, rs.blend_constant[3]);
            col = o;
        }
        if (!(rs.write_mask & 1)) col.x = dv.x;
        if (!(rs.write_mask & 2)) col.y = dv.y;
        if (!(rs.write_mask & 4)) col.z = dv.z;
        if (!(rs.write_mask & 8)) col.w = dv.w;
    }
    encode_color(tg.color_format, col, c);
    if (tg.color_bpp == 4) *reinterpret_cast<uint32_t*>(dst) = c[0];
    else if (tg.color_bpp == 8) reinterpret_cast<uint2*>(dst)[0] = make_uint2(c[0], c[1]);
    else if (tg.color_bpp == 16) reinterpret_cast<uint4*>(dst)[0] = make_uint4(c[0], c[1], c[2], c[3]);
    else if (tg.color_bpp == 2) *reinterpret_cast<uint16_t*>(dst) = (uint16_t)c[0];
    else *dst = (uint8_t)c[0];
}

// LoadOp::Clear of a batch's targets (texture.rs:199-211) for passes drawn by k_lines_points.
__global__ void k_clear_targets(BatchParams bp) {
    for (uint32_t ti = 0; ti < bp.num_targets; ++ti) {
        const TargetDesc& t = bp.targets[ti];
        const bool cc = t.color && t.color_load == 1, cd = t.depth && t.depth_load == 1;
        if (!cc && !cd) continue;
        uint32_t c[4] = {0, 0, 0, 0};
        if (cc) encode_color(t.color_format, V4{t.clear[0], t.clear[1], t.clear[2], t.clear[3]}, c);
        const size_t n = (size_t)t.width * t.height;
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
            if (cd) t.depth[i] = t.depth_clear;
            if (cc) {
                uint8_t* dst = t.color + t.slice_offset + i * t.color_bpp;
                if (t.color_bpp == 4) *reinterpret_cast<uint32_t*>(dst) = c[0];
                else if (t.color_bpp == 8) reinterpret_cast<uint2*>(dst)[0] = make_uint2(c[0], c[1]);
                else if (t.color_bpp == 16) reinterpret_cast<uint4*>(dst)[0] = make_uint4(c[0], c[1], c[2], c[3]);
                else if (t.color_bpp == 2) *reinterpret_cast<uint16_t*>(dst) = (uint16_t)c[0];
                else *dst = (uint8_t)c[0];
            }
        }
    }
}

constexpr int kLineThreads = 256;

// The line / point draw of a batch (one draw per batch), one CTA.
__global__ void __launch_bounds__(kLineThreads) k_lines_points(BatchParams bp) {
    __shared__ RasterState s_rs;
    __shared__ float s_lut[256];
    __shared__ LinePrim s_p;
    __shared__ unsigned long long s_frag;
    if (bp.status->error || *bp.abort_flag || bp.num_draws == 0) return;  // (an empty draw only clears)
    const DrawDesc& d = bp.draws[0];
    const TargetDesc& tg = bp.targets[d.target];
    for (int i = threadIdx.x; i < 256; i += kLineThreads) s_lut[i] = fdiv((float)i, 255.0f);
    if (threadIdx.x == 0) {
        build_raster_state(d, 0, s_rs);
        s_frag = 0;
    }
    __syncthreads();
    const bool point = d.topology == 0;
    const bool strip = d.topology == 2;
    uint32_t frag_count = 0, fs_count = 0;
    for (uint32_t inst = 0; inst < d.instance_count; ++inst) {
        uint32_t compact = 0;  // primitive_index of the next primitive (thread 0)
        for (uint32_t p = 0; p < d.prims_per_instance; ++p) {
            if (threadIdx.x == 0) {
                LinePrim& lp = s_p;
                lp.ok = 0;
                lp.verts = point ? 1 : 2;
                uint32_t sp[2] = {point ? p : strip ? p : 2 * p, strip ? p + 1 : 2 * p + 1};
                bool skip = false;
                if (d.strip_restart) {  // a separator at either end: no line here (primitive.rs:287-322)
                    const bool u16 = d.index_format == 1;
                    for (int k = 0; k < 2 && !skip; ++k) {
                        const uint32_t at = d.first + sp[k];
                        if ((uint64_t)(at + 1) * (u16 ? 2u : 4u) > d.index_bytes) break;  // reported below
                        skip = u16 ? __ldg(reinterpret_cast<const uint16_t*>(d.index_data) + at) == 0xFFFFu
                                   : __ldg(reinterpret_cast<const uint32_t*>(d.index_data) + at) == 0xFFFFFFFFu;
                    }
                }
                if (!skip) {
                    lp.prim_index = compact++;
                    V4 pos[2];
                    uint32_t err = 0;
                    bool ok = true;
                    for (int k = 0; k < lp.verts && ok; ++k) {
                        uint32_t vertex = 0;
                        ok = resolve_vertex(d, sp[k], vertex, &err) &&
                             run_vs(d, nullptr, vertex, d.instance_start + inst, pos[k], lp.var[k], &err);
                    }
                    if (!ok) {
                        raise_error(bp.status, err, d.prim_base + p);
                    } else if (!d.has_fragment) {
                    } else if (point) {
                        // PointRasterizer (raster.rs:197-218): the snapped vertex, if inside
                        uint32_t fx, fy;
                        V4 f;
                        if (pos[0].w == 0.0f || !to_raster(d, pos[0], fx, fy, f)) {
                            raise_error(bp.status, ERR_W_ZERO, d.prim_base + p);
                        } else {
                            lp.inv_w[0] = fdiv(1.0f, pos[0].w);
                            lp.frag[0] = f;
                            lp.fbx[0] = fx;
                            lp.fby[0] = fy;
                            lp.ok = 1;
                        }
                    } else {
                        lp.inv_w[0] = fdiv(1.0f, pos[0].w);
                        lp.inv_w[1] = fdiv(1.0f, pos[1].w);
                        if (clip_line_dev(pos, lp.alpha)) {
                            bool r0 = to_raster(d, pos[0], lp.fbx[0], lp.fby[0], lp.frag[0]);
                            bool r1 = to_raster(d, pos[1], lp.fbx[1], lp.fby[1], lp.frag[1]);
                            if (!r0 || !r1) raise_error(bp.status, ERR_W_ZERO, d.prim_base + p);
                            else lp.ok = 1;
                        }
                    }
                }
            }
            __syncthreads();
            if (s_p.ok && bp.status->error == 0) {
                const LinePrim& lp = s_p;
                if (lp.verts == 1) {
                    if (threadIdx.x == 0) {
                        const uint32_t x = lp.fbx[0], y = lp.fby[0];
                        if (x >= d.sc_x0 && x < d.sc_x1 && y >= d.sc_y0 && y < d.sc_y1 && x < tg.width && y < tg.height) {
                            const float coeff[2] = {1.0f, 0.0f};
                            line_fragment(bp, d, tg, s_rs, s_lut, lp, x, y, lp.frag[0], coeff, frag_count, fs_count);
                        }
                    }
                } else {
                    // Bresenham in octant 0 (util/bresenham.rs:78-153), end point excluded
                    int64_t sx = lp.fbx[0], sy = lp.fby[0], ex = lp.fbx[1], ey = lp.fby[1];
                    int64_t dx = ex - sx, dy = ey - sy;
                    int oct = 0;
                    if (dy < 0) {
                        dx = -dx;
                        dy = -dy;
                        oct += 4;
                    }
                    if (dx < 0) {
                        const int64_t tmp = dx;
                        dx = dy;
                        dy = -tmp;
                        oct += 2;
                    }
                    if (dx < dy) oct += 1;
                    int64_t px, py, qx, qy;
                    oct_to0(oct, sx, sy, px, py);
                    oct_to0(oct, ex, ey, qx, qy);
                    const int64_t Dx = qx - px, Dy = qy - py;
                    const float dt = fdiv(1.0f, (float)Dx);
                    // this thread's run of steps [j0, j1)
                    const int64_t per = (Dx + kLineThreads - 1) / kLineThreads;
                    const int64_t j0 = min(Dx, per * (int64_t)threadIdx.x), j1 = min(Dx, j0 + per);
                    int64_t diff = Dy - Dx;
                    float t = 0.0f;
                    for (int64_t j = 0; j < j0; ++j) {  // replay the state up to the run
                        if (diff >= 0) {
                            py += 1;
                            diff -= Dx;
                        }
                        diff += Dy;
                        t = fadd(t, dt);
                        px += 1;
                    }
                    for (int64_t j = j0; j < j1; ++j) {
                        const int64_t cx = px, cy = py;
                        if (diff >= 0) {
                            py += 1;
                            diff -= Dx;
                        }
                        diff += Dy;
                        const float tt = t;
                        t = fadd(t, dt);
                        px += 1;
                        int64_t ox, oy;
                        oct_from0(oct, cx, cy, ox, oy);
                        if (ox < 0 || oy < 0 || ox > 0xFFFFFFFFll || oy > 0xFFFFFFFFll) continue;
                        const uint32_t x = (uint32_t)ox, y = (uint32_t)oy;
                        if (x < d.sc_x0 || x >= d.sc_x1 || y < d.sc_y0 || y >= d.sc_y1 || x >= tg.width || y >= tg.height)
                            continue;
                        // Lerp(t) of the clip alphas, then of the end points' fragments (raster.rs:248-254)
                        const float T = fadd(fmul(lp.alpha[0], fsub(1.0f, tt)), fmul(lp.alpha[1], tt));
                        const float omT = fsub(1.0f, T);
                        const V4 fragment = v4_add(v4_mul(lp.frag[0], omT), v4_mul(lp.frag[1], T));
                        const float coeff[2] = {omT, T};
                        line_fragment(bp, d, tg, s_rs, s_lut, lp, x, y, fragment, coeff, frag_count, fs_count);
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        frag_count += __shfl_xor_sync(0xFFFFFFFFu, frag_count, o);
        fs_count += __shfl_xor_sync(0xFFFFFFFFu, fs_count, o);
    }
    if ((threadIdx.x & 31) == 0 && frag_count) {
        atomicAdd(&s_frag, (unsigned long long)frag_count);
        if (tg.frag_count) {  // one draw per CTA: its program samples a texture or not
            atomicAdd(tg.frag_count, (unsigned long long)frag_count);
            if (fs_count) atomicAdd(tg.frag_count + 1, (unsigned long long)fs_count);
            if (fs_count && s_rs.tex_data) atomicAdd(tg.frag_count + 2, (unsigned long long)fs_count);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_frag) atomicAdd(&bp.status->fragments, s_frag);
}

}  // namespace gbr
