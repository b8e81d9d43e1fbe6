// raster.cuh — the render-pass kernels.
//
//   k_setup   one thread per primitive: index resolution, vertex fetch + vertex stage for the
//             three corners, TriFace / cull, homogeneous clipping, viewport transform and the
//             per-sub-triangle raster record; counts the screen tiles each record covers.
//   k_scan    exclusive scan of the per-tile counts (bin offsets).
//   k_fill    writes each record's order key into the bins of the tiles it covers.
//   k_raster  persistent: one CTA per (target, tile) work item.  Sorts the tile's keys (the
//             reference order: draw, instance, primitive, sub-triangle), then walks them in
//             order; every thread owns pixels of the tile and keeps their colour and depth in
//             registers, so per-pixel fragment order — and with it depth test, blending and
//             last-writer-wins — is exactly the reference's sequential order.  The pass's
//             LoadOp::Clear is fused into the register initialisation.
//
// Coverage, barycentrics, interpolation, depth and colour encoding restate render_pass/
// raster.rs:129-363, util/scanline.rs:14-198, render_pass/fragment.rs:127-214,427-489 and
// texture.rs:213-239,373-411, operation for operation.
#pragma once

#include "exact.cuh"
#include "gbr_types.h"
#include "programs.cuh"

namespace gbr {

__device__ __forceinline__ TriRecord* rec_at(uint8_t* base, uint32_t stride, uint32_t i) {
    return reinterpret_cast<TriRecord*>(base + (size_t)i * stride);
}
__device__ __forceinline__ float* rec_var(TriRecord* r) { return reinterpret_cast<float*>(r + 1); }
__device__ __forceinline__ const float* rec_var(const TriRecord* r) { return reinterpret_cast<const float*>(r + 1); }

__device__ __forceinline__ void raise_error(BatchStatus* st, uint32_t code, uint32_t detail) {
    if (atomicCAS(&st->error, 0u, code) == 0u) st->error_detail = detail;
}

// The draw of global primitive `prim`: a binary search over the draws' first primitives, in the
// batch's contiguous table when it has one (a few cache lines) or else in the descriptors.
__device__ __forceinline__ uint32_t find_draw(const BatchParams& bp, uint32_t prim) {
    uint32_t lo = 0, hi = bp.num_draws;
    if (bp.draw_base) {
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(bp.draw_base + mid) <= prim) lo = mid; else hi = mid;
        }
    } else {
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(&bp.draws[mid].prim_base) <= prim) lo = mid; else hi = mid;
        }
    }
    return lo;
}
__device__ __forceinline__ uint32_t find_target(const TargetDesc* t, uint32_t n, uint32_t tile) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&t[mid].tile_base) <= tile) lo = mid; else hi = mid;
    }
    return lo;
}

// ------------------------------------------------------------------------- clipping
// tri_clip::Vertex (clipper.rs:590-613): clip position + barycentric w.r.t. the input triangle.
struct CV {
    V4 p;
    float b[3];
};

__device__ __forceinline__ CV cv_lerp(const CV& a, const CV& c, float t) {
    float omt = fsub(1.0f, t);
    CV r;
    r.p = v4_add(v4_mul(a.p, omt), v4_mul(c.p, t));
#pragma unroll
    for (int k = 0; k < 3; ++k) r.b[k] = fadd(fmul(a.b[k], omt), fmul(c.b[k], t));
    return r;
}

__device__ __forceinline__ V4 clip_plane(int i) {
    switch (i) {
        case 0: return {1.0f, 0.0f, 0.0f, 1.0f};
        case 1: return {-1.0f, 0.0f, 0.0f, 1.0f};
        case 2: return {0.0f, 1.0f, 0.0f, 1.0f};
        case 3: return {0.0f, -1.0f, 0.0f, 1.0f};
        case 4: return {0.0f, 0.0f, 1.0f, 0.0f};
        default: return {0.0f, 0.0f, -1.0f, 1.0f};
    }
}

// clip_tri_against_plane (clipper.rs:625-728): same case table, same output vertex orders.
__device__ __forceinline__ int clip_against(const CV v[3], int plane, CV out[2][3]) {
    V4 n = clip_plane(plane);
    float d[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) d[i] = dot4(v[i].p, n);
    bool o0 = d[0] < 0.0f, o1 = d[1] < 0.0f, o2 = d[2] < 0.0f;
    auto clip = [&](int i, int j) { return cv_lerp(v[i], v[j], fdiv(d[i], fsub(d[i], d[j]))); };
    if (o0 && o1 && o2) return 0;
    if (!o0 && !o1 && !o2) {
        out[0][0] = v[0]; out[0][1] = v[1]; out[0][2] = v[2];
        return 1;
    }
    if (o0 && o1 && !o2) {
        CV an = clip(2, 0), bn = clip(1, 2);
        out[0][0] = an; out[0][1] = bn; out[0][2] = v[2];
        return 1;
    }
    if (!o0 && o1 && o2) {
        CV bn = clip(0, 1), cn = clip(2, 0);
        out[0][0] = v[0]; out[0][1] = bn; out[0][2] = cn;
        return 1;
    }
    if (o0 && !o1 && o2) {
        CV an = clip(0, 1), cn = clip(1, 2);
        out[0][0] = an; out[0][1] = v[1]; out[0][2] = cn;
        return 1;
    }
    if (o0 && !o1 && !o2) {
        CV bn = clip(0, 1), cn = clip(0, 2);
        out[0][0] = bn; out[0][1] = v[1]; out[0][2] = cn;
        out[1][0] = v[1]; out[1][1] = v[2]; out[1][2] = cn;
        return 2;
    }
    if (!o0 && o1 && !o2) {
        CV an = clip(0, 1), cn = clip(1, 2);
        out[0][0] = v[0]; out[0][1] = an; out[0][2] = cn;
        out[1][0] = v[0]; out[1][1] = cn; out[1][2] = v[2];
        return 2;
    }
    CV bn = clip(1, 2), an = clip(0, 2);
    out[0][0] = v[0]; out[0][1] = v[1]; out[0][2] = bn;
    out[1][0] = v[0]; out[1][1] = bn; out[1][2] = an;
    return 2;
}

// TriClipper::clip_tri (clipper.rs:756-776) processes the planes breadth first through a FIFO;
// its output order is the lexicographic order of the split paths, which is what this
// depth-first walk (first child first, second child parked on a stack) produces.
template <class Emit>
__device__ __noinline__ void clip_tri_ordered(const V4 pos[3], Emit& emit) {
    struct Entry {
        CV v[3];
        int plane;
    };
    Entry stack[7];
    int sp = 0;
    Entry cur;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        cur.v[i].p = pos[i];
        cur.v[i].b[0] = i == 0 ? 1.0f : 0.0f;
        cur.v[i].b[1] = i == 1 ? 1.0f : 0.0f;
        cur.v[i].b[2] = i == 2 ? 1.0f : 0.0f;
    }
    cur.plane = 0;
    for (;;) {
        bool dropped = false;
        while (cur.plane < 6) {
            CV out[2][3];
            int m = clip_against(cur.v, cur.plane, out);
            if (m == 0) {
                dropped = true;
                break;
            }
            if (m == 2 && sp < 7) {
                stack[sp].v[0] = out[1][0];
                stack[sp].v[1] = out[1][1];
                stack[sp].v[2] = out[1][2];
                stack[sp].plane = cur.plane + 1;
                ++sp;
            }
            cur.v[0] = out[0][0];
            cur.v[1] = out[0][1];
            cur.v[2] = out[0][2];
            cur.plane += 1;
        }
        if (!dropped) emit(cur.v);
        if (sp == 0) break;
        cur = stack[--sp];
    }
}

__device__ __forceinline__ bool inside_all_planes(const V4 pos[3]) {
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        V4 n = clip_plane(p);
#pragma unroll
        for (int i = 0; i < 3; ++i)
            if (dot4(pos[i], n) < 0.0f) return false;
    }
    return true;
}

// ------------------------------------------------------------------------- edge-function rule
// Extension profile, RASTER_RULE_EDGE (no reference counterpart: wgpu-cpu walks scanlines):
// viewport coordinates snap to 1/256 pixel (round to nearest even), a pixel is covered when its
// centre (x + 1/2, y + 1/2) lies inside all three edges, with the top-left rule on edges through
// the centre.  Integer arithmetic throughout (snapped coordinates stay below 2^30, products below
// 2^62), so the oracle reproduces every decision exactly.
__device__ __forceinline__ int64_t floor_div(int64_t a, int64_t b) {  // b > 0
    int64_t q = a / b;
    if ((a % b) != 0 && a < 0) --q;
    return q;
}
__device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return -floor_div(-a, b); }

// Snapped vertices in an order with positive doubled area (X1-X0)(Y2-Y0) - (Y1-Y0)(X2-X0); returns
// that area (0: nothing is covered).
__device__ __forceinline__ int64_t snap_triangle(const float vx[3], const float vy[3], int64_t X[3], int64_t Y[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        X[i] = (int64_t)rintf(fmul(vx[i], 256.0f));
        Y[i] = (int64_t)rintf(fmul(vy[i], 256.0f));
    }
    int64_t a2 = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
    if (a2 < 0) {
        int64_t t = X[1]; X[1] = X[2]; X[2] = t;
        t = Y[1]; Y[1] = Y[2]; Y[2] = t;
        a2 = -a2;
    }
    return a2;
}

// Row y's covered pixels [x1, x2] (empty when x1 > x2): per edge i -> j with d = (dx, dy),
// E(P) = dx (P.y - Y_i) - dy (P.x - X_i) >= 0 on the inside; a top edge (dy == 0, dx > 0) or a
// left edge (dy < 0) also owns the centres exactly on it.  At P.x = 256 x + 128 each edge bounds
// x from one side.  Only the EDGE instantiations of the kernels contain it.
__device__ __forceinline__ void span_edge(const TriRecord& r, int y, int& x1, int& x2) {
    int64_t X[3], Y[3];
    snap_triangle(r.vpx, r.vpy, X, Y);
    const int64_t py = (int64_t)y * 256 + 128;
    int64_t lo = -((int64_t)1 << 30), hi = (int64_t)1 << 30;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int i = e, j = e == 2 ? 0 : e + 1;
        const int64_t dx = X[j] - X[i], dy = Y[j] - Y[i];
        const int64_t bias = (dy < 0 || (dy == 0 && dx > 0)) ? 0 : 1;
        const int64_t a = -256 * dy;
        const int64_t b = -128 * dy + dx * (py - Y[i]) + dy * X[i] - bias;  // a x + b >= 0
        if (a > 0) lo = max(lo, ceil_div(-b, a));
        else if (a < 0) hi = min(hi, floor_div(b, -a));
        else if (b < 0) { lo = 1; hi = 0; }
    }
    const int64_t lim = (int64_t)1 << 30;
    x1 = (int)(lo < -lim ? -lim : lo);
    x2 = (int)(hi > lim ? lim : hi);
}

// ------------------------------------------------------------------------- spans
// The row's inclusive span [x1, x2] of the scanline state machine, in closed form
// (util/scanline.rs:14-146): x1 on edge AC, x2 on AB before row b.y and on BC from row b.y.
// EDGE: the kernels are instantiated for the edge-function rule, whose records all use span_edge
// (a batch's draws share their device's rule).
// The scanline rule's span of row y for the framebuffer vertices a, b, c sorted by y.
__device__ __forceinline__ void span_rows(int ax, int ay, int bx, int by, int cx, int cy, int y, int& x1, int& x2) {
    int64_t i = y - ay;
    int64_t a = ax + div_trunc_span((int64_t)(cx - ax) * i, (int64_t)(cy - ay));
    int64_t b;
    if (y < by) b = ax + div_trunc_span((int64_t)(bx - ax) * i, (int64_t)(by - ay));
    else b = bx + div_trunc_span((int64_t)(cx - bx) * (int64_t)(y - by), (int64_t)(cy - by));
    x1 = (int)(a < b ? a : b);
    x2 = (int)(a < b ? b : a);
}

template <bool EDGE = false>
__device__ __forceinline__ void span_at(const TriRecord& r, int y, int& x1, int& x2) {
    if constexpr (EDGE) {
        span_edge(r, y, x1, x2);
        return;
    }
    if (r.flags & (SPAN_DEGENERATE << 2)) {
        x1 = r.xmin;
        x2 = r.xmax;
        return;
    }
    span_rows(r.sx[0], r.sy[0], r.sx[1], r.sy[1], r.sx[2], r.sy[2], y, x1, x2);
}

// The rows [lo, hi] a record can emit into, clipped to the scissor and the target (lo > hi: none).
__device__ __forceinline__ void record_rows(const TriRecord& r, const DrawDesc& d, const TargetDesc& t, int& lo, int& hi) {
    lo = max(r.row0, (int)d.sc_y0);
    hi = min(r.row1, min((int)d.sc_y1 - 1, (int)t.height - 1));
}

// Tiles of the record's unclipped bounding box (an upper bound of the tiles it emits into).
__device__ __forceinline__ uint32_t bbox_tiles(const TriRecord& r, uint32_t shift) {
    return (uint32_t)((r.row1 >> shift) - (r.row0 >> shift) + 1) * (uint32_t)((r.xmax >> shift) - (r.xmin >> shift) + 1);
}

// The tile columns [c0, c1] of tile row ty (within rows [lo, hi]) the record can emit into: the
// spans at the row band's ends and around the middle vertex bound the band's pixels (c0 > c1: none).
// A record whose bounding box spans at most eight tiles takes the box's columns instead, without
// evaluating spans: binning it into a tile it misses costs the raster one empty visit, and every
// walker (counting and filling alike) goes through here, so the tile set stays the same.
template <bool EDGE>
__device__ __forceinline__ void tile_row_cols(const TriRecord& r, const DrawDesc& d, const TargetDesc& t, uint32_t shift,
                                              int lo, int hi, int ty, int& c0, int& c1) {
    if (bbox_tiles(r, shift) <= 8u) {
        const int mn = max(r.xmin, (int)d.sc_x0), mx = min(r.xmax, min((int)d.sc_x1 - 1, (int)t.width - 1));
        c0 = mn > mx ? 1 : mn >> shift;
        c1 = mn > mx ? 0 : mx >> shift;
        return;
    }
    const int T = 1 << shift;
    const int y0 = max(lo, ty << shift), y1 = min(hi, (ty << shift) + T - 1);
    int xa, xb, mn, mx;
    span_at<EDGE>(r, y0, xa, xb);
    mn = xa; mx = xb;
    span_at<EDGE>(r, y1, xa, xb);
    mn = min(mn, xa); mx = max(mx, xb);
    const int by = r.sy[1];
    if (by - 1 >= y0 && by - 1 <= y1) {
        span_at<EDGE>(r, by - 1, xa, xb);
        mn = min(mn, xa); mx = max(mx, xb);
    }
    if (by >= y0 && by <= y1) {
        span_at<EDGE>(r, by, xa, xb);
        mn = min(mn, xa); mx = max(mx, xb);
    }
    mn = max(mn, (int)d.sc_x0);
    mx = min(mx, min((int)d.sc_x1 - 1, (int)t.width - 1));
    c0 = mn > mx ? 1 : mn >> shift;
    c1 = mn > mx ? 0 : mx >> shift;
}

// Calls f(tile_index_in_target) for every tile whose pixels the record can emit.
// Tile rows are visited from `first` in steps of `step` (1, or 32 when a warp shares a record).
template <bool EDGE, class F>
__device__ __forceinline__ void for_each_tile(const TriRecord& r, const DrawDesc& d, const TargetDesc& t, uint32_t shift,
                                              F&& f, int first = 0, int step = 1) {
    int lo, hi;
    record_rows(r, d, t, lo, hi);
    if (lo > hi) return;
    for (int ty = (lo >> shift) + first; ty <= (hi >> shift); ty += step) {
        int c0, c1;
        tile_row_cols<EDGE>(r, d, t, shift, lo, hi, ty, c0, c1);
        for (int tx = c0; tx <= c1; ++tx) f((uint32_t)ty * t.tiles_x + (uint32_t)tx);
    }
}

// ------------------------------------------------------------------------- setup
// to_raster (raster.rs:145-160)
__device__ __forceinline__ bool to_raster(const DrawDesc& d, V4 c, uint32_t& fbx, uint32_t& fby, V4& frag) {
    if (c.w == 0.0f) return false;
    float nx = fdiv(c.x, c.w), ny = fdiv(c.y, c.w), nz = fdiv(c.z, c.w);
    float pd = fdiv(1.0f, c.w);
    float vx = rust_max0(fadd(fmul(nx, d.vp_sx), d.vp_tx));
    float vy = rust_max0(fadd(fmul(ny, d.vp_sy), d.vp_ty));
    fbx = rust_f2u32(vx);
    fby = rust_f2u32(vy);
    frag = {vx, vy, nz, pd};
    return true;
}

// Index resolution (render_pass/index.rs:45-88) for stream position k of a draw.
__device__ __forceinline__ bool resolve_vertex(const DrawDesc& d, uint32_t k, uint32_t& vertex, uint32_t* err) {
    uint32_t pos = d.first + k;
    if (d.index_format == 0) {
        vertex = pos;
        return true;
    }
    uint32_t raw;
    if (d.index_format == 1) {
        if ((uint64_t)(pos + 1) * 2 > d.index_bytes) { *err = ERR_INDEX_OOB; return false; }
        raw = __ldg(reinterpret_cast<const uint16_t*>(d.index_data) + pos);
    } else {
        if ((uint64_t)(pos + 1) * 4 > d.index_bytes) { *err = ERR_INDEX_OOB; return false; }
        raw = __ldg(reinterpret_cast<const uint32_t*>(d.index_data) + pos);
    }
    int64_t v = (int64_t)raw + (int64_t)d.base_vertex;  // u32::strict_add_signed
    if (v < 0 || v > 0xFFFFFFFFll) { *err = ERR_BASE_VERTEX; return false; }
    vertex = (uint32_t)v;
    return true;
}

// Fills one sub-triangle record from its vertices' framebuffer coordinates and to_raster
// outputs (viewport x, y, ndc z, 1/w); var holds up to NVMAX varyings per vertex.
// Extension-profile texture LOD of a finished record: screen-space derivatives of the draw's
// (u, v) varyings (u at varying index q) from the record's viewport vertices, area and clip
// barycentrics.  Kept out of line: only extension-profile textured draws call it, and the setup
// kernels' register budget stays with the common path.
static __device__ __noinline__ void record_lod(const DrawDesc& dd, uint32_t q, uint32_t nvar, TriRecord* r) {
    float dcx[3], dcy[3];
    bary_gradients(r->vpx, r->vpy, r->area, r->cb, dcx, dcy);
    const float* rv = rec_var(r);
    auto dvar = [&](uint32_t c, const float* dc) {
        return fadd(fadd(fmul(rv[q + c], dc[0]), fmul(rv[nvar + q + c], dc[1])), fmul(rv[2 * nvar + q + c], dc[2]));
    };
    r->lod = lod_from_grad(dvar(0, dcx), dvar(1, dcx), dvar(0, dcy), dvar(1, dcy), dd.tex.width, dd.tex.height,
                           dd.samp.lod_min, dd.samp.lod_max);
}

// The record header as eleven 16-byte words, in the order build_record_frag stores them.
#ifndef __CUDACC_RTC__  // (offsetof needs <cstddef>; the layout is the same under NVRTC)
static_assert(offsetof(TriRecord, row0) == 16 && offsetof(TriRecord, sx) == 32 && offsetof(TriRecord, sy) == 44 &&
                  offsetof(TriRecord, vpx) == 56 && offsetof(TriRecord, vpy) == 68 && offsetof(TriRecord, area) == 80 &&
                  offsetof(TriRecord, fz) == 84 && offsetof(TriRecord, fw) == 96 && offsetof(TriRecord, cb) == 108 &&
                  offsetof(TriRecord, inv_w0) == 144 && offsetof(TriRecord, ovf) == 156 &&
                  offsetof(TriRecord, nsub) == 160 && offsetof(TriRecord, lod) == 164 && sizeof(TriRecord) == 176,
              "TriRecord layout assumed by build_record_frag");
static_assert(offsetof(DrawDesc, sc_x0) % 8 == 0 && offsetof(DrawDesc, sc_y1) == offsetof(DrawDesc, sc_x0) + 12 &&
                  sizeof(DrawDesc) % 16 == 0,
              "DrawDesc scissor read as two 8-byte words by k_raster_vis");
#endif

// Writes a complete record (nsub = 1, ovf = 0; callers that emit more sub-triangles overwrite
// both).  `r` is 16-byte aligned (records, overflow records and the setup stage all are): the
// header goes out as eleven 16-byte stores, which a warp whose lanes write records 240 bytes
// apart in shared memory issues without bank conflicts (scalar stores there conflict 4 ways).
template <uint32_t NVMAX, bool EDGE>
__device__ __forceinline__ void build_record_frag(const BatchParams& bp, TriRecord* r, uint32_t key, uint32_t draw,
                                                  uint32_t prim_index, bool front_facing, const CV v[3],
                                                  const uint32_t fbx[3], const uint32_t fby[3], const V4 frag[3],
                                                  const float inv_w0[3], const float (*var)[NVMAX], uint32_t nvar) {
    float area = shoelace(frag[0].x, frag[0].y, frag[1].x, frag[1].y, frag[2].x, frag[2].y);
    // scanlines(): sort the framebuffer vertices by y with bubblesort3 (util/sort.rs:3-8)
    uint32_t px[3] = {fbx[0], fbx[1], fbx[2]}, py[3] = {fby[0], fby[1], fby[2]};
    auto cas = [&](int l, int rr) {
        if (py[l] > py[rr]) {
            uint32_t tx = px[l], tyy = py[l];
            px[l] = px[rr]; py[l] = py[rr];
            px[rr] = tx; py[rr] = tyy;
        }
    };
    cas(0, 1);
    cas(0, 2);
    cas(1, 2);
    uint32_t flags = front_facing ? 1u : 0u;
    int row0, row1, xmin, xmax;
    int sxv[3], syv[3];
    const DrawDesc& dd = bp.draws[draw];
    if constexpr (EDGE) {
        // rows whose centres lie within the snapped y extent, columns likewise; the span of each
        // row comes from span_edge, and sy[1] is the first row past the middle vertex (where a
        // span bound changes edge), which the tile and block range helpers sample
        flags |= SPAN_EDGE << 2;
        bool ok = true;
#pragma unroll
        for (int i = 0; i < 3; ++i)
            ok = ok && fabsf(frag[i].x) < 4194304.0f && fabsf(frag[i].y) < 4194304.0f;  // 2^22 px
        int sy1 = 0;
        if (!ok) {
            raise_error(bp.status, ERR_SPAN_RANGE, key);
            flags |= 2u;
            row0 = 1; row1 = 0;
            xmin = 1; xmax = 0;
        } else {
            const float vx[3] = {frag[0].x, frag[1].x, frag[2].x}, vy[3] = {frag[0].y, frag[1].y, frag[2].y};
            int64_t X[3], Y[3];
            if (snap_triangle(vx, vy, X, Y) == 0 || area == 0.0f) flags |= 2u;
            const int64_t ylo = min(Y[0], min(Y[1], Y[2])), yhi = max(Y[0], max(Y[1], Y[2]));
            const int64_t ymid = Y[0] + Y[1] + Y[2] - ylo - yhi;
            const int64_t xlo = min(X[0], min(X[1], X[2])), xhi = max(X[0], max(X[1], X[2]));
            row0 = (int)ceil_div(ylo - 128, 256);
            row1 = (int)floor_div(yhi - 128, 256);
            xmin = (int)ceil_div(xlo - 128, 256);
            xmax = (int)floor_div(xhi - 128, 256);
            sy1 = (int)floor_div(ymid - 128, 256) + 1;
            if (row0 > row1 || xmin > xmax) flags |= 2u;
        }
        sxv[0] = sxv[1] = sxv[2] = 0;
        syv[0] = 0;
        syv[1] = sy1;
        syv[2] = 0;
    } else {
        const uint32_t lim = 1u << 30;
        if (px[0] >= lim || px[1] >= lim || px[2] >= lim || py[2] >= lim) {
            raise_error(bp.status, ERR_SPAN_RANGE, key);
            flags |= 2u;
        }
        if (area == 0.0f) flags |= 2u;  // raster.rs:308-311: no fragments
        row0 = (int)py[0];
        if (py[2] == py[0]) {
            flags |= SPAN_DEGENERATE << 2;
            row1 = row0;
        } else if (py[1] == py[0]) {
            row1 = (int)py[2];
        } else if (py[2] == py[1]) {
            row1 = (int)py[1] - 1;  // the state machine stops before row c.y (scanline.rs:114-121)
        } else {
            row1 = (int)py[2];
        }
        xmin = (int)min(px[0], min(px[1], px[2]));
        xmax = (int)max(px[0], max(px[1], px[2]));
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            sxv[i] = (int)px[i];
            syv[i] = (int)py[i];
        }
    }
    // bit 4: the clip barycentrics are exactly the unit vectors, bit for bit (+0, no -0: an
    // unclipped triangle)
    {
        bool ident = true;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) ident = ident && __float_as_uint(v[i].b[j]) == (i == j ? 0x3F800000u : 0u);
        if (ident) flags |= 16u;
    }
    auto fb = [](float x) { return __float_as_uint(x); };
    auto ib = [](int x) { return (uint32_t)x; };
    uint4* h = reinterpret_cast<uint4*>(r);
    h[0] = make_uint4(key, draw, prim_index, flags);
    h[1] = make_uint4(ib(row0), ib(row1), ib(xmin), ib(xmax));
    h[2] = make_uint4(ib(sxv[0]), ib(sxv[1]), ib(sxv[2]), ib(syv[0]));
    h[3] = make_uint4(ib(syv[1]), ib(syv[2]), fb(frag[0].x), fb(frag[1].x));
    h[4] = make_uint4(fb(frag[2].x), fb(frag[0].y), fb(frag[1].y), fb(frag[2].y));
    h[5] = make_uint4(fb(area), fb(frag[0].z), fb(frag[1].z), fb(frag[2].z));
    h[6] = make_uint4(fb(frag[0].w), fb(frag[1].w), fb(frag[2].w), fb(v[0].b[0]));
    h[7] = make_uint4(fb(v[0].b[1]), fb(v[0].b[2]), fb(v[1].b[0]), fb(v[1].b[1]));
    h[8] = make_uint4(fb(v[1].b[2]), fb(v[2].b[0]), fb(v[2].b[1]), fb(v[2].b[2]));
    h[9] = make_uint4(fb(inv_w0[0]), fb(inv_w0[1]), fb(inv_w0[2]), 0u);  // ovf
    h[10] = make_uint4(1u, fb(0.0f), 0u, 0u);                          // nsub, lod, padding
    float* rv = rec_var(r);
    if (nvar == NVMAX) {
        // all of the draw's varyings (a compile-time count on the fast path): 16-byte stores
        constexpr uint32_t NF = 3 * NVMAX;
        uint32_t flat[NF];
#pragma unroll
        for (uint32_t q = 0; q < NF; ++q) flat[q] = fb(var[q / NVMAX][q % NVMAX]);
        uint4* hv = reinterpret_cast<uint4*>(rv);
#pragma unroll
        for (uint32_t q = 0; q + 4 <= NF; q += 4) hv[q / 4] = make_uint4(flat[q], flat[q + 1], flat[q + 2], flat[q + 3]);
        uint32_t* tail = reinterpret_cast<uint32_t*>(rv);
#pragma unroll
        for (uint32_t q = NF & ~3u; q < NF; ++q) tail[q] = flat[q];
    } else {
#pragma unroll
        for (uint32_t q = 0; q < 3; ++q)
#pragma unroll
            for (uint32_t k = 0; k < NVMAX; ++k)
                if (k < nvar) rv[q * nvar + k] = var[q][k];
    }
    if (dd.lod_var != 0 && !(flags & 2u)) record_lod(dd, dd.lod_var - 1, nvar, r);
}

// Fills one sub-triangle record; returns false for a w == 0 vertex.
template <bool EDGE>
__device__ __forceinline__ bool build_record(const BatchParams& bp, const DrawDesc& d, TriRecord* r, uint32_t key,
                                             uint32_t draw, uint32_t prim_index, bool front_facing, const CV v[3],
                                             const float inv_w0[3], const float var[3][MAX_VARYING_FLOATS],
                                             uint32_t nvar) {
    uint32_t fbx[3], fby[3];
    V4 frag[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        if (!to_raster(d, v[i].p, fbx[i], fby[i], frag[i])) return false;
    build_record_frag<MAX_VARYING_FLOATS, EDGE>(bp, r, key, draw, prim_index, front_facing, v, fbx, fby, frag, inv_w0, var,
                                          nvar);
    return true;
}

// The one tile a record can emit into, when its bounding box lies inside a single tile and
// inside the draw's scissor and the target (then every row's span, which lies within the box,
// is wholly visible there: for_each_tile would visit exactly this tile).
__device__ __forceinline__ bool single_tile(const TriRecord& r, const DrawDesc& d, const TargetDesc& t, uint32_t shift,
                                            uint32_t& lt) {
    if ((r.xmin >> shift) != (r.xmax >> shift) || (r.row0 >> shift) != (r.row1 >> shift)) return false;
    if (r.xmin < (int)d.sc_x0 || r.row0 < (int)d.sc_y0 || r.xmax >= (int)min(d.sc_x1, t.width) ||
        r.row1 >= (int)min(d.sc_y1, t.height))
        return false;
    lt = (uint32_t)(r.row0 >> shift) * t.tiles_x + (uint32_t)(r.xmin >> shift);
    return true;
}

template <bool EDGE>
__device__ __forceinline__ void count_tiles(const BatchParams& bp, const TriRecord* r, const DrawDesc& d) {
    if (r->flags & 2u) return;
    const TargetDesc& t = bp.targets[d.target];
    uint32_t base = t.tile_base, one;
    if (single_tile(*r, d, t, bp.tile_shift, one)) {
        atomicAdd(&bp.tile_count[base + one], 1u);
        return;
    }
    for_each_tile<EDGE>(*r, d, t, bp.tile_shift, [&](uint32_t lt) { atomicAdd(&bp.tile_count[base + lt], 1u); });
}

// A record spanning more than two tile rows is handed to the whole warp, whose lanes take its
// tile rows in turn, so a large triangle does not serialise its thousands of tiles on one lane.
__device__ __forceinline__ bool tiles_are_many(const TriRecord& r, uint32_t shift) {
    return (r.row1 >> shift) - (r.row0 >> shift) >= 2;
}
// Binning hint of a primary record, written by the fast setup so that k_fill need not read the
// record back: the record covers nothing, exactly one tile (its global index), or anything else.
enum : uint32_t { TILE_HINT_EMPTY = 0xFFFFFFFEu, TILE_HINT_WALK = 0xFFFFFFFFu };
__device__ __forceinline__ uint32_t tile_hint_of(const BatchParams& bp, const TriRecord& r, const DrawDesc& d,
                                                 const TargetDesc& t) {
    if (r.flags & 2u) return TILE_HINT_EMPTY;
    uint32_t one;
    if (!tiles_are_many(r, bp.tile_shift) && single_tile(r, d, t, bp.tile_shift, one)) return t.tile_base + one;
    return TILE_HINT_WALK;
}
template <bool EDGE, class F>
__device__ __forceinline__ void coop_tiles(const BatchParams& bp, const TriRecord* mine, uint32_t lane, F&& f) {
    uint32_t todo = __ballot_sync(0xFFFFFFFFu, mine != nullptr);
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        __syncwarp();  // the record was written by lane `src`
        const TriRecord* r = reinterpret_cast<const TriRecord*>(
            __shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(mine), src));
        const DrawDesc& d = bp.draws[r->draw];
        const TargetDesc& t = bp.targets[d.target];
        const uint32_t key = r->key;
        for_each_tile<EDGE>(*r, d, t, bp.tile_shift, [&](uint32_t lt) { f(t.tile_base + lt, key); }, (int)lane, 32);
    }
}

// The tiles of the lanes' records (mine, or null) walked by the whole warp, one record at a time,
// in row-major order 32 tiles per pass: the column ranges of up to 32 tile rows are computed one
// row per lane, a warp scan numbers the rows' tiles, and each lane finds the row of its tile by a
// shuffle search — the tiles for_each_tile visits, for records wide or tall alike.
template <bool EDGE, class F>
__device__ __forceinline__ void coop_tiles_flat(const BatchParams& bp, const TriRecord* mine, uint32_t lane, F&& f) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    uint32_t todo = __ballot_sync(kFull, mine != nullptr);
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        __syncwarp();  // the record was written by lane `src`
        const TriRecord* r = reinterpret_cast<const TriRecord*>(
            __shfl_sync(kFull, reinterpret_cast<unsigned long long>(mine), src));
        const DrawDesc& d = bp.draws[r->draw];
        const TargetDesc& t = bp.targets[d.target];
        const uint32_t key = r->key;
        int lo, hi;
        record_rows(*r, d, t, lo, hi);
        if (lo > hi) continue;  // warp-uniform
        const int ty_hi = hi >> bp.tile_shift;
        for (int base = lo >> bp.tile_shift; base <= ty_hi; base += 32) {
            const int ty = base + (int)lane;
            int c0 = 1, c1 = 0;
            if (ty <= ty_hi) tile_row_cols<EDGE>(*r, d, t, bp.tile_shift, lo, hi, ty, c0, c1);
            const uint32_t n = c1 >= c0 ? (uint32_t)(c1 - c0 + 1) : 0u;
            uint32_t incl = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(kFull, incl, o);
                if (lane >= (uint32_t)o) incl += v;
            }
            const uint32_t total = __shfl_sync(kFull, incl, 31), excl = incl - n;
            for (uint32_t k0 = 0; k0 < total; k0 += 32) {  // warp-uniform
                const uint32_t k = k0 + lane;
                int row = 0;  // the last lane whose first tile number is <= k (it has tiles)
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(kFull, excl, row + step) <= k) row += step;
                const int rc0 = __shfl_sync(kFull, c0, row);
                const uint32_t rexcl = __shfl_sync(kFull, excl, row);
                if (k < total)
                    f(t.tile_base + (uint32_t)(base + row) * t.tiles_x + (uint32_t)rc0 + (k - rexcl), key);
            }
        }
    }
}

// ---- strips with primitive restart (render_pass/primitive.rs:428-487, index.rs:90-106)
// Each run of indices between separators is a strip of its own: the triangle completed at stream
// position k (at least two positions into its run) is (k-2, k-1, k) or, when k - run_start is
// odd, (k-1, k-2, k).  k_strip_table writes for every position of a restart draw
//   (compact primitive index << 1) | parity, or ~0 when k completes no triangle,
// scanning the index stream once (separator positions by a max-scan, completed triangles by a
// sum-scan), one CTA per draw.  Setup reads it for primitive slot k - 2.
constexpr uint32_t kNoStripTri = 0xFFFFFFFFu;

// (a template only so that both kernel translation units can instantiate it)
template <int = 0>
__global__ void __launch_bounds__(1024) k_strip_table(BatchParams bp) {
    const DrawDesc& d = bp.draws[blockIdx.x];
    if (!d.strip_restart) return;
    __shared__ int s_wmax[32];
    __shared__ uint32_t s_wsum[32];
    __shared__ int s_carry_max;
    __shared__ uint32_t s_carry_sum;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) {
        s_carry_max = -1;  // last separator position so far
        s_carry_sum = 0;   // triangles so far
    }
    __syncthreads();
    const uint32_t n = d.count;
    const bool u16 = d.index_format == 1;
    const uint32_t isz = u16 ? 2u : 4u;
    for (uint32_t base = 0; base < n; base += 1024) {
        const uint32_t k = base + tid;
        bool sep = false, valid = k < n;
        if (valid) {
            const uint32_t at = d.first + k;
            if ((uint64_t)(at + 1) * isz <= d.index_bytes) {
                sep = u16 ? __ldg(reinterpret_cast<const uint16_t*>(d.index_data) + at) == 0xFFFFu
                          : __ldg(reinterpret_cast<const uint32_t*>(d.index_data) + at) == 0xFFFFFFFFu;
            }
        }
        // inclusive max-scan of separator positions
        int m = sep ? (int)k : -1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, m, o);
            if (lane >= o) m = max(m, y);
        }
        if (lane == 31) s_wmax[wid] = m;
        __syncthreads();
        if (wid == 0) {
            int w = s_wmax[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w = max(w, y);
            }
            s_wmax[lane] = w;
        }
        __syncthreads();
        const int last_sep = max(max(m, wid ? s_wmax[wid - 1] : -1), s_carry_max);
        const int run_start = last_sep + 1;
        const bool tri = valid && !sep && (int)k - run_start >= 2;
        // exclusive sum-scan of completed triangles
        uint32_t c = tri ? 1u : 0u, x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_wsum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = s_wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w += y;
            }
            s_wsum[lane] = w;
        }
        __syncthreads();
        const uint32_t before = s_carry_sum + (wid ? s_wsum[wid - 1] : 0u) + x - c;
        if (valid)
            bp.strip_info[d.strip_table + k] = tri ? ((before << 1) | (uint32_t)(((int)k - run_start) & 1)) : kNoStripTri;
        __syncthreads();
        if (tid == 1023) {
            s_carry_max = max(s_carry_max, s_wmax[31]);
            s_carry_sum = before + c;
        }
        __syncthreads();
    }
}

// ---- generic setup: any program, format, topology; clipping; error reporting
// Sets up primitive gp of draw di (record written in place); a record spanning many tile rows
// is returned in `coop` for the warp to count together.
template <bool EDGE>
__device__ __forceinline__ void setup_generic(const BatchParams& bp, uint32_t gp, const TriRecord*& coop) {
    if (bp.tile_hint) bp.tile_hint[gp] = TILE_HINT_WALK;  // k_fill reads the generic path's records
    TriRecord* prim_rec = rec_at(bp.records, bp.record_stride, gp);
    const uint32_t di = find_draw(bp, gp);
    const DrawDesc& d = bp.draws[di];
    const uint32_t local = gp - d.prim_base;
    const uint32_t inst = local / d.prims_per_instance;
    const uint32_t p = local - inst * d.prims_per_instance;
    const uint32_t instance = d.instance_start + inst;
    prim_rec->key = gp << SUBTRI_BITS;
    prim_rec->flags = 2u;
    prim_rec->nsub = 0;
    prim_rec->draw = di;
    uint32_t sp[3];
    uint32_t prim_index = p;  // @builtin(primitive_index)
    if (d.strip_restart) {
        // slot p is stream position p + 2 (strip table above)
        const uint32_t info = bp.strip_info[d.strip_table + p + 2];
        if (info == kNoStripTri) return;  // no triangle ends here: the record stays empty
        const uint32_t k = p + 2;
        sp[0] = (info & 1u) ? k - 1 : k - 2;
        sp[1] = (info & 1u) ? k - 2 : k - 1;
        sp[2] = k;
        prim_index = info >> 1;
    } else if (d.topology == 4) {  // triangle strip (primitive.rs:360-392)
        sp[0] = (p & 1u) ? p + 1 : p;
        sp[1] = (p & 1u) ? p : p + 1;
        sp[2] = p + 2;
    } else {
        sp[0] = 3 * p;
        sp[1] = 3 * p + 1;
        sp[2] = 3 * p + 2;
    }
    V4 pos[3];
    float var[3][MAX_VARYING_FLOATS];
    uint32_t err = 0;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        uint32_t vertex = 0;
        ok = ok && resolve_vertex(d, sp[k], vertex, &err) && run_vs(d, nullptr, vertex, instance, pos[k], var[k], &err);
    }
    if (!ok) {
        raise_error(bp.status, err, gp);
        return;
    }
    if (!d.has_fragment) return;
    // TriFace (primitive.rs:169-197) and the cull decision (state.rs:542-561)
    if (pos[0].w == 0.0f || pos[1].w == 0.0f || pos[2].w == 0.0f) {
        raise_error(bp.status, ERR_W_ZERO, gp);
        return;
    }
    float n[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        n[i][0] = fdiv(pos[i].x, pos[i].w);
        n[i][1] = fdiv(pos[i].y, pos[i].w);
    }
    float abx = fsub(n[1][0], n[0][0]), aby = fsub(n[1][1], n[0][1]);
    float acx = fsub(n[2][0], n[0][0]), acy = fsub(n[2][1], n[0][1]);
    bool ccw = fsub(fmul(abx, acy), fmul(aby, acx)) > 0.0f;
    bool front_facing = (ccw ? 0u : 1u) == d.front_face;
    bool cull = d.cull_mode == 1 ? front_facing : d.cull_mode == 2 ? !front_facing : false;
    if (cull) return;
    const float inv_w0[3] = {fdiv(1.0f, pos[0].w), fdiv(1.0f, pos[1].w), fdiv(1.0f, pos[2].w)};
    const uint32_t nvar = d.num_varyings;
    if (inside_all_planes(pos)) {
        CV v[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            v[i].p = pos[i];
            v[i].b[0] = i == 0 ? 1.0f : 0.0f;
            v[i].b[1] = i == 1 ? 1.0f : 0.0f;
            v[i].b[2] = i == 2 ? 1.0f : 0.0f;
        }
        if (!build_record<EDGE>(bp, d, prim_rec, gp << SUBTRI_BITS, di, prim_index, front_facing, v, inv_w0, var, nvar)) {
            raise_error(bp.status, ERR_W_ZERO, gp);
            prim_rec->flags = 2u;
            return;
        }
        prim_rec->nsub = 1;
        prim_rec->ovf = 0;
        if (!(prim_rec->flags & 2u) && tiles_are_many(*prim_rec, bp.tile_shift)) coop = prim_rec;
        else count_tiles<EDGE>(bp, prim_rec, d);
        return;
    }
    // clipped: count the sub-triangles, reserve overflow slots, then emit in order
    struct Counter {
        uint32_t n;
        __device__ void operator()(const CV*) { ++n; }
    } counter{0};
    clip_tri_ordered(pos, counter);
    const uint32_t nsub = counter.n;
    uint32_t ovf = 0;
    if (nsub > 1) {
        ovf = atomicAdd(&bp.status->ovf_used, nsub - 1);
        if (ovf + nsub - 1 > bp.ovf_capacity) {
            raise_error(bp.status, ERR_OVERFLOW_RECORDS, gp);
            return;
        }
    }
    struct Emitter {
        const BatchParams* bp;
        const DrawDesc* d;
        TriRecord* prim_rec;
        uint32_t gp, di, p, ovf, s;
        bool ff;
        const float* inv_w0;
        const float (*var)[MAX_VARYING_FLOATS];
        uint32_t nvar;
        __device__ void operator()(const CV* v) {
            TriRecord* r = s == 0 ? prim_rec : rec_at(bp->ovf_records, bp->record_stride, ovf + s - 1);
            if (!build_record<EDGE>(*bp, *d, r, (gp << SUBTRI_BITS) | s, di, p, ff, v, inv_w0, var, nvar)) {
                raise_error(bp->status, ERR_W_ZERO, gp);
                r->flags = 2u;
            } else {
                count_tiles<EDGE>(*bp, r, *d);
            }
            ++s;
        }
    };
    Emitter emitter{&bp, &d, prim_rec, gp, di, prim_index, ovf, 0, front_facing, inv_w0, var, nvar};
    clip_tri_ordered(pos, emitter);
    if (nsub == 0) prim_rec->flags = 2u;
    prim_rec->nsub = nsub;
    prim_rec->ovf = ovf;
}

// The primitives the fast kernel queued, one lane each.
template <bool EDGE>
__global__ void __launch_bounds__(128) k_setup_slow(BatchParams bp) {
    const uint32_t n = bp.status->slow_count;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31;
    if (bp.slow_builds_states) {
        // the visibility raster's per-draw states (k_build_states' work), by the grid's last
        // threads, which the queued primitives reach last if at all
        RasterState* states = static_cast<RasterState*>(bp.states);
        const uint32_t rt = stride - 1 - (blockIdx.x * blockDim.x + threadIdx.x);
        for (uint32_t i = rt; i < bp.num_draws; i += stride) build_raster_state(bp.draws[i], i, states[i]);
    }
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        if (*bp.abort_flag) return;  // written only by earlier kernels: uniform across the warp
        const TriRecord* coop = nullptr;
        if (base + lane < n) setup_generic<EDGE>(bp, bp.slow_prims[base + lane], coop);
        coop_tiles<EDGE>(bp, coop, lane, [&](uint32_t tile, uint32_t) { atomicAdd(&bp.tile_count[tile], 1u); });
    }
}

// ---- fast setup
// A warp's copy of the draw all its lanes work on, with the mesh programs' matrix.
struct alignas(16) DrawCache {
    DrawDesc d;
    float mvp[16];
    TargetDesc t;  // the draw's target
    uint32_t id;   // draw index, ~0 = empty
    uint32_t _pad[3];
};
static_assert(sizeof(DrawDesc) % 16 == 0 && sizeof(TargetDesc) % 8 == 0 && sizeof(TargetDesc) / 8 <= 16,
              "DrawCache is filled with 16-byte descriptor and 8-byte target loads");

constexpr int kSetupWarps = 4;

// Bulk copies shared -> global (the copy engine behind cp.async.bulk): both addresses 16-byte
// aligned, the size a multiple of 16.  The issuing thread commits each copy as its own bulk group
// and waits for its groups itself.
__device__ __forceinline__ void bulk_store_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(ssrc);
    asm volatile(
        "cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n\t"
        "cp.async.bulk.commit_group;" ::"l"(gdst),
        "r"(s), "r"(bytes)
        : "memory");
}
// the issuing thread's bulk copies have read their shared-memory source
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the issuing thread's bulk copies are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// orders this thread's shared-memory writes before later bulk copies that read them
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared memory of k_setup beyond its static part: each warp stages its 32 primary records.
__host__ __device__ __forceinline__ size_t setup_stage_bytes(uint32_t record_stride) {
    return (size_t)kSetupWarps * 32 * record_stride;
}

template <int C>
__device__ __forceinline__ void fetch_f32_unchecked(const DrawDesc& d, int loc, uint32_t vertex, uint32_t instance,
                                                    float* out) {
    const int b = d.attr[loc].buffer;
    const uint64_t start = (uint64_t)instance * d.vb_stride_instance[b] + (uint64_t)vertex * d.vb_stride_vertex[b] +
                           d.attr[loc].offset;
    const float* f = reinterpret_cast<const float*>(d.vb_data[b] + start);
#pragma unroll
    for (int k = 0; k < C; ++k) out[k] = __ldg(f + k);
}

__host__ __device__ constexpr uint32_t fast_vs_varyings(int fvs) {
    return fvs == FAST_VS_MVP_COLOR ? 3u : fvs == FAST_VS_MVP_TEX ? 5u : 4u;
}

// Whether every attribute fetch of one FastVs vertex stays inside its vertex buffer.
__device__ __forceinline__ bool attr_in_range(const DrawDesc& d, int loc, uint32_t vertex, uint32_t instance,
                                              uint32_t bytes) {
    const int b = d.attr[loc].buffer;
    return (uint64_t)instance * d.vb_stride_instance[b] + (uint64_t)vertex * d.vb_stride_vertex[b] + d.attr[loc].offset +
               bytes <= d.vb_size[b];
}
template <int FVS>
__device__ __forceinline__ bool fast_vertex_in_range(const DrawDesc& d, uint32_t vertex, uint32_t instance) {
    if constexpr (FVS == FAST_VS_MVP_COLOR)
        return attr_in_range(d, 0, vertex, instance, 12) && attr_in_range(d, 1, vertex, instance, 12);
    else if constexpr (FVS == FAST_VS_MVP_TEX)
        return attr_in_range(d, 0, vertex, instance, 12) && attr_in_range(d, 1, vertex, instance, 12) &&
               attr_in_range(d, 2, vertex, instance, 8);
    else if constexpr (FVS == FAST_VS_QUAD)
        return attr_in_range(d, 0, vertex, instance, 12) && attr_in_range(d, 1, vertex, instance, 16);
    else if constexpr (FVS == FAST_VS_QUAD_F16)
        return attr_in_range(d, 0, vertex, instance, 12) && attr_in_range(d, 1, vertex, instance, 8);
    else if constexpr (FVS == FAST_VS_CLIP)
        return attr_in_range(d, 0, vertex, instance, 16) && attr_in_range(d, 1, vertex, instance, 16);
    else
        return true;
}

// The vertex stage of run_vs for one FastVs shape (same operations), for a vertex whose fetches
// fast_vertex_in_range has checked: no branch stands between the loads of a primitive's three
// vertices, so they are all in flight together.
template <int FVS>
__device__ __forceinline__ void fast_vertex(const DrawDesc& d, const float* mvp, uint32_t vertex, uint32_t instance,
                                            V4& pos, float* var) {
    float a0[4], a1[4], a2[2];
    if constexpr (FVS == FAST_VS_MVP_COLOR || FVS == FAST_VS_MVP_TEX) {
        if (d.fast_packed) {  // the whole vertex: two 16-byte (textured) or three 8-byte loads
            const uint8_t* vp = d.vb_data[d.attr[0].buffer] + (uint64_t)vertex * (FVS == FAST_VS_MVP_TEX ? 32u : 24u);
            if constexpr (FVS == FAST_VS_MVP_TEX) {
                const uint4 w0 = __ldg(reinterpret_cast<const uint4*>(vp)), w1 = __ldg(reinterpret_cast<const uint4*>(vp) + 1);
                a0[0] = __uint_as_float(w0.x); a0[1] = __uint_as_float(w0.y); a0[2] = __uint_as_float(w0.z);
                a1[0] = __uint_as_float(w0.w); a1[1] = __uint_as_float(w1.x); a1[2] = __uint_as_float(w1.y);
                a2[0] = __uint_as_float(w1.z); a2[1] = __uint_as_float(w1.w);
            } else {
                const uint2* q = reinterpret_cast<const uint2*>(vp);
                const uint2 w0 = __ldg(q), w1 = __ldg(q + 1), w2 = __ldg(q + 2);
                a0[0] = __uint_as_float(w0.x); a0[1] = __uint_as_float(w0.y); a0[2] = __uint_as_float(w1.x);
                a1[0] = __uint_as_float(w1.y); a1[1] = __uint_as_float(w2.x); a1[2] = __uint_as_float(w2.y);
            }
        } else {
            fetch_f32_unchecked<3>(d, 0, vertex, instance, a0);
            fetch_f32_unchecked<3>(d, 1, vertex, instance, a1);
            if constexpr (FVS == FAST_VS_MVP_TEX) fetch_f32_unchecked<2>(d, 2, vertex, instance, a2);
        }
        if constexpr (FVS == FAST_VS_MVP_TEX) {
            var[3] = a2[0];
            var[4] = a2[1];
        }
        pos = mat4_mul_vec4(mvp, V4{a0[0], a0[1], a0[2], 1.0f});
        var[0] = a1[0];
        var[1] = a1[1];
        var[2] = a1[2];
    } else if constexpr (FVS == FAST_VS_QUAD) {
        fetch_f32_unchecked<3>(d, 0, vertex, instance, a0);
        fetch_f32_unchecked<4>(d, 1, vertex, instance, a1);
        pos = {a0[0], a0[1], a0[2], 1.0f};
        for (int k = 0; k < 4; ++k) var[k] = a1[k];
    } else if constexpr (FVS == FAST_VS_QUAD_F16) {
        // Float16x4 colour widened to f32 (the extension profile's fetch_attr conversion)
        fetch_f32_unchecked<3>(d, 0, vertex, instance, a0);
        const AttrDesc& a = d.attr[1];
        const int b = a.buffer;
        const uint64_t start = (uint64_t)instance * d.vb_stride_instance[b] + (uint64_t)vertex * d.vb_stride_vertex[b] +
                               a.offset;
        const uint16_t* h = reinterpret_cast<const uint16_t*>(d.vb_data[b] + start);
        pos = {a0[0], a0[1], a0[2], 1.0f};
        for (int k = 0; k < 4; ++k) var[k] = f16_bits_to_f32(__ldg(h + k));
    } else if constexpr (FVS == FAST_VS_CLIP) {
        fetch_f32_unchecked<4>(d, 0, vertex, instance, a0);
        fetch_f32_unchecked<4>(d, 1, vertex, instance, a1);
        pos = {a0[0], a0[1], a0[2], a0[3]};
        for (int k = 0; k < 4; ++k) var[k] = a1[k];
    } else {
        const uint32_t vi = vertex % 3u;
        pos = {(float)((int32_t)vi - 1), (float)((int32_t)(vi & 1u) * 2 - 1), 0.0f, 1.0f};
        var[0] = (float)(vi == 0u);
        var[1] = (float)(vi == 1u);
        var[2] = (float)(vi == 2u);
        var[3] = 1.0f;
    }
}

// Sets up primitive gp completely when it needs no clipping and raises no error (returns
// false otherwise: the generic kernel redoes it, reports errors and clips).
template <int FVS, bool EDGE>
__device__ __forceinline__ bool fast_prim(const BatchParams& bp, const DrawDesc& d, const float* mvp, uint32_t gp,
                                          uint32_t di, TriRecord* rec, const TriRecord*& coop) {
    constexpr uint32_t NV = fast_vs_varyings(FVS);
    const uint32_t local = gp - d.prim_base;
    const uint32_t inst = d.instance_count == 1 ? 0u : local / d.prims_per_instance;
    const uint32_t p = local - inst * d.prims_per_instance;
    const uint32_t instance = d.instance_start + inst;
    // an empty record until it is built (the exits below that drop the primitive leave it so)
    *reinterpret_cast<uint4*>(rec) = make_uint4(gp << SUBTRI_BITS, di, p, 2u);
    rec->nsub = 0;
    uint32_t sp[3];
    if (d.topology == 4) {  // triangle strip (primitive.rs:360-392)
        sp[0] = (p & 1u) ? p + 1 : p;
        sp[1] = (p & 1u) ? p : p + 1;
        sp[2] = p + 2;
    } else {
        sp[0] = 3 * p;
        sp[1] = 3 * p + 1;
        sp[2] = 3 * p + 2;
    }
    // index resolution (render_pass/index.rs:45-88) and the vertex stage, every range check first
    // (any failure hands the primitive to the generic kernel, which reports it in the reference's
    // order), so the three index loads and then all attribute loads issue back to back
    uint32_t vtx[3];
    const uint64_t at_last = (uint64_t)d.first + max(sp[0], max(sp[1], sp[2]));
#pragma unroll
    for (int k = 0; k < 3; ++k) vtx[k] = d.first + sp[k];
    if (d.index_format != 0) {
        const uint32_t isz = d.index_format == 1 ? 2u : 4u;
        if ((at_last + 1) * isz > d.index_bytes) return false;
        uint32_t raw[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            raw[k] = d.index_format == 1 ? (uint32_t)__ldg(reinterpret_cast<const uint16_t*>(d.index_data) + vtx[k])
                                         : __ldg(reinterpret_cast<const uint32_t*>(d.index_data) + vtx[k]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int64_t v = (int64_t)raw[k] + (int64_t)d.base_vertex;
            if (v < 0 || v > 0xFFFFFFFFll) return false;
            vtx[k] = (uint32_t)v;
        }
    }
    if (max(vtx[0], max(vtx[1], vtx[2])) >= d.fast_vcount) {  // past the draw's safe range: check each fetch
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (!fast_vertex_in_range<FVS>(d, vtx[k], instance)) return false;
    }
    V4 pos[3];
    float var[3][NV];
#pragma unroll
    for (int k = 0; k < 3; ++k) fast_vertex<FVS>(d, mvp, vtx[k], instance, pos[k], var[k]);
    if (!d.has_fragment) return true;
    if (pos[0].w == 0.0f || pos[1].w == 0.0f || pos[2].w == 0.0f) return false;
    // x/w, y/w, z/w by the correctly rounded reciprocal RN(1/w) (also the reference's
    // `1.0 / w`) and div_by_recip's exact quotient
    float rw[3], n[3][2];
    bool wok[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        rw[i] = __frcp_rn(pos[i].w);
        wok[i] = div_fast_ok(pos[i].w);
        n[i][0] = div_by_recip(pos[i].x, pos[i].w, rw[i], wok[i]);
        n[i][1] = div_by_recip(pos[i].y, pos[i].w, rw[i], wok[i]);
    }
    // TriFace (primitive.rs:169-197) and the cull decision (state.rs:542-561)
    const float abx = fsub(n[1][0], n[0][0]), aby = fsub(n[1][1], n[0][1]);
    const float acx = fsub(n[2][0], n[0][0]), acy = fsub(n[2][1], n[0][1]);
    const bool ccw = fsub(fmul(abx, acy), fmul(aby, acx)) > 0.0f;
    const bool front_facing = (ccw ? 0u : 1u) == d.front_face;
    const bool cull = d.cull_mode == 1 ? front_facing : d.cull_mode == 2 ? !front_facing : false;
    if (cull) return true;
    // clipping: nothing to do inside all planes; dropped, exactly as clip_tri_ordered drops it,
    // when all three vertices are outside the first plane any of them is outside (the planes
    // before it pass the triangle through unchanged); a real split goes to the generic path
    // For finite coordinates dot4 against these planes (coefficients 0 and +-1) is the plain sum
    // of its two non-zero terms up to the sign of a zero result, and only `< 0` is asked: the
    // sums (x + w, -x + w, y + w, -y + w, z, -z + w) decide exactly as dot4 does.
    const float inf = __int_as_float(0x7F800000);
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 3; ++i)
        finite = finite && fabsf(pos[i].x) < inf && fabsf(pos[i].y) < inf && fabsf(pos[i].z) < inf &&
                 fabsf(pos[i].w) < inf;
    if (finite) {
        float dist[3][6];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            dist[i][0] = fadd(pos[i].x, pos[i].w);
            dist[i][1] = fadd(-pos[i].x, pos[i].w);
            dist[i][2] = fadd(pos[i].y, pos[i].w);
            dist[i][3] = fadd(-pos[i].y, pos[i].w);
            dist[i][4] = pos[i].z;
            dist[i][5] = fadd(-pos[i].z, pos[i].w);
        }
#pragma unroll
        for (int pl = 0; pl < 6; ++pl) {
            const int out = (dist[0][pl] < 0.0f) + (dist[1][pl] < 0.0f) + (dist[2][pl] < 0.0f);
            if (out == 3) return true;  // no sub-triangles: the record stays empty
            if (out != 0) return false;
        }
    } else {
#pragma unroll
        for (int pl = 0; pl < 6; ++pl) {
            const V4 nrm = clip_plane(pl);
            const int out = (dot4(pos[0], nrm) < 0.0f) + (dot4(pos[1], nrm) < 0.0f) + (dot4(pos[2], nrm) < 0.0f);
            if (out == 3) return true;
            if (out != 0) return false;
        }
    }
    // to_raster (raster.rs:145-160) on the quotients at hand
    CV v[3];
    uint32_t fbx[3], fby[3];
    V4 frag[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        v[i].p = pos[i];
        v[i].b[0] = i == 0 ? 1.0f : 0.0f;
        v[i].b[1] = i == 1 ? 1.0f : 0.0f;
        v[i].b[2] = i == 2 ? 1.0f : 0.0f;
        const float nz = div_by_recip(pos[i].z, pos[i].w, rw[i], wok[i]);
        const float vx = rust_max0(fadd(fmul(n[i][0], d.vp_sx), d.vp_tx));
        const float vy = rust_max0(fadd(fmul(n[i][1], d.vp_sy), d.vp_ty));
        fbx[i] = rust_f2u32(vx);
        fby[i] = rust_f2u32(vy);
        if ((fbx[i] | fby[i]) >= (1u << 30)) return false;  // the generic path reports it
        frag[i] = {vx, vy, nz, rw[i]};
    }
    build_record_frag<NV, EDGE>(bp, rec, gp << SUBTRI_BITS, di, p, front_facing, v, fbx, fby, frag, rw, var, NV);
    if (!(rec->flags & 2u) && tiles_are_many(*rec, bp.tile_shift)) coop = rec;  // k_setup counts the rest
    return true;
}

// One lane per primitive.  A warp whose lanes share a draw copies its descriptor (and matrix)
// to shared memory and runs the vertex stage specialised for the draw's FastVs shape; its 32
// primary records are built in shared memory and written out as one contiguous, coalesced
// block (records of consecutive primitives are adjacent).  Primitives it cannot finish are
// queued for k_setup_slow.
//
// ONLY >= 0: this launch sets up the draws whose FastVs shape is ONLY, so its code holds one
// vertex-stage variant; the launch sequence runs one such launch per shape present.  Its work is
// the shape's draws cut into 32-primitive groups aligned at each draw's first primitive
// (bp.shape_groups lists them), so every group lies within one draw; a warp finds its group's
// draw by a 32-way search of that list (two rounds for a thousand draws).
// ONLY = -1 sets up every primitive of the batch in 32-primitive groups of the batch's primitive
// order (all variants inlined); a group straddling draws goes to the generic kernel.
template <bool EDGE, int ONLY = -1>
__global__ void __launch_bounds__(kSetupWarps * 32) k_setup(BatchParams bp) {
    extern __shared__ __align__(16) uint8_t s_stage_raw[];
    __shared__ DrawCache s_dc[kSetupWarps];
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t rstride = bp.record_stride;
    uint8_t* stage = s_stage_raw + (size_t)warp * 32 * rstride;
    DrawCache& dc = s_dc[warp];
    if (lane == 0) dc.id = 0xFFFFFFFFu;
    __syncwarp();
    if (*bp.abort_flag) return;  // written only by earlier kernels: uniform across the grid

    // the draw's descriptor, matrix and target to the warp's cache (warp-uniform).  A warp's
    // groups lie a grid apart, so nearly every group changes draws: the loads of each step issue
    // together before any is used, so the copy costs two dependent loads (the descriptor with the
    // matrix's address and the target's index, then the matrix and the target)
    auto cache_draw = [&](uint32_t di) {
        constexpr uint32_t NQ = sizeof(DrawDesc) / 16, NR = (NQ + 31) / 32, NT = sizeof(TargetDesc) / 8;
        const uint4* src = reinterpret_cast<const uint4*>(bp.draws + di);
        uint4 q[NR];
#pragma unroll
        for (uint32_t r = 0; r < NR; ++r)
            if (lane + 32 * r < NQ) q[r] = __ldg(src + lane + 32 * r);
        const uint8_t* u = bp.draws[di].uniform[0][0];
        const bool has = u != nullptr && bp.draws[di].uniform_size[0][0] >= 64;
        const uint32_t ti = bp.draws[di].target;
        float m = 0.0f;
        uint2 tw = make_uint2(0u, 0u);
        if (lane < 16) {
            if (has) m = __ldg(reinterpret_cast<const float*>(u) + lane);
        } else if (lane < 16 + NT) {
            tw = __ldg(reinterpret_cast<const uint2*>(bp.targets + ti) + (lane - 16));
        }
        __syncwarp();  // the warp is done with the previous draw's cache
        uint4* dst = reinterpret_cast<uint4*>(&dc.d);
#pragma unroll
        for (uint32_t r = 0; r < NR; ++r)
            if (lane + 32 * r < NQ) dst[lane + 32 * r] = q[r];
        if (lane < 16) dc.mvp[lane] = m;
        else if (lane < 16 + NT) reinterpret_cast<uint2*>(&dc.t)[lane - 16] = tw;
        if (lane == 0) dc.id = di;
        __syncwarp();
    };
    // primitives [base, base + nrec) of the batch, lane -> base + lane (live: a primitive of the
    // batch; uniform: the warp's live lanes share draw di, which is in the cache)
    auto setup_group = [&](uint32_t base, uint32_t nrec, bool live, bool uniform, uint32_t di) {
        const uint32_t gp = base + lane;
        // the previous group's bulk copy has read the stage before its records are overwritten
        if (lane == 0) bulk_wait_read();
        __syncwarp();
        TriRecord* rec = reinterpret_cast<TriRecord*>(stage + (size_t)lane * rstride);
        const TriRecord* coop = nullptr;
        bool done = false;
        if (live && uniform) {
            if constexpr (ONLY > 0) {
                done = fast_prim<ONLY, EDGE>(bp, dc.d, dc.mvp, gp, di, rec, coop);
            } else if constexpr (ONLY < 0) {
                switch (dc.d.fast_vs) {  // warp-uniform
                    case FAST_VS_MVP_COLOR: done = fast_prim<FAST_VS_MVP_COLOR, EDGE>(bp, dc.d, dc.mvp, gp, di, rec, coop); break;
                    case FAST_VS_MVP_TEX: done = fast_prim<FAST_VS_MVP_TEX, EDGE>(bp, dc.d, dc.mvp, gp, di, rec, coop); break;
                    case FAST_VS_QUAD: done = fast_prim<FAST_VS_QUAD, EDGE>(bp, dc.d, dc.mvp, gp, di, rec, coop); break;
                    case FAST_VS_CLIP: done = fast_prim<FAST_VS_CLIP, EDGE>(bp, dc.d, dc.mvp, gp, di, rec, coop); break;
                    case FAST_VS_TRIANGLE: done = fast_prim<FAST_VS_TRIANGLE, EDGE>(bp, dc.d, dc.mvp, gp, di, rec, coop); break;
                    case FAST_VS_QUAD_F16: done = fast_prim<FAST_VS_QUAD_F16, EDGE>(bp, dc.d, dc.mvp, gp, di, rec, coop); break;
                    default: break;
                }
            }
        }
        // tile counts of the finished records: one atomic per distinct tile of the warp's
        // single-tile records (neighbouring triangles of a mesh mostly share one), a walk over the
        // tiles for the other records but those handed to the warp as a whole (coop)
        uint32_t hint = TILE_HINT_EMPTY;
        if (live && done) {
            hint = tile_hint_of(bp, *rec, dc.d, dc.t);
            if (bp.tile_hint) bp.tile_hint[gp] = hint;
        }
        const uint32_t single = hint < TILE_HINT_EMPTY ? hint : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(kFull, single);
        if (single != 0xFFFFFFFFu && (int)lane == __ffs(peers) - 1) atomicAdd(&bp.tile_count[single], (uint32_t)__popc(peers));
        if (hint == TILE_HINT_WALK && coop == nullptr) {
            const TargetDesc& t = dc.t;
            for_each_tile<EDGE>(*rec, dc.d, t, bp.tile_shift,
                                [&](uint32_t lt) { atomicAdd(&bp.tile_count[t.tile_base + lt], 1u); });
        }
        // the rest to the generic kernel (its record is rewritten there)
        const uint32_t m = __ballot_sync(kFull, live && !done);
        if (m) {
            const int leader = __ffs(m) - 1;
            uint32_t at = 0;
            if ((int)lane == leader) at = atomicAdd(&bp.status->slow_count, (uint32_t)__popc(m));
            at = __shfl_sync(kFull, at, leader);
            if (live && !done) bp.slow_prims[at + __popc(m & ((1u << lane) - 1u))] = gp;
        }
        coop_tiles<EDGE>(bp, coop, lane, [&](uint32_t tile, uint32_t) { atomicAdd(&bp.tile_count[tile], 1u); });
        // the warp's records, staged above, out as one block by the bulk-copy engine (16-byte
        // aligned: the record stride is a multiple of 16)
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) bulk_store_s2g(bp.records + (size_t)base * rstride, stage, nrec * rstride);
    };

    if constexpr (ONLY >= 0) {
        // grid-stride over the shape's draw-aligned groups
        const uint32_t e0 = bp.sg_off[ONLY], e1 = bp.sg_off[ONLY + 1];
        if (e1 == e0) return;
        const uint2* tab = reinterpret_cast<const uint2*>(bp.shape_groups);
        const uint32_t groups = __ldg(&tab[e1 - 1].y);
        const uint32_t nwarps = gridDim.x * kSetupWarps;
        for (uint32_t g = blockIdx.x * kSetupWarps + warp; g < groups; g += nwarps) {
            // the last of the shape's draws whose first group is <= g; tab[lo].y <= g throughout
            uint32_t lo = e0, cnt = e1 - 1 - e0;
            while (cnt > 32) {
                const uint32_t step = (cnt + 31) / 32;
                const bool le = lane * step < cnt && __ldg(&tab[lo + lane * step].y) <= g;
                const uint32_t at = 31 - __clz(__ballot_sync(kFull, le)) ;
                lo += at * step;
                cnt = min(step, cnt - at * step);
            }
            const bool le = lane < cnt && __ldg(&tab[lo + lane].y) <= g;
            const uint2 ent = __ldg(&tab[lo + 31 - __clz(__ballot_sync(kFull, le))]);
            if (dc.id != ent.x) cache_draw(ent.x);
            const uint32_t first = dc.d.prim_base + (g - ent.y) * 32u;
            const uint32_t end = dc.d.prim_base + dc.d.prims_per_instance * dc.d.instance_count;
            setup_group(first, min(32u, end - first), first + lane < end, true, ent.x);
        }
    } else {
        // grid-stride over 32-primitive groups (measured faster than giving each warp a contiguous
        // run of groups: 3.3 against 4.1 ms on the batched workload, whose expensive draws then
        // pile up on a few warps)
        const uint32_t stride = gridDim.x * blockDim.x;
        for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < bp.total_prims; base += stride) {
            const uint32_t gp = base + lane;
            const bool live = gp < bp.total_prims;
            uint32_t di = 0;
            if (live) {
                if (dc.id != 0xFFFFFFFFu && gp >= dc.d.prim_base &&
                    gp - dc.d.prim_base < dc.d.prims_per_instance * dc.d.instance_count)
                    di = dc.id;
                else
                    di = find_draw(bp, gp);
            }
            const uint32_t di0 = __shfl_sync(kFull, di, 0);
            const bool uniform = __all_sync(kFull, !live || di == di0);
            if (uniform && dc.id != di0) cache_draw(di0);
            setup_group(base, min(32u, bp.total_prims - base), live, uniform, di);
        }
    }
    if (lane == 0) bulk_wait_all();  // the last copy is done before the CTA (and its stage) ends
}

// Single-CTA exclusive scan of tile counts -> tile_offset; zeroes tile_cursor.
// Chunks of 4096 counts are loaded coalesced into shared memory, each thread scans four
// consecutive counts, and warps combine through shuffles; a carry links the chunks.
// For the visibility raster it also lists the tiles over split_chunk records and gives each of
// them ceil(count / split_chunk) chunk work items, as many as the split buffers hold (a tile that
// does not fit is rasterised whole).
// (a template only so that both kernel translation units can instantiate it)
template <int = 0>
__global__ void __launch_bounds__(1024) k_scan(BatchParams bp) {
    __shared__ uint32_t buf[4096];
    __shared__ uint32_t warp_sum[32];
    __shared__ unsigned long long s_carry;
    __shared__ uint32_t s_heavy;
    const uint32_t n = bp.total_tiles;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) {
        s_carry = 0;
        s_heavy = 0;
    }
    __syncthreads();
    // the counts of a chunk are loaded while the chunk before it is scanned
    uint32_t ahead[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t i = tid + j * 1024;
        ahead[j] = i < n ? bp.tile_count[i] : 0u;
    }
    for (uint32_t base = 0; base < n; base += 4096) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            buf[tid + j * 1024] = ahead[j];
            const uint32_t i = base + 4096 + tid + j * 1024;
            ahead[j] = i < n ? bp.tile_count[i] : 0u;
        }
        __syncthreads();
        const uint32_t a0 = buf[4 * tid], a1 = buf[4 * tid + 1], a2 = buf[4 * tid + 2], a3 = buf[4 * tid + 3];
        const uint32_t s = a0 + a1 + a2 + a3;
        if (bp.split_heavy && max(max(a0, a1), max(a2, a3)) > bp.split_chunk) {
            const uint32_t a[4] = {a0, a1, a2, a3};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (a[k] <= bp.split_chunk) continue;
                const uint32_t tile = base + 4 * tid + k;  // < n: counts past the end load as 0
                const uint32_t h = atomicAdd(&s_heavy, 1u);
                if (h < bp.split_cap_heavy) {
                    uint32_t* e = bp.split_heavy + 4 * (size_t)h;
                    e[0] = tile;
                    e[1] = (a[k] - 1) / bp.split_chunk + 1;
                }
                bp.split_tile[tile] = h < bp.split_cap_heavy ? h : ~0u;
            }
        }
        uint32_t x = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w += y;
            }
            warp_sum[lane] = w;
        }
        __syncthreads();
        const uint32_t excl = (uint32_t)s_carry + (wid ? warp_sum[wid - 1] : 0u) + x - s;
        buf[4 * tid] = excl;
        buf[4 * tid + 1] = excl + a0;
        buf[4 * tid + 2] = excl + a0 + a1;
        buf[4 * tid + 3] = excl + a0 + a1 + a2;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t i = base + tid + j * 1024;
            if (i < n) {
                bp.tile_offset[i] = buf[tid + j * 1024];
                bp.tile_cursor[i] = 0;
            }
        }
        __syncthreads();
        if (tid == 0) s_carry += warp_sum[31];
        __syncthreads();
    }
    if (tid == 0) {
        const unsigned long long total = s_carry;
        bp.tile_offset[n] = (uint32_t)total;
        bp.status->bin_entries = total;
        if (total > bp.bin_capacity) raise_error(bp.status, ERR_OVERFLOW_BINS, (uint32_t)min(total, 0xFFFFFFFFull));
    }
    if (bp.split_heavy) {
        // chunk work items of the listed tiles in list order, while their running total fits
        // split_cap_items (a prefix of the list, the running total being monotone); the tiles
        // past it are rasterised whole.  Four entries per thread, block scan, carry per 4096.
        __shared__ uint32_t s_items;
        const uint32_t nh = min(s_heavy, bp.split_cap_heavy);
        if (tid == 0) {
            s_items = 0;
            s_carry = 0;
        }
        __syncthreads();
        for (uint32_t base = 0; base < nh; base += 4096) {
            uint32_t c[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t h = base + 4 * tid + k;
                c[k] = h < nh ? bp.split_heavy[4 * (size_t)h + 1] : 0u;
            }
            const uint32_t sum = c[0] + c[1] + c[2] + c[3];
            uint32_t x = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) warp_sum[wid] = x;
            __syncthreads();
            if (wid == 0) {
                uint32_t w = warp_sum[lane];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
                    if (lane >= o) w += y;
                }
                warp_sum[lane] = w;
            }
            __syncthreads();
            unsigned long long first = s_carry + (wid ? warp_sum[wid - 1] : 0u) + x - sum;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t h = base + 4 * tid + k;
                if (h >= nh) break;
                uint32_t* e = bp.split_heavy + 4 * (size_t)h;
                if (first + c[k] <= bp.split_cap_items) {
                    e[2] = (uint32_t)first;
                    e[3] = 0;
                    for (uint32_t j = 0; j < c[k]; ++j) bp.split_item[first + j] = h;
                    atomicMax(&s_items, (uint32_t)(first + c[k]));
                } else {
                    bp.split_tile[e[0]] = ~0u;
                }
                first += c[k];
            }
            __syncthreads();
            if (tid == 0) s_carry += warp_sum[31];
            __syncthreads();
        }
        if (tid == 0) bp.status->split_items = s_items;
    }
}

template <bool EDGE>
__global__ void __launch_bounds__(128) k_fill(BatchParams bp) {
    // after an abort the setup kernels returned early: the records are not this batch's
    if (bp.status->error || *bp.abort_flag) return;
    const uint32_t n_ovf = min(bp.status->ovf_used, bp.ovf_capacity);
    const uint32_t total = bp.total_prims + n_ovf;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31;
    auto put = [&](uint32_t tile, uint32_t key) {
        const uint32_t pos = atomicAdd(&bp.tile_cursor[tile], 1u);
        bp.bins[bp.tile_offset[tile] + pos] = key;
    };
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total; base += stride) {
        const uint32_t i = base + lane;
        const TriRecord* coop = nullptr;
        const uint32_t hint = i < bp.total_prims && bp.tile_hint ? bp.tile_hint[i] : TILE_HINT_WALK;
        // single-tile records (a primary record is sub-triangle 0 of its primitive): one cursor
        // atomic per distinct tile of the warp, each lane taking the slot of its rank among peers
        const uint32_t single = hint < TILE_HINT_EMPTY ? hint : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, single);
        if (single != 0xFFFFFFFFu) {
            const uint32_t bin0 = bp.tile_offset[single];  // loaded while the cursor atomic is out
            const int leader = __ffs(peers) - 1;
            uint32_t pos = 0;
            if ((int)lane == leader) pos = atomicAdd(&bp.tile_cursor[single], (uint32_t)__popc(peers));
            pos = __shfl_sync(peers, pos, leader) + (uint32_t)__popc(peers & ((1u << lane) - 1u));
            bp.bins[bin0 + pos] = i << SUBTRI_BITS;
        } else if (i < total && hint == TILE_HINT_WALK) {
            const TriRecord* r = i < bp.total_prims ? rec_at(bp.records, bp.record_stride, i)
                                                    : rec_at(bp.ovf_records, bp.record_stride, i - bp.total_prims);
            if (!(r->flags & 2u)) {
                if (tiles_are_many(*r, bp.tile_shift) || bbox_tiles(*r, bp.tile_shift) > 8u) {
                    coop = r;  // the warp walks it (coop_tiles_flat below)
                } else {
                    const DrawDesc& d = bp.draws[r->draw];
                    const TargetDesc& t = bp.targets[d.target];
                    const uint32_t key = r->key;
                    // A box of at most eight tiles, to which tile_row_cols gives every tile row the
                    // box's columns: for_each_tile's tiles are the rectangle of rows [lo, hi] and
                    // columns [c0, c1].  Their cursor atomics and bin offsets go out together
                    // (not one tile's round trip after another's), then the keys are stored.
                    int lo, hi;
                    record_rows(*r, d, t, lo, hi);
                    if (lo <= hi) {
                        const int ty0 = lo >> bp.tile_shift, ty1 = hi >> bp.tile_shift;
                        int c0, c1;
                        tile_row_cols<EDGE>(*r, d, t, bp.tile_shift, lo, hi, ty0, c0, c1);
                        const int n = c1 >= c0 ? (ty1 - ty0 + 1) * (c1 - c0 + 1) : 0;
                        if (n <= 8) {
                            uint32_t slot[8];
                            uint32_t lt = t.tile_base + (uint32_t)ty0 * t.tiles_x + (uint32_t)c0;
                            const uint32_t row_step = t.tiles_x - (uint32_t)(c1 - c0);
                            int tx = c0;
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                slot[k] = 0;
                                if (k < n) {
                                    slot[k] = bp.tile_offset[lt] + atomicAdd(&bp.tile_cursor[lt], 1u);
                                    if (tx == c1) {
                                        tx = c0;
                                        lt += row_step;
                                    } else {
                                        ++tx;
                                        ++lt;
                                    }
                                }
                            }
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                if (k < n) bp.bins[slot[k]] = key;
                        } else {  // not reached (the box holds at most eight tiles); kept exact
                            for_each_tile<EDGE>(*r, d, t, bp.tile_shift, [&](uint32_t lt) { put(t.tile_base + lt, key); });
                        }
                    }
                }
            }
        }
        coop_tiles_flat<EDGE>(bp, coop, lane, put);
    }
}

// ------------------------------------------------------------------------- raster
// Ascending bitonic sort of n keys (n need not be a power of two: the comparators whose upper
// index is >= n are skipped, as if those slots held +infinity).  All threads of the CTA call it.
__device__ __forceinline__ void block_sort(uint32_t* a, uint32_t n) {
    uint32_t N = 1;
    while (N < n) N <<= 1;
    const uint32_t half = N >> 1;
    for (uint32_t k = 2; k <= N; k <<= 1) {
        const uint32_t hk = k >> 1;
        for (uint32_t i = threadIdx.x; i < half; i += blockDim.x) {
            uint32_t blk = i / hk, off = i - blk * hk;
            uint32_t lo = blk * k + off, hi = blk * k + k - 1 - off;
            if (hi < n) {
                uint32_t x = a[lo], y = a[hi];
                if (x > y) { a[lo] = y; a[hi] = x; }
            }
        }
        __syncthreads();
        for (uint32_t j = k >> 2; j >= 1; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < half; i += blockDim.x) {
                uint32_t blk = i / j, off = i - blk * j;
                uint32_t lo = blk * 2 * j + off, hi = lo + j;
                if (hi < n) {
                    uint32_t x = a[lo], y = a[hi];
                    if (x > y) { a[lo] = y; a[hi] = x; }
                }
            }
            __syncthreads();
        }
    }
}

__device__ __forceinline__ bool depth_compare(uint32_t f, float v, float r) {  // render_pass/mod.rs:434-452
    switch (f) {
        case 1: return false;
        case 2: return v < r;
        case 3: return v == r;
        case 4: return v <= r;
        case 5: return v > r;
        case 6: return v != r;
        case 7: return v >= r;
        default: return true;
    }
}

// Encodes a colour into the target format (texture.rs:373-411); c[] holds the texel bytes.
__device__ __forceinline__ void encode_color(uint32_t fmt, V4 col, uint32_t c[4]) {
    switch (fmt) {
        case 1: c[0] = unorm8_trunc(col.x); break;
        case 2: c[0] = unorm8_trunc(col.x) | (unorm8_trunc(col.y) << 8); break;
        case 3: case 4:
            c[0] = unorm8_trunc(col.x) | (unorm8_trunc(col.y) << 8) | (unorm8_trunc(col.z) << 16) |
                   (unorm8_trunc(col.w) << 24);
            break;
        case 5: case 6:
            c[0] = unorm8_trunc(col.z) | (unorm8_trunc(col.y) << 8) | (unorm8_trunc(col.x) << 16) |
                   (unorm8_trunc(col.w) << 24);
            break;
        case 7: {  // two round-to-nearest-even conversions per instruction, low half first
            const __half2 lo = __floats2half2_rn(col.x, col.y), hi = __floats2half2_rn(col.z, col.w);
            c[0] = *reinterpret_cast<const uint32_t*>(&lo);
            c[1] = *reinterpret_cast<const uint32_t*>(&hi);
            break;
        }
        case 8:
            c[0] = __float_as_uint(col.x); c[1] = __float_as_uint(col.y);
            c[2] = __float_as_uint(col.z); c[3] = __float_as_uint(col.w);
            break;
        case TFMT_RGBA8_SRGB_ENCODE:  // extension profile: RGB encoded to sRGB, alpha linear
            c[0] = linear_to_srgb8(col.x) | (linear_to_srgb8(col.y) << 8) | (linear_to_srgb8(col.z) << 16) |
                   (unorm8_round(col.w) << 24);
            break;
        case TFMT_BGRA8_SRGB_ENCODE:
            c[0] = linear_to_srgb8(col.z) | (linear_to_srgb8(col.y) << 8) | (linear_to_srgb8(col.x) << 16) |
                   (unorm8_round(col.w) << 24);
            break;
        default: break;
    }
}
__device__ __forceinline__ V4 decode_color(uint32_t fmt, const uint32_t c[4]) {
    switch (fmt) {
        case 3: case 4:
            return {fdiv((float)(c[0] & 0xFF), 255.0f), fdiv((float)((c[0] >> 8) & 0xFF), 255.0f),
                    fdiv((float)((c[0] >> 16) & 0xFF), 255.0f), fdiv((float)(c[0] >> 24), 255.0f)};
        case 5: case 6:
            return {fdiv((float)((c[0] >> 16) & 0xFF), 255.0f), fdiv((float)((c[0] >> 8) & 0xFF), 255.0f),
                    fdiv((float)(c[0] & 0xFF), 255.0f), fdiv((float)(c[0] >> 24), 255.0f)};
        case 7: {
            const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&c[0]));
            const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&c[1]));
            return {lo.x, lo.y, hi.x, hi.y};
        }
        case 8: return {__uint_as_float(c[0]), __uint_as_float(c[1]), __uint_as_float(c[2]), __uint_as_float(c[3])};
        case TFMT_RGBA8_SRGB_ENCODE:
            return {srgb_to_linear(c[0]), srgb_to_linear(c[0] >> 8), srgb_to_linear(c[0] >> 16),
                    fdiv((float)(c[0] >> 24), 255.0f)};
        case TFMT_BGRA8_SRGB_ENCODE:
            return {srgb_to_linear(c[0] >> 16), srgb_to_linear(c[0] >> 8), srgb_to_linear(c[0]),
                    fdiv((float)(c[0] >> 24), 255.0f)};
        default: return {0.0f, 0.0f, 0.0f, 0.0f};
    }
}

__device__ __forceinline__ float blend_factor(uint32_t f, float s, float sa, float dd, float da, float k) {
    switch (f) {
        case 0: return 0.0f;
        case 1: return 1.0f;
        case 2: return s;
        case 3: return fsub(1.0f, s);
        case 4: return sa;
        case 5: return fsub(1.0f, sa);
        case 6: return dd;
        case 7: return fsub(1.0f, dd);
        case 8: return da;
        case 9: return fsub(1.0f, da);
        case 11: return k;
        case 12: return fsub(1.0f, k);
        default: return 0.0f;
    }
}
__device__ __forceinline__ float blend_channel(const uint32_t bc[3], float s, float sa, float dd, float da, float k) {
    if (bc[2] == 3) return fminf(s, dd);
    if (bc[2] == 4) return fmaxf(s, dd);
    float fs = blend_factor(bc[0], s, sa, dd, da, k);
    float fd = blend_factor(bc[1], s, sa, dd, da, k);
    float a = fmul(s, fs), b = fmul(dd, fd);
    switch (bc[2]) {
        case 1: return fsub(a, b);
        case 2: return fsub(b, a);
        default: return fadd(a, b);
    }
}

struct PixelState {
    uint32_t c[4];
    float depth;
};

// The fragment stage of any program: native programs on the cached state; a JIT module's WGSL
// program with its builtins — front_facing, primitive_index and @builtin(position), the
// rasterizer's fragment (x, y, z, 1/w) composed with the barycentrics like any inter-stage
// value (render_pass/fragment.rs:127-160, raster.rs:338-346).  False when discarded.
__device__ __forceinline__ bool run_fs_any(const BatchParams& bp, const RasterState& rs, const TriRecord& r,
                                           const float cmp[3], const float* var, const float* lut, V4& col) {
#ifdef GBR_JIT
    if (rs.program == PROG_JIT) {
        auto lerp3 = [&](const float* v) {
            return fadd(fadd(fmul(v[0], cmp[0]), fmul(v[1], cmp[1])), fmul(v[2], cmp[2]));
        };
        const V4 frag = {lerp3(r.vpx), lerp3(r.vpy), lerp3(r.fz), lerp3(r.fw)};
        const int st = jit_fs(*rs.dd, var, (r.flags & 1u) != 0, r.prim_index, frag, col);
        if (st == 2) raise_error(bp.status, ERR_SHADER_TRAP, r.key >> SUBTRI_BITS);
        return st == 1;
    }
#endif
    return run_fs_rs(rs, var, lut, col, r.lod);
}

// Rank sort for small bins: every key counts the keys below it (keys are unique per tile) and
// goes straight to its place; two barriers instead of a sorting network's log^2 stages.
__device__ __forceinline__ void rank_sort(const uint32_t* in, uint32_t* out, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t k = in[i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < n; ++j) rank += in[j] < k ? 1u : 0u;
        out[rank] = k;
    }
}

// One tile per CTA iteration.  Pixels are owned by threads in 8x4 blocks (one block per warp
// per PPT slot); their colour and depth stay in registers for the whole tile.  Records are
// staged RW at a time; for each staged record the CTA computes which 8x4 blocks it can touch
// (exact per-block-row x ranges of its spans), and every warp walks only the records whose bit
// is set for its block, in key order (ballot + find-first-set), without further barriers.
template <int T, int WARPS, int CAP, int RW, int KIND, bool EDGE = false>
__global__ void __launch_bounds__(WARPS * 32) k_raster(BatchParams bp) {
    constexpr int NT = WARPS * 32;
    constexpr int BLK_X = T / 8, BLK_Y = T / 4, NBLK = BLK_X * BLK_Y;
    constexpr int PPT = (NBLK + WARPS - 1) / WARPS;  // 8x4 blocks per warp
    constexpr int SMALL = 2 * NT;                    // bins up to this size use rank_sort
    static_assert(NBLK <= 32, "block mask is 32 bits");
    extern __shared__ __align__(16) uint8_t smem_raw[];
    uint32_t* s_keys = reinterpret_cast<uint32_t*>(smem_raw);  // CAP
    uint32_t* s_sorted = s_keys + CAP;                         // SMALL
    uint8_t* s_recs = reinterpret_cast<uint8_t*>(s_sorted + SMALL);
    __shared__ uint32_t s_mask[RW];
    __shared__ float4 s_kc[RW];  // p-independent shoelace terms of the three barycentrics, RN(1/area)
    __shared__ int2 s_span[RW * T];  // per staged record and tile row: emitted [x1, x2] within scissor and tile
    __shared__ const uint8_t* s_rec_ptr[RW];
    __shared__ RasterState s_rs[WARPS];
    __shared__ float s_lut[256];
    __shared__ uint32_t s_tile;
    __shared__ unsigned long long s_frag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool failed = bp.status->error != 0 || *bp.abort_flag != 0;
    if (failed && blockIdx.x == 0 && threadIdx.x == 0) *bp.abort_flag = 1u;
    for (int i = threadIdx.x; i < 256; i += NT) s_lut[i] = fdiv((float)i, 255.0f);  // `x as f32 / 255.0`
    if (lane == 0) s_rs[warp].draw = 0xFFFFFFFFu;
    if (threadIdx.x == 0) s_frag = 0;

    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(bp.work_counter, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= bp.total_tiles || failed) break;
        const uint32_t ti = find_target(bp.targets, bp.num_targets, tile);
        const TargetDesc& tg = bp.targets[ti];
        const uint32_t lt = tile - tg.tile_base;
        const int tx = (int)(lt % tg.tiles_x), ty = (int)(lt / tg.tiles_x);
        const uint32_t n = bp.tile_count[tile];
        const uint32_t off = bp.tile_offset[tile];

        // pixel state: LoadOp::Clear from the clear value, otherwise the stored texels
        PixelState px[PPT];
        int pxx[PPT], pxy[PPT];
        float pfx[PPT], pfy[PPT];
        bool pvalid[PPT];
        uint32_t clear_c[4] = {0, 0, 0, 0};
        if (tg.color) encode_color(tg.color_format, V4{tg.clear[0], tg.clear[1], tg.clear[2], tg.clear[3]}, clear_c);
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            const int blk = warp + k * WARPS;
            const int bx = blk % BLK_X, byy = blk / BLK_X;
            pxx[k] = tx * T + bx * 8 + (lane & 7);
            pxy[k] = ty * T + byy * 4 + (lane >> 3);
            pvalid[k] = blk < NBLK && pxx[k] < (int)tg.width && pxy[k] < (int)tg.height;
            pfx[k] = (float)pxx[k];
            pfy[k] = (float)pxy[k];
            const size_t pix = (size_t)pxy[k] * tg.width + pxx[k];
            px[k].c[0] = clear_c[0]; px[k].c[1] = clear_c[1]; px[k].c[2] = clear_c[2]; px[k].c[3] = clear_c[3];
            px[k].depth = tg.depth_clear;
            if (pvalid[k]) {
                if (tg.color && tg.color_load != 1) {
                    const uint8_t* src = tg.color + tg.slice_offset + pix * tg.color_bpp;
                    if (tg.color_bpp == 4) px[k].c[0] = *reinterpret_cast<const uint32_t*>(src);
                    else if (tg.color_bpp == 8) { px[k].c[0] = reinterpret_cast<const uint32_t*>(src)[0]; px[k].c[1] = reinterpret_cast<const uint32_t*>(src)[1]; }
                    else if (tg.color_bpp == 16) { for (int q = 0; q < 4; ++q) px[k].c[q] = reinterpret_cast<const uint32_t*>(src)[q]; }
                    else if (tg.color_bpp == 2) px[k].c[0] = *reinterpret_cast<const uint16_t*>(src);
                    else px[k].c[0] = *src;
                }
                if (tg.depth && tg.depth_load != 1) px[k].depth = tg.depth[pix];
            }
        }

        // the tile's keys in reference order
        const uint32_t* keys;
        if (n <= (uint32_t)SMALL) {
            for (uint32_t i = threadIdx.x; i < n; i += NT) s_keys[i] = bp.bins[off + i];
            __syncthreads();
            rank_sort(s_keys, s_sorted, n);
            keys = s_sorted;
        } else if (n <= (uint32_t)CAP) {
            for (uint32_t i = threadIdx.x; i < n; i += NT) s_keys[i] = bp.bins[off + i];
            __syncthreads();
            block_sort(s_keys, n);
            keys = s_keys;
        } else {
            block_sort(bp.bins + off, n);
            __threadfence_block();
            keys = bp.bins + off;
        }
        __syncthreads();

        uint32_t frag_count = 0;
        uint32_t fs_runs = 0, tex_runs = 0;  // fragment-stage invocations, and those that sample a texture
        const uint32_t stride = bp.record_stride;
        for (uint32_t w0 = 0; w0 < n; w0 += RW) {
            const uint32_t nb = min((uint32_t)RW, n - w0);
            for (uint32_t i = threadIdx.x; i < nb; i += NT) {
                const uint32_t key = keys[w0 + i];
                const uint32_t prim = key >> SUBTRI_BITS, sub = key & ((1u << SUBTRI_BITS) - 1u);
                const TriRecord* pr = rec_at(bp.records, stride, prim);
                s_rec_ptr[i] = sub == 0 ? reinterpret_cast<const uint8_t*>(pr)
                                        : reinterpret_cast<const uint8_t*>(
                                              rec_at(bp.ovf_records, stride, pr->ovf + sub - 1));
                s_mask[i] = 0;
            }
            __syncthreads();
            const uint32_t words = stride >> 4;
            for (uint32_t w = threadIdx.x; w < nb * words; w += NT) {
                const uint32_t ri = w / words, wi = w - ri * words;
                reinterpret_cast<uint4*>(s_recs + (size_t)ri * stride)[wi] =
                    __ldg(reinterpret_cast<const uint4*>(s_rec_ptr[ri]) + wi);
            }
            __syncthreads();
            // per (record, tile row): the span the scanline rule emits on that row, cut to the
            // draw's scissor and to the tile (empty = x1 > x2)
            for (uint32_t q = threadIdx.x; q < nb * T; q += NT) {
                const uint32_t ri = q / T, row = q - ri * T;
                const TriRecord& r = *reinterpret_cast<const TriRecord*>(s_recs + (size_t)ri * stride);
                if (row == 0)
                    s_kc[ri] = make_float4(fmul(fsub(r.vpy[2], r.vpy[1]), fadd(r.vpx[2], r.vpx[1])),
                                           fmul(fsub(r.vpy[0], r.vpy[2]), fadd(r.vpx[0], r.vpx[2])),
                                           fmul(fsub(r.vpy[1], r.vpy[0]), fadd(r.vpx[1], r.vpx[0])),
                                           __frcp_rn(r.area));
                const int y = ty * T + (int)row;
                int2 sp = make_int2(1, 0);
                if (y >= r.row0 && y <= r.row1 && y < (int)tg.height) {
                    const DrawDesc& d = bp.draws[r.draw];
                    if ((uint32_t)y >= d.sc_y0 && (uint32_t)y < d.sc_y1) {
                        int x1, x2;
                        span_at<EDGE>(r, y, x1, x2);
                        sp.x = max(max(x1, (int)d.sc_x0), tx * T);
                        sp.y = min(min(min(x2, (int)d.sc_x1 - 1), tx * T + T - 1), (int)tg.width - 1);
                    }
                }
                s_span[q] = sp;  // also empty outside the target, so no pixel test is needed below
            }
            __syncthreads();
            // which 8x4 blocks of the tile each staged record can emit into
            for (uint32_t ri = threadIdx.x; ri < nb; ri += NT) {
                uint32_t bits = 0;
#pragma unroll
                for (int band = 0; band < BLK_Y; ++band) {
                    int mn = T, mx = -1;
#pragma unroll
                    for (int rr = 0; rr < 4; ++rr) {
                        const int2 sp = s_span[ri * T + band * 4 + rr];
                        if (sp.x <= sp.y) {
                            mn = min(mn, sp.x - tx * T);
                            mx = max(mx, sp.y - tx * T);
                        }
                    }
                    if (mn <= mx)
                        for (int bx = mn >> 3; bx <= (mx >> 3); ++bx) bits |= 1u << (band * BLK_X + bx);
                }
                s_mask[ri] = bits;
            }
            __syncthreads();
            // the warp's 8x4 blocks, as bits of the record masks
            uint32_t wbits = 0;
#pragma unroll
            for (int k = 0; k < PPT; ++k)
                if (warp + k * WARPS < NBLK) wbits |= 1u << (warp + k * WARPS);
            for (uint32_t c0 = 0; c0 < nb; c0 += 32) {
                uint32_t todo = __ballot_sync(0xFFFFFFFFu, c0 + lane < nb && (s_mask[c0 + lane] & wbits));
                while (todo) {
                    const uint32_t ri = c0 + __ffs(todo) - 1;
                    todo &= todo - 1;
                    const TriRecord& r = *reinterpret_cast<const TriRecord*>(s_recs + (size_t)ri * stride);
                    RasterState& rs = s_rs[warp];
                    if (rs.draw != r.draw) {  // warp-uniform
                        __syncwarp();
                        if (lane == 0) build_raster_state(bp.draws[r.draw], r.draw, rs);
                        __syncwarp();
                    }
                    // per-record constants, held in registers across this lane's pixels
                    const uint32_t rmask = s_mask[ri];
                    const float ax = r.vpx[0], ay = r.vpy[0], bx = r.vpx[1], by = r.vpy[1], cx = r.vpx[2], cy = r.vpy[2];
                    const float4 kc = s_kc[ri];
                    const float kc0 = kc.x, kc1 = kc.y, kc2 = kc.z, rcp = kc.w;
                    const float area = r.area;
                    const bool area_ok = div_fast_ok(area);
                    const bool ident = (r.flags & 16u) != 0;
                    const float* rv = rec_var(&r);
                    constexpr uint32_t KNV = KIND == 1 ? 4 : KIND == 2 ? 5 : 0;
                    float rvv[3 * (KNV ? KNV : 1)];
                    if constexpr (KNV == 4) {
                        // 16-byte aligned: the record header is a multiple of 16 bytes
#pragma unroll
                        for (uint32_t q = 0; q < 3; ++q) {
                            const float4 v4 = reinterpret_cast<const float4*>(rv)[q];
                            rvv[4 * q] = v4.x; rvv[4 * q + 1] = v4.y; rvv[4 * q + 2] = v4.z; rvv[4 * q + 3] = v4.w;
                        }
                    } else if constexpr (KNV != 0) {
#pragma unroll
                        for (uint32_t q = 0; q < 3 * KNV; ++q) rvv[q] = rv[q];
                    }
                    // every pixel slot of a thread lies in one column when the warps of a tile
                    // cover whole block rows: x + a.x (likewise b, c) is then a per-record term
                    constexpr bool ONE_COL = WARPS % BLK_X == 0;
                    // the sample point: the integer pixel corner (the reference), or the pixel
                    // centre under the edge-function rule (x + 1/2 is exact)
                    const float px0 = EDGE ? fadd(pfx[0], 0.5f) : pfx[0];
                    const float xa0 = fadd(px0, ax), xb0 = fadd(px0, bx), xc0 = fadd(px0, cx);
#pragma unroll
                    for (int k = 0; k < PPT; ++k) {
                        const int blk = warp + k * WARPS;
                        if (blk >= NBLK || !((rmask >> blk) & 1u)) continue;  // warp-uniform
                        const int x = pxx[k], y = pxy[k];
                        {
                            // coverage: the row's span (already cut to scissor and tile)
                            const int2 sp = s_span[ri * T + (y - ty * T)];
                            if (x < sp.x || x > sp.y) continue;
                        }
                        // barycentrics at the integer pixel corner (raster.rs:313-321, 334-335); an
                        // IEEE sum does not depend on operand order, so x + a.x serves both shoelace
                        // terms that contain it (likewise b, c)
                        const float fx = EDGE ? fadd(pfx[k], 0.5f) : pfx[k], fy = EDGE ? fadd(pfy[k], 0.5f) : pfy[k];
                        const float xa = ONE_COL ? xa0 : fadd(fx, ax), xb = ONE_COL ? xb0 : fadd(fx, bx),
                                    xc = ONE_COL ? xc0 : fadd(fx, cx);
                        if constexpr (KIND == 1) {
                            // The same operations as the scalar path below, sums and differences
                            // two lanes per packed f32x2 instruction (each lane rounds exactly like
                            // the scalar op; products stay scalar, see f2mul_rn); a - b is
                            // a + (-b) in IEEE arithmetic, signed zeros included.
                            const float2 d02 = f2add(make_float2(by, fy), make_float2(-fy, -by));
                            const float2 t02 = f2add(f2mul_rn(d02, make_float2(xb, xb)), make_float2(kc0, kc2));
                            const float2 e02 = f2add(make_float2(fy, ay), make_float2(-cy, -fy));
                            const float2 s02 = f2add(t02, f2mul_rn(e02, make_float2(xc, xa)));
                            const float2 e1 = f2add(make_float2(fy, cy), make_float2(-ay, -fy));
                            const float2 m1 = f2mul_rn(e1, make_float2(xa, xc));
                            const float s1v = fadd(fadd(m1.x, m1.y), kc1);
                            float c0, c1, c2;
                            if (area_ok && div_fast_ok(s02.x) && div_fast_ok(s1v) && div_fast_ok(s02.y)) {
                                // div_by_recip's in-range path for s0 and s2 together (every
                                // product here feeds a fused multiply-add, as in the scalar steps)
                                const float2 y2 = make_float2(rcp, rcp), nb2 = make_float2(-area, -area);
                                float2 q = f2mul(s02, y2);
                                float2 rr = f2fma(nb2, q, s02);
                                q = f2fma(rr, y2, q);
                                rr = f2fma(nb2, q, s02);
                                const float2 l02 = f2fma(rr, y2, q);
                                const float l1 = div_by_recip(s1v, area, rcp, true);
                                if (ident) {
                                    c0 = l02.x; c1 = l1; c2 = l02.y;
                                } else {
                                    c0 = fadd(fadd(fmul(r.cb[0], l02.x), fmul(r.cb[3], l1)), fmul(r.cb[6], l02.y));
                                    c1 = fadd(fadd(fmul(r.cb[1], l02.x), fmul(r.cb[4], l1)), fmul(r.cb[7], l02.y));
                                    c2 = fadd(fadd(fmul(r.cb[2], l02.x), fmul(r.cb[5], l1)), fmul(r.cb[8], l02.y));
                                }
                            } else {
                                const float l0 = div_by_recip(s02.x, area, rcp, area_ok);
                                const float l1 = div_by_recip(s1v, area, rcp, area_ok);
                                const float l2 = div_by_recip(s02.y, area, rcp, area_ok);
                                c0 = fadd(fadd(fmul(r.cb[0], l0), fmul(r.cb[3], l1)), fmul(r.cb[6], l2));
                                c1 = fadd(fadd(fmul(r.cb[1], l0), fmul(r.cb[4], l1)), fmul(r.cb[7], l2));
                                c2 = fadd(fadd(fmul(r.cb[2], l0), fmul(r.cb[5], l1)), fmul(r.cb[8], l2));
                            }
                            ++frag_count;
                            ++fs_runs;
                            // linear vec4f colour straight to the output, then Rgba16Float blending
                            // (colour SrcAlpha/OneMinusSrcAlpha/Add, alpha One/OneMinusSrcAlpha/Add)
                            const float2 cc0 = make_float2(c0, c0), cc1 = make_float2(c1, c1), cc2 = make_float2(c2, c2);
                            const float2 v01 = f2add(f2add(f2mul_rn(make_float2(rvv[0], rvv[1]), cc0),
                                                           f2mul_rn(make_float2(rvv[4], rvv[5]), cc1)),
                                                     f2mul_rn(make_float2(rvv[8], rvv[9]), cc2));
                            const float2 v23 = f2add(f2add(f2mul_rn(make_float2(rvv[2], rvv[3]), cc0),
                                                           f2mul_rn(make_float2(rvv[6], rvv[7]), cc1)),
                                                     f2mul_rn(make_float2(rvv[10], rvv[11]), cc2));
                            const float2 dlo = __half22float2(*reinterpret_cast<const __half2*>(&px[k].c[0]));
                            const float2 dhi = __half22float2(*reinterpret_cast<const __half2*>(&px[k].c[1]));
                            const float w = v23.y;
                            const float2 oma = make_float2(fsub(1.0f, w), fsub(1.0f, w));
                            const float2 olo = f2add(f2mul_rn(v01, make_float2(w, w)), f2mul_rn(dlo, oma));
                            const float2 ohi = f2add(f2mul_rn(v23, make_float2(w, 1.0f)), f2mul_rn(dhi, oma));
                            const __half2 hlo = __float22half2_rn(olo), hhi = __float22half2_rn(ohi);
                            px[k].c[0] = *reinterpret_cast<const uint32_t*>(&hlo);
                            px[k].c[1] = *reinterpret_cast<const uint32_t*>(&hhi);
                            continue;
                        }
                        const float s0 = fadd(fadd(fmul(fsub(by, fy), xb), kc0), fmul(fsub(fy, cy), xc));
                        const float s1 = fadd(fadd(fmul(fsub(fy, ay), xa), fmul(fsub(cy, fy), xc)), kc1);
                        const float s2 = fadd(fadd(kc2, fmul(fsub(fy, by), xb)), fmul(fsub(ay, fy), xa));
                        const float l0 = div_by_recip(s0, area, rcp, area_ok);
                        const float l1 = div_by_recip(s1, area, rcp, area_ok);
                        const float l2 = div_by_recip(s2, area, rcp, area_ok);
                        // composed with the clip barycentrics (raster.rs:338-343).  For an unclipped
                        // record the composition is ((1*l0 + 0*l1) + 0*l2, ...), which equals
                        // (l0, l1, l2) exactly when every l is finite and non-zero — guaranteed when
                        // all three quotients took div_by_recip's in-range path.
                        float cmp[3];
                        if (ident && area_ok && div_fast_ok(s0) && div_fast_ok(s1) && div_fast_ok(s2)) {
                            cmp[0] = l0;
                            cmp[1] = l1;
                            cmp[2] = l2;
                        } else {
#pragma unroll
                            for (int j = 0; j < 3; ++j)
                                cmp[j] = fadd(fadd(fmul(r.cb[j], l0), fmul(r.cb[3 + j], l1)), fmul(r.cb[6 + j], l2));
                        }
                        ++frag_count;
                        if constexpr (KIND == 0) {
                            // @early_depth_test (fragment.rs:166-194): the depth test, and the
                            // depth write when it passes, before the fragment stage runs; a
                            // rejected fragment never reaches it
                            if (rs.early_depth != EARLY_DEPTH_NONE && rs.depth_test) {
                                const float z =
                                    fadd(fadd(fmul(r.fz[0], cmp[0]), fmul(r.fz[1], cmp[1])), fmul(r.fz[2], cmp[2]));
                                if (!depth_compare(rs.depth_compare, z, px[k].depth)) continue;
                                if (rs.depth_write) px[k].depth = z;
                            }
                        }
                        // inter-stage values (fragment.rs:319-378) and the fragment stage
                        V4 col;
                        ++fs_runs;
                        tex_runs += KIND == 2 || rs.tex_data != nullptr;
                        if constexpr (KIND == 2) {
                            float v[5];
#pragma unroll
                            for (int q = 0; q < 5; ++q)
                                v[q] = fadd(fadd(fmul(rvv[q], cmp[0]), fmul(rvv[5 + q], cmp[1])), fmul(rvv[10 + q], cmp[2]));
                            run_fs_rs(rs, v, s_lut, col);
                        } else {
                            const uint32_t nvar = rs.nvar;
                            float var[MAX_VARYING_FLOATS];
                            if (rs.interp == INTERP_PERSPECTIVE) {
                                const float den = fadd(fadd(fmul(cmp[0], r.inv_w0[0]), fmul(cmp[1], r.inv_w0[1])),
                                                       fmul(cmp[2], r.inv_w0[2]));
#pragma unroll
                                for (uint32_t qv = 0; qv < MAX_VARYING_FLOATS; ++qv) {
                                    if (qv >= nvar) break;
                                    float num = fmul(fmul(rv[qv], cmp[0]), r.inv_w0[0]);
                                    num = fadd(num, fmul(fmul(rv[nvar + qv], cmp[1]), r.inv_w0[1]));
                                    num = fadd(num, fmul(fmul(rv[2 * nvar + qv], cmp[2]), r.inv_w0[2]));
                                    var[qv] = fdiv(num, den);
                                }
                            } else {
#pragma unroll
                                for (uint32_t qv = 0; qv < MAX_VARYING_FLOATS; ++qv) {
                                    if (qv >= nvar) break;
                                    var[qv] = fadd(fadd(fmul(rv[qv], cmp[0]), fmul(rv[nvar + qv], cmp[1])),
                                                   fmul(rv[2 * nvar + qv], cmp[2]));
                                }
                            }
                            // @interpolate(flat): the first vertex's value, bits unchanged (fragment.rs:395-405)
                            if (rs.flat_mask) {
#pragma unroll
                                for (uint32_t qv = 0; qv < MAX_VARYING_FLOATS; ++qv)
                                    if (qv < nvar && ((rs.flat_mask >> qv) & 1u)) var[qv] = rv[qv];
                            }
                            if (!run_fs_any(bp, rs, r, cmp, var, s_lut, col)) continue;  // discard: no depth test, no write
                        }
                        // late depth test at the first colour output (fragment.rs:427-453, 470-479);
                        // with @early_depth_test(force) the early result stands (fragment.rs:185-191)
                        if (KIND == 2 || (KIND == 0 && rs.depth_test && rs.early_depth != EARLY_DEPTH_FORCE)) {
                            // fragment.z (raster.rs:345-346); only the depth test reads it here
                            const float z =
                                fadd(fadd(fmul(r.fz[0], cmp[0]), fmul(r.fz[1], cmp[1])), fmul(r.fz[2], cmp[2]));
                            if (!depth_compare(rs.depth_compare, z, px[k].depth)) continue;
                            if (rs.depth_write) px[k].depth = z;
                        }
                        if constexpr (KIND == 2) {
                            encode_color(3, col, px[k].c);  // Rgba8Unorm / Rgba8UnormSrgb: same bytes here
                        } else {
                            if (!tg.color) continue;
                            if (rs.blend_enabled && rs.blend_over) {
                                // the generic formula below with its factors resolved: s*sa + d*(1-sa), alpha s*1 + d*(1-sa)
                                const V4 dst = decode_color(tg.color_format, px[k].c);
                                const float oma = fsub(1.0f, col.w);
                                col = V4{fadd(fmul(col.x, col.w), fmul(dst.x, oma)), fadd(fmul(col.y, col.w), fmul(dst.y, oma)),
                                         fadd(fmul(col.z, col.w), fmul(dst.z, oma)), fadd(fmul(col.w, 1.0f), fmul(dst.w, oma))};
                            } else if (rs.blend_enabled) {
                                const V4 dst = decode_color(tg.color_format, px[k].c);
                                V4 o;
                                o.x = blend_channel(rs.blend_color, col.x, col.w, dst.x, dst.w, rs.blend_constant[0]);
                                o.y = blend_channel(rs.blend_color, col.y, col.w, dst.y, dst.w, rs.blend_constant[1]);
                                o.z = blend_channel(rs.blend_color, col.z, col.w, dst.z, dst.w, rs.blend_constant[2]);
                                o.w = blend_channel(rs.blend_alpha, col.w, col.w, dst.w, dst.w, rs.blend_constant[3]);
                                col = o;
                            }
                            if (rs.write_mask != 0xF) {
                                const V4 dst = decode_color(tg.color_format, px[k].c);
                                if (!(rs.write_mask & 1)) col.x = dst.x;
                                if (!(rs.write_mask & 2)) col.y = dst.y;
                                if (!(rs.write_mask & 4)) col.z = dst.z;
                                if (!(rs.write_mask & 8)) col.w = dst.w;
                            }
                            encode_color(tg.color_format, col, px[k].c);
                        }
                    }
                }
            }
            __syncthreads();
        }

        // write the tile back
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            if (!pvalid[k]) continue;
            const size_t pix = (size_t)pxy[k] * tg.width + pxx[k];
            if (tg.color) {
                uint8_t* dst = tg.color + tg.slice_offset + pix * tg.color_bpp;
                if (tg.color_bpp == 4) *reinterpret_cast<uint32_t*>(dst) = px[k].c[0];
                else if (tg.color_bpp == 8) { reinterpret_cast<uint2*>(dst)[0] = make_uint2(px[k].c[0], px[k].c[1]); }
                else if (tg.color_bpp == 16) { reinterpret_cast<uint4*>(dst)[0] = make_uint4(px[k].c[0], px[k].c[1], px[k].c[2], px[k].c[3]); }
                else if (tg.color_bpp == 2) *reinterpret_cast<uint16_t*>(dst) = (uint16_t)px[k].c[0];
                else *dst = (uint8_t)px[k].c[0];
            }
            if (tg.depth) tg.depth[pix] = px[k].depth;
        }
        for (int o = 16; o > 0; o >>= 1) {
            frag_count += __shfl_xor_sync(0xFFFFFFFFu, frag_count, o);
            fs_runs += __shfl_xor_sync(0xFFFFFFFFu, fs_runs, o);
            tex_runs += __shfl_xor_sync(0xFFFFFFFFu, tex_runs, o);
        }
        if (lane == 0 && frag_count) {
            atomicAdd(&s_frag, (unsigned long long)frag_count);
            if (tg.frag_count) {
                atomicAdd(tg.frag_count, (unsigned long long)frag_count);
                if (fs_runs) atomicAdd(tg.frag_count + 1, (unsigned long long)fs_runs);
                if (tex_runs) atomicAdd(tg.frag_count + 2, (unsigned long long)tex_runs);
            }
        }
        __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_frag) atomicAdd(&bp.status->fragments, s_frag);
}

}  // namespace gbr
