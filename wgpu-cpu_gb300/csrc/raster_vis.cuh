// raster_vis.cuh — visibility raster for opaque, depth-tested batches.
//
// The reference walks fragments in primitive order and runs the late depth test at the first
// colour output (render_pass/fragment.rs:427-453, 470-479).  When every draw into a target
// writes depth with one of Less / LessEqual / Greater / GreaterEqual, does not blend and
// never discards, the last fragment that passes at a pixel is determined without walking in
// order:
//
//   Less          the passing sequence has strictly falling depth; the survivor is the fragment
//                 of minimum depth, the earliest of those in order.
//   LessEqual     non-increasing depth; all fragments of minimum depth pass; the survivor is the
//                 latest of them.
//   Greater(Eq.)  the same with maximum depth.
//
// and it passes iff it passes against the stored depth (every other fragment lies on the far
// side of it).  So each fragment's (depth, order) is packed into one 64-bit key that orders it
// by that rule, the tile's keys are reduced with shared-memory atomicMin in any order, and the
// fragment stage runs once per pixel, for the survivor only.  Coverage, barycentrics and depth
// are computed with exactly the operations of the ordered kernel (raster.rs:129-363), so the
// colour, depth and fragment count come out identical; the count still includes every covered
// fragment, because the reference runs the fragment stage before the depth test.
//
// -0 and +0 compare equal in the depth test, so -0 is keyed as +0; a NaN depth fails all four
// comparisons and takes no part.
#pragma once

#include "raster.cuh"

namespace gbr {

// The record an order key names: sub-triangle 0 is the primitive's own record, the others are in
// the overflow area.
__device__ __forceinline__ const TriRecord* record_of(const BatchParams& bp, uint32_t key) {
    const uint32_t prim = key >> SUBTRI_BITS, sub = key & ((1u << SUBTRI_BITS) - 1u);
    const TriRecord* pr = rec_at(bp.records, bp.record_stride, prim);
    return sub == 0 ? pr : rec_at(bp.ovf_records, bp.record_stride, __ldg(&pr->ovf) + sub - 1);
}

// Per-record constants of the barycentric evaluation (the same terms the ordered kernel keeps in
// shared memory).
struct BaryK {
    float ax, ay, bx, by, cx, cy;
    float kc0, kc1, kc2, rcp, area;
    bool area_ok, ident;
};

__device__ __forceinline__ void bary_consts(const TriRecord& r, BaryK& k) {
    k.ax = r.vpx[0]; k.ay = r.vpy[0];
    k.bx = r.vpx[1]; k.by = r.vpy[1];
    k.cx = r.vpx[2]; k.cy = r.vpy[2];
    k.kc0 = fmul(fsub(k.cy, k.by), fadd(k.cx, k.bx));
    k.kc1 = fmul(fsub(k.ay, k.cy), fadd(k.ax, k.cx));
    k.kc2 = fmul(fsub(k.by, k.ay), fadd(k.bx, k.ax));
    k.area = r.area;
    k.rcp = __frcp_rn(k.area);
    k.area_ok = div_fast_ok(k.area);
    k.ident = (r.flags & 16u) != 0;
}

// bary_consts from the record's header words 0, 3, 4 and 5 (16-byte loads: flags, viewport
// vertices, area).
__device__ __forceinline__ void bary_consts_words(uint4 h0, uint4 h3, uint4 h4, uint4 h5, BaryK& k) {
    k.ax = __uint_as_float(h3.z); k.bx = __uint_as_float(h3.w); k.cx = __uint_as_float(h4.x);
    k.ay = __uint_as_float(h4.y); k.by = __uint_as_float(h4.z); k.cy = __uint_as_float(h4.w);
    k.kc0 = fmul(fsub(k.cy, k.by), fadd(k.cx, k.bx));
    k.kc1 = fmul(fsub(k.ay, k.cy), fadd(k.ax, k.cx));
    k.kc2 = fmul(fsub(k.by, k.ay), fadd(k.bx, k.ax));
    k.area = __uint_as_float(h5.x);
    k.rcp = __frcp_rn(k.area);
    k.area_ok = div_fast_ok(k.area);
    k.ident = (h0.w & 16u) != 0;
}

// Barycentrics at the integer pixel corner (the edge-function rule: the pixel centre) composed
// with the clip barycentrics (raster.rs:313-321, 334-343), as in k_raster.  get_cb() returns the
// record's clip barycentrics; it is called only for a clipped record (k.ident false), an
// unclipped one composes with the unit vectors it holds.
template <bool EDGE, class GetCb>
__device__ __forceinline__ void bary_eval(const BaryK& k, int x, int y, float cmp[3], GetCb get_cb) {
    // an IEEE sum does not depend on operand order: x + a.x serves both terms containing it
    // The operations of the scalar formulas, sums and differences two lanes per packed f32x2
    // instruction (exact per lane; products scalar, see f2mul_rn); a - b is a + (-b).
    const float fx = EDGE ? fadd((float)x, 0.5f) : (float)x, fy = EDGE ? fadd((float)y, 0.5f) : (float)y;
    const float2 xab = f2add(make_float2(fx, fx), make_float2(k.ax, k.bx));
    const float xa = xab.x, xb = xab.y, xc = fadd(fx, k.cx);
    // s0 = ((b.y - y) (x + b.x) + kc0) + (y - c.y) (x + c.x); s2 = (kc2 + (y - b.y) (x + b.x)) + (a.y - y) (x + a.x)
    const float2 d02 = f2add(make_float2(k.by, fy), make_float2(-fy, -k.by));
    const float2 t02 = f2add(f2mul_rn(d02, make_float2(xb, xb)), make_float2(k.kc0, k.kc2));
    const float2 e02 = f2add(make_float2(fy, k.ay), make_float2(-k.cy, -fy));
    const float2 s02 = f2add(t02, f2mul_rn(e02, make_float2(xc, xa)));
    // s1 = ((y - a.y) (x + a.x) + (c.y - y) (x + c.x)) + kc1
    const float2 e1 = f2add(make_float2(fy, k.cy), make_float2(-k.ay, -fy));
    const float2 m1 = f2mul_rn(e1, make_float2(xa, xc));
    const float s1 = fadd(fadd(m1.x, m1.y), k.kc1);
    if (k.area_ok && div_fast_ok(s02.x) && div_fast_ok(s1) && div_fast_ok(s02.y)) {
        // div_by_recip's in-range path for s0 and s2 together
        const float2 y2 = make_float2(k.rcp, k.rcp), nb2 = make_float2(-k.area, -k.area);
        float2 q = f2mul(s02, y2);
        float2 rr = f2fma(nb2, q, s02);
        q = f2fma(rr, y2, q);
        rr = f2fma(nb2, q, s02);
        const float2 l02 = f2fma(rr, y2, q);
        const float l1 = div_by_recip(s1, k.area, k.rcp, true);
        if (k.ident) {
            cmp[0] = l02.x;
            cmp[1] = l1;
            cmp[2] = l02.y;
            return;
        }
        const float* cb = get_cb();
#pragma unroll
        for (int j = 0; j < 3; ++j)
            cmp[j] = fadd(fadd(fmul(cb[j], l02.x), fmul(cb[3 + j], l1)), fmul(cb[6 + j], l02.y));
        return;
    }
    const float l0 = div_by_recip(s02.x, k.area, k.rcp, k.area_ok);
    const float l1 = div_by_recip(s1, k.area, k.rcp, k.area_ok);
    const float l2 = div_by_recip(s02.y, k.area, k.rcp, k.area_ok);
    if (k.ident) {  // the same operations with the unit vectors (a non-finite l makes 0 * l a NaN)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            cmp[j] = fadd(fadd(fmul(j == 0 ? 1.0f : 0.0f, l0), fmul(j == 1 ? 1.0f : 0.0f, l1)),
                          fmul(j == 2 ? 1.0f : 0.0f, l2));
        return;
    }
    const float* cb = get_cb();
#pragma unroll
    for (int j = 0; j < 3; ++j) cmp[j] = fadd(fadd(fmul(cb[j], l0), fmul(cb[3 + j], l1)), fmul(cb[6 + j], l2));
}
template <bool EDGE>
__device__ __forceinline__ void bary_at(const TriRecord& r, const BaryK& k, int x, int y, float cmp[3]) {
    bary_eval<EDGE>(k, x, y, cmp, [&] { return r.cb; });
}

__device__ __forceinline__ float frag_z(const TriRecord& r, const float cmp[3]) {  // raster.rs:345-346
    return fadd(fadd(fmul(r.fz[0], cmp[0]), fmul(r.fz[1], cmp[1])), fmul(r.fz[2], cmp[2]));
}

// Monotone map of a float onto u32 (as integers, the keys order like the floats), -0 as +0.
__device__ __forceinline__ uint32_t depth_order_bits(float z) {
    const uint32_t u = __float_as_uint(z == 0.0f ? 0.0f : z);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Survivor key (smaller wins) of a fragment at depth z with order key `order`.
__device__ __forceinline__ unsigned long long vis_key(uint32_t cmpf, float z, uint32_t order) {
    uint32_t d = depth_order_bits(z);
    if (cmpf == 5u || cmpf == 7u) d = ~d;                           // Greater(Equal): the deepest
    const uint32_t o = (cmpf == 4u || cmpf == 7u) ? ~order : order;  // *Equal: the latest of a tie
    return ((unsigned long long)d << 32) | o;
}
__device__ __forceinline__ uint32_t vis_order(uint32_t cmpf, unsigned long long key) {
    const uint32_t o = (uint32_t)key;
    return (cmpf == 4u || cmpf == 7u) ? ~o : o;
}

template <int WARPS>
__device__ __forceinline__ void tile_sync() {
    if constexpr (WARPS == 1) __syncwarp();
    else __syncthreads();
}

// One CTA per tile (persistent); a CTA of one warp synchronises with __syncwarp only, so many
// independent tiles share an SM and hide each other's memory latency.
// Phase 1: the row segments of the tile's records are dealt to lanes (one span per segment), each
// covered fragment atomicMin-ing its key into the tile's key array.  Phase 2: one thread per
// pixel re-evaluates the survivor's barycentrics, tests it against the stored depth, runs the
// fragment stage and writes colour and depth.
// Work items: first the chunks of the split tiles (split_chunk records each; k_scan lists them), then every tile that is not split.  A chunk runs phase 1 over its records only and stores
// its key array in its own global slot; the chunk that finishes last (a per-tile ticket) takes
// the minimum over the tile's slots, which is the key array of the whole tile since the survivor
// key is a minimum, and runs phase 2.  No CTA waits for another.
template <int T, int WARPS, bool EDGE = false>
__global__ void __launch_bounds__(WARPS * 32, 32 / WARPS) k_raster_vis(BatchParams bp) {
    constexpr int NT = WARPS * 32, NPIX = T * T;
    constexpr unsigned long long kNone = ~0ull;
    __shared__ unsigned long long s_vis[NPIX];
    __shared__ float s_lut[256];
    // phase 1: the record table of the chunk being rasterised (per thread: record, key, clipped box,
    // exclusive prefix of the row counts) and the warps' partial sums
    // rows of the record: first row, pixel range clipped to tile and scissor, first row in the chunk
    __shared__ int4 s_box[NT];
    // per record of the chunk: barycentric terms (a, b, c, the three shoelace constants, 1/area,
    // area), vertex depths, flags (bit 0 area in the fast-division range, bit 1 unclipped) and
    // order key; the span rule's sorted vertices (the degenerate row's extent and -1 instead of
    // the first two when all three lie on one row)
    __shared__ float4 s_b0[NT], s_b1[NT], s_b2[NT], s_b3[NT];
    __shared__ int4 s_sp0[NT];
    __shared__ int2 s_sp1[NT];
    // a wave of the chunk's rows: the record of each, (record | row << 8 | first pixel << 16) and
    // the exclusive prefix of their covered widths; the row of each pixel of a block of PIXB
    constexpr int WAVE = 2 * NT, PIXB = 8 * NT;
    __shared__ uint8_t s_rrec[WAVE];
    __shared__ uint32_t s_row[WAVE], s_pre[WAVE];
    __shared__ uint16_t s_pix[PIXB];
    __shared__ uint32_t s_wsum[WARPS];
    __shared__ uint32_t s_tile, s_last;
    __shared__ uint2 s_runs;  // fragment-stage runs of the tile, and those that sample a texture
    __shared__ unsigned long long s_frag;

    const int lane = threadIdx.x & 31;
    const bool failed = bp.status->error != 0 || *bp.abort_flag != 0;
    if (failed && blockIdx.x == 0 && threadIdx.x == 0) *bp.abort_flag = 1u;
    for (int i = threadIdx.x; i < 256; i += NT) s_lut[i] = fdiv((float)i, 255.0f);  // `x as f32 / 255.0`
    if (threadIdx.x == 0) s_frag = 0;
    const uint32_t cmpf = bp.vis_compare;
    const RasterState* states = static_cast<const RasterState*>(bp.states);
    const uint32_t n_split = bp.split_heavy ? bp.status->split_items : 0u;  // written by k_scan

    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(bp.work_counter, 1u);
        for (int p = threadIdx.x; p < NPIX; p += NT) s_vis[p] = kNone;
        tile_sync<WARPS>();
        const uint32_t item = s_tile;
        if (failed) break;
        uint32_t tile, heavy = ~0u, r_begin = 0, r_end;
        if (item < n_split) {  // a chunk of a split tile
            heavy = bp.split_item[item];
            const uint32_t* e = bp.split_heavy + 4 * (size_t)heavy;
            tile = e[0];
            r_begin = (item - e[2]) * bp.split_chunk;
            r_end = min(bp.tile_count[tile], r_begin + bp.split_chunk);
        } else {
            tile = item - n_split;
            if (tile >= bp.total_tiles) break;
            r_end = bp.tile_count[tile];
            if (n_split && r_end > bp.split_chunk && bp.split_tile[tile] != ~0u) {
                tile_sync<WARPS>();  // s_tile is rewritten at the top
                continue;            // its chunks rasterise it
            }
        }
        const uint32_t ti = find_target(bp.targets, bp.num_targets, tile);
        const TargetDesc& tg = bp.targets[ti];
        const uint32_t lt = tile - tg.tile_base;
        const int X0 = (int)(lt % tg.tiles_x) * T, Y0 = (int)(lt / tg.tiles_x) * T;
        const int XE = min(X0 + T, (int)tg.width) - 1, YE = min(Y0 + T, (int)tg.height) - 1;
        const uint32_t off = bp.tile_offset[tile];
        uint32_t frag_count = 0;

        // phase 1: coverage and survivor keys.  The CTA takes the tile's records NT at a time;
        // each thread stages its record's constants in shared memory once (the span rule's sorted
        // framebuffer vertices, the barycentric terms, the vertex depths) and counts its rows
        // clipped to tile and scissor.  The chunk's rows are then processed in waves of WAVE rows:
        // (a) every thread takes WAVE / NT consecutive rows, computes each row's span once and
        // stores it (record, row, first pixel, width); (b) a block scan of the widths deals the
        // wave's covered pixels to the threads in equal, contiguous ranges, so every lane of a warp
        // evaluates the same number of fragments (barycentrics, depth, survivor atomicMin).
        constexpr unsigned kFull = 0xFFFFFFFFu;
        constexpr int RPT = WAVE / NT;  // rows per thread and wave
        const int warp = (int)(threadIdx.x >> 5);
        // exclusive block scan of v (one value per thread); returns the prefix, *tot the sum
        auto block_scan = [&](uint32_t v, uint32_t* tot) -> uint32_t {
            uint32_t incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += u;
            }
            if (lane == 31) s_wsum[warp] = incl;
            tile_sync<WARPS>();
            uint32_t woff = 0, total = 0;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) {
                const uint32_t ws = s_wsum[w];
                woff += w < warp ? ws : 0u;
                total += ws;
            }
            *tot = total;
            return woff + incl - v;
        };
        for (uint32_t c0 = r_begin; c0 < r_end; c0 += NT) {
            const uint32_t i = c0 + threadIdx.x;
            uint32_t rows = 0;
            if (i < r_end) {
                const uint32_t key = bp.bins[off + i];
                // the record's first 96 bytes (order, draw, flags, rows, sorted vertices, viewport
                // vertices, area, vertex depths) as six 16-byte loads, the draw's scissor as two
                const uint4* rv = reinterpret_cast<const uint4*>(record_of(bp, key));
                const uint4 h0 = __ldg(rv), h1 = __ldg(rv + 1), h2 = __ldg(rv + 2), h3 = __ldg(rv + 3),
                            h4 = __ldg(rv + 4), h5 = __ldg(rv + 5);
                const uint2* sc = reinterpret_cast<const uint2*>(&bp.draws[h0.y].sc_x0);
                const uint2 sc0 = __ldg(sc), sc1 = __ldg(sc + 1);  // (x0, y0), (x1, y1)
                const int y0 = max(max((int)h1.x, Y0), (int)sc0.y);
                const int y1 = min(min((int)h1.y, YE), (int)sc1.y - 1);
                const int xl = max(max((int)h1.z, X0), (int)sc0.x);
                const int xr = min(min((int)h1.w, XE), (int)sc1.x - 1);
                if (y1 >= y0 && xr >= xl) {
                    rows = (uint32_t)(y1 - y0 + 1);
                    BaryK k;
                    bary_consts_words(h0, h3, h4, h5, k);
                    s_b0[threadIdx.x] = make_float4(k.ax, k.ay, k.bx, k.by);
                    s_b1[threadIdx.x] = make_float4(k.cx, k.cy, k.kc0, k.kc1);
                    s_b2[threadIdx.x] = make_float4(k.kc2, k.rcp, k.area, __uint_as_float(h5.y));
                    const int fl = (k.area_ok ? 1 : 0) | (k.ident ? 2 : 0);
                    s_b3[threadIdx.x] = make_float4(__uint_as_float(h5.z), __uint_as_float(h5.w), __int_as_float(fl),
                                                    __uint_as_float(key));
                    if (!EDGE) {  // the span rule's rows (the framebuffer coordinates are >= 0)
                        if (h0.w & (SPAN_DEGENERATE << 2))
                            s_sp0[threadIdx.x] = make_int4((int)h1.z, (int)h1.w, -1, -1);
                        else
                            s_sp0[threadIdx.x] = make_int4((int)h2.x, (int)h2.w, (int)h2.y, (int)h3.x);
                        s_sp1[threadIdx.x] = make_int2((int)h2.z, (int)h3.y);
                    }
                    s_box[threadIdx.x] = make_int4(y0, xl, xr, 0);
                }
            }
            uint32_t total_rows;
            const uint32_t excl = block_scan(rows, &total_rows);  // this record's first row in the chunk
            if (rows) s_box[threadIdx.x].w = (int)excl;
            for (uint32_t w0 = 0; w0 < total_rows; w0 += WAVE) {
                // (0) the record of each row of the wave
                {
                    const uint32_t q1 = min(excl + rows, w0 + WAVE);
                    for (uint32_t q = max(excl, w0); q < q1; ++q) s_rrec[q - w0] = (uint8_t)threadIdx.x;
                }
                tile_sync<WARPS>();
                // (a) spans of this thread's rows [q0, q0 + RPT) of the wave
                const uint32_t q0 = (uint32_t)threadIdx.x * RPT;
                uint32_t widths = 0;
                uint32_t ent[RPT], wid[RPT];
#pragma unroll
                for (int k = 0; k < RPT; ++k) {
                    ent[k] = 0;
                    wid[k] = 0;
                    if (w0 + q0 + k < total_rows) {
                        const int j = s_rrec[q0 + k];
                        const int4 bx = s_box[j];
                        const int y = bx.x + (int)(w0 + q0 + k - (uint32_t)bx.w);
                        int x1, x2;
                        if constexpr (EDGE) {
                            span_at<EDGE>(*record_of(bp, __float_as_uint(s_b3[j].w)), y, x1, x2);
                        } else {
                            const int4 sp0 = s_sp0[j];
                            if (sp0.w < 0) {
                                x1 = sp0.x;
                                x2 = sp0.y;
                            } else {
                                const int2 sp1 = s_sp1[j];
                                span_rows(sp0.x, sp0.y, sp0.z, sp0.w, sp1.x, sp1.y, y, x1, x2);
                            }
                        }
                        x1 = max(x1, bx.y);
                        x2 = min(x2, bx.z);
                        if (x1 <= x2) {
                            wid[k] = (uint32_t)(x2 - x1 + 1);
                            ent[k] = (uint32_t)j | ((uint32_t)(y - Y0) << 8) | ((uint32_t)(x1 - X0) << 16);
                        }
                    }
                    widths += wid[k];
                }
                uint32_t total_px;
                uint32_t pre = block_scan(widths, &total_px);
                uint32_t pre_k[RPT];
#pragma unroll
                for (int k = 0; k < RPT; ++k) {
                    pre_k[k] = pre;
                    s_row[q0 + k] = ent[k];
                    s_pre[q0 + k] = pre;
                    pre += wid[k];
                }
                // (b) the wave's covered pixels in blocks of PIXB: a table gives each pixel its row,
                // and thread t takes pixels t, t + NT, ... of the block, so the lanes of a warp work
                // on neighbouring pixels of the same few rows (shared constants, no divergence)
                for (uint32_t b0 = 0; b0 < total_px; b0 += PIXB) {
#pragma unroll
                    for (int k = 0; k < RPT; ++k) {
                        const uint32_t u1 = min(pre_k[k] + wid[k], b0 + PIXB);
                        for (uint32_t u = max(pre_k[k], b0); u < u1; ++u) s_pix[u - b0] = (uint16_t)(q0 + k);
                    }
                    tile_sync<WARPS>();
                    const uint32_t nb = min((uint32_t)PIXB, total_px - b0);
                    for (uint32_t i = threadIdx.x; i < nb; i += NT) {
                        const uint32_t q = s_pix[i];
                        const uint32_t e = s_row[q];
                        const int jj = (int)(e & 0xFFu), y = Y0 + (int)((e >> 8) & 0xFFu);
                        const int x = X0 + (int)(e >> 16) + (int)(b0 + i - s_pre[q]);
                        const float4 b0v = s_b0[jj], b1 = s_b1[jj], b2 = s_b2[jj], b3 = s_b3[jj];
                        const int fl = __float_as_int(b3.z);
                        BaryK k;
                        k.ax = b0v.x; k.ay = b0v.y; k.bx = b0v.z; k.by = b0v.w;
                        k.cx = b1.x; k.cy = b1.y; k.kc0 = b1.z; k.kc1 = b1.w;
                        k.kc2 = b2.x; k.rcp = b2.y; k.area = b2.z;
                        k.area_ok = (fl & 1) != 0;
                        k.ident = (fl & 2) != 0;
                        float cmp[3];
                        const uint32_t rkey = __float_as_uint(b3.w);
                        bary_eval<EDGE>(k, x, y, cmp, [&] { return record_of(bp, rkey)->cb; });
                        ++frag_count;
                        // fragment.z (raster.rs:345-346) from the staged vertex depths
                        const float z = fadd(fadd(fmul(b2.w, cmp[0]), fmul(b3.x, cmp[1])), fmul(b3.y, cmp[2]));
                        if (z != z) continue;
                        atomicMin(&s_vis[(y - Y0) * T + (x - X0)], vis_key(cmpf, z, rkey));
                    }
                    tile_sync<WARPS>();  // the block's table (and after the last, the wave's rows) is rewritten
                }
            }
        }
        tile_sync<WARPS>();
        for (int o = 16; o > 0; o >>= 1) frag_count += __shfl_xor_sync(0xFFFFFFFFu, frag_count, o);
        if (lane == 0 && frag_count) {
            atomicAdd(&s_frag, (unsigned long long)frag_count);
            if (tg.frag_count) atomicAdd(tg.frag_count, (unsigned long long)frag_count);
        }

        if (heavy != ~0u) {
            // a chunk: its keys to its slot; the last of the tile's chunks merges them all
            unsigned long long* slot = bp.split_keys + (size_t)item * NPIX;
            for (int p = threadIdx.x; p < NPIX; p += NT) slot[p] = s_vis[p];
            __threadfence();
            tile_sync<WARPS>();
            uint32_t* e = bp.split_heavy + 4 * (size_t)heavy;
            if (threadIdx.x == 0) {
                s_last = atomicAdd(&e[3], 1u) == e[1] - 1u;
                __threadfence();
            }
            tile_sync<WARPS>();
            if (!s_last) continue;  // no shared state is read past the barrier above
            const unsigned long long* slots = bp.split_keys + (size_t)e[2] * NPIX;
            const uint32_t chunks = e[1];
            for (int p = threadIdx.x; p < NPIX; p += NT) {
                unsigned long long m = kNone;
                uint32_t c = 0;
                for (; c + 8 <= chunks; c += 8) {  // eight independent loads in flight
                    unsigned long long v[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) v[u] = __ldcg(slots + (size_t)(c + u) * NPIX + p);
#pragma unroll
                    for (int u = 0; u < 8; ++u) m = min(m, v[u]);
                }
                for (; c < chunks; ++c) m = min(m, __ldcg(slots + (size_t)c * NPIX + p));
                s_vis[p] = m;
            }
            tile_sync<WARPS>();
        }

        // phase 2: the survivor of each pixel against the stored depth, fragment stage, write-back
        uint32_t clear_c[4] = {0, 0, 0, 0};
        encode_color(tg.color_format, V4{tg.clear[0], tg.clear[1], tg.clear[2], tg.clear[3]}, clear_c);
        if (threadIdx.x == 0) s_runs = make_uint2(0u, 0u);
        tile_sync<WARPS>();
        for (int p = threadIdx.x; p < NPIX; p += NT) {
            const int x = X0 + (p % T), y = Y0 + (p / T);
            // fragment-stage runs of this pass over the tile's pixels, counted per warp below
            bool ran = false, sampled = false;
            if (x <= XE && y <= YE) {
            const size_t pix = (size_t)y * tg.width + x;
            const unsigned long long key = s_vis[p];
            uint8_t* cdst = tg.color + tg.slice_offset + pix * tg.color_bpp;
            uint32_t c[4] = {clear_c[0], clear_c[1], clear_c[2], clear_c[3]};
            const bool load_color = tg.color_load != 1;
            float depth = tg.depth_load != 1 ? tg.depth[pix] : tg.depth_clear;
            bool write_color = !load_color;  // a cleared target is written even where nothing lands
            bool write_depth = tg.depth_load == 1;
            if (key != kNone) {
                const TriRecord& r = *record_of(bp, vis_order(cmpf, key));
                const uint4* rv4 = reinterpret_cast<const uint4*>(&r);
                const uint4 h0 = __ldg(rv4), h3 = __ldg(rv4 + 3), h4 = __ldg(rv4 + 4), h5 = __ldg(rv4 + 5);
                BaryK k;
                bary_consts_words(h0, h3, h4, h5, k);
                float cmp[3];
                bary_at<EDGE>(r, k, x, y, cmp);
                // fragment.z (raster.rs:345-346)
                const float z = fadd(fadd(fmul(__uint_as_float(h5.y), cmp[0]), fmul(__uint_as_float(h5.z), cmp[1])),
                                     fmul(__uint_as_float(h5.w), cmp[2]));
                if (depth_compare(cmpf, z, depth)) {
                    const RasterState& rs = states[h0.y];
                    const uint32_t nvar = rs.nvar;
                    const float* rv = rec_var(&r);
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
                            // @interpolate(flat): the first vertex's value, bits unchanged
                            const float v0 = rv[qv];
                            var[qv] = ((rs.flat_mask >> qv) & 1u)
                                          ? v0
                                          : fadd(fadd(fmul(v0, cmp[0]), fmul(rv[nvar + qv], cmp[1])),
                                                 fmul(rv[2 * nvar + qv], cmp[2]));
                        }
                    }
                    V4 col;
                    ran = true;
                    sampled = rs.tex_data != nullptr;
                    run_fs_any(bp, rs, r, cmp, var, s_lut, col);  // eligible programs never discard
                    if (rs.write_mask != 0xF) {
                        uint32_t dc[4] = {c[0], c[1], c[2], c[3]};
                        if (load_color) {
                            for (uint32_t q = 0; q < 4; ++q) dc[q] = 0;
                            if (tg.color_bpp == 4) dc[0] = *reinterpret_cast<const uint32_t*>(cdst);
                            else if (tg.color_bpp == 8) { dc[0] = reinterpret_cast<const uint32_t*>(cdst)[0]; dc[1] = reinterpret_cast<const uint32_t*>(cdst)[1]; }
                            else if (tg.color_bpp == 16) { for (int q = 0; q < 4; ++q) dc[q] = reinterpret_cast<const uint32_t*>(cdst)[q]; }
                            else if (tg.color_bpp == 2) dc[0] = *reinterpret_cast<const uint16_t*>(cdst);
                            else dc[0] = *cdst;
                        }
                        const V4 dst = decode_color(tg.color_format, dc);
                        if (!(rs.write_mask & 1)) col.x = dst.x;
                        if (!(rs.write_mask & 2)) col.y = dst.y;
                        if (!(rs.write_mask & 4)) col.z = dst.z;
                        if (!(rs.write_mask & 8)) col.w = dst.w;
                    }
                    encode_color(tg.color_format, col, c);
                    write_color = true;
                    depth = z;
                    write_depth = true;
                }
            }
            if (write_color) {
                if (tg.color_bpp == 4) *reinterpret_cast<uint32_t*>(cdst) = c[0];
                else if (tg.color_bpp == 8) reinterpret_cast<uint2*>(cdst)[0] = make_uint2(c[0], c[1]);
                else if (tg.color_bpp == 16) reinterpret_cast<uint4*>(cdst)[0] = make_uint4(c[0], c[1], c[2], c[3]);
                else if (tg.color_bpp == 2) *reinterpret_cast<uint16_t*>(cdst) = (uint16_t)c[0];
                else *cdst = (uint8_t)c[0];
            }
            if (write_depth) tg.depth[pix] = depth;
            }
            const uint32_t mr = __ballot_sync(0xFFFFFFFFu, ran), ms = __ballot_sync(0xFFFFFFFFu, sampled);
            if (lane == 0 && mr) {
                atomicAdd(&s_runs.x, (uint32_t)__popc(mr));
                atomicAdd(&s_runs.y, (uint32_t)__popc(ms));
            }
        }
        tile_sync<WARPS>();
        if (threadIdx.x == 0 && s_runs.x && tg.frag_count) {
            atomicAdd(tg.frag_count + 1, (unsigned long long)s_runs.x);
            if (s_runs.y) atomicAdd(tg.frag_count + 2, (unsigned long long)s_runs.y);
        }
        tile_sync<WARPS>();
    }
    tile_sync<WARPS>();
    if (threadIdx.x == 0 && s_frag) atomicAdd(&bp.status->fragments, s_frag);
}

// Per-draw fragment-stage state for k_raster_vis, built once per batch.
// (a template only so that both kernel translation units can instantiate it)
template <int = 0>
__global__ void k_build_states(BatchParams bp) {
    RasterState* states = static_cast<RasterState*>(bp.states);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < bp.num_draws; i += gridDim.x * blockDim.x)
        build_raster_state(bp.draws[i], i, states[i]);
}

}  // namespace gbr
