// TEST INFRASTRUCTURE — the oracle.  Not part of the product: only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline leg load it, as the checker.
//
// orc_core.hpp — a CPU restatement of wgpu-cpu's render-pass arithmetic, stage by stage, in the
// reference's own order of operations.  Every function cites the reference file:line it
// follows (paths relative to the wgpu-cpu repository).  Built with -ffp-contract=off and
// without -ffast-math so that every float operation is one IEEE-754 binary32 operation, as in
// the reference's Rust (which never contracts multiply-adds).
//
// Third-party arithmetic restated here (the crates are not vendored with the reference):
//  - nalgebra 0.34.1 `Matrix::dot` for 4-vectors (src/base/blas.rs, `dotx`): products
//    p0..p3, then (p0 + p2) + (p1 + p3).
//  - nalgebra `Point3::from_homogeneous`: xyz / w (three divisions); None when w == 0.
//  - nalgebra `Vector3::cross`: z = a.x*b.y - a.y*b.x.
//  - simba's f32 -> u32 subset cast used by `try_cast::<u32>()`: Rust `as u32` (saturating,
//    NaN -> 0).
//  - Rust `f32::max(x, 0.0)`: returns 0.0 for NaN.  Whether (-0.0).max(0.0) is +0.0 or -0.0 is
//    platform-dependent in Rust; this restatement returns +0.0 (IEEE 754-2019 maximumNumber,
//    the aarch64 `fmaxnm` result).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <vector>

namespace orc {

struct V4 {
    float x, y, z, w;
};

static inline V4 v4_mul(V4 a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
static inline V4 v4_add(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }

// nalgebra 0.34.1 blas.rs `dotx`, 4-vector special case.
static inline float dot4(V4 a, V4 b) {
    float p0 = a.x * b.x;
    float p1 = a.y * b.y;
    float p2 = a.z * b.z;
    float p3 = a.w * b.w;
    p0 += p2;
    p1 += p3;
    return p0 + p1;
}

// Rust `f32::max(v, 0.0)` (raster.rs:150-151).
static inline float rust_max0(float v) { return v > 0.0f ? v : 0.0f; }

// Rust `v as u32` for f32 (saturating, NaN -> 0).
static inline uint32_t rust_f32_to_u32(float v) {
    if (!(v > 0.0f)) return 0u;  // NaN, negatives, zeros
    if (v >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}
// Rust `v as u8` for f32 (saturating, NaN -> 0).
static inline uint8_t rust_f32_to_u8(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 256.0f) return 255u;
    return (uint8_t)v;
}

// ------------------------------------------------------------------------------------------
// Barycentric<3> (util/interpolation.rs:127-183)
struct Bary3 {
    float c[3];
};
static inline Bary3 bary_at_vertex(int i) {  // interpolation.rs:133-139
    Bary3 b{{0.0f, 0.0f, 0.0f}};
    b.c[i] = 1.0f;
    return b;
}

// `Barycentric::interpolate` (interpolation.rs:149-163): accu = p0*c0; accu = accu + p1*c1; ...
static inline float interp3(const float p[3], const Bary3& k) {
    float accu = p[0] * k.c[0];
    accu = accu + p[1] * k.c[1];
    accu = accu + p[2] * k.c[2];
    return accu;
}
static inline V4 interp3_v4(const V4 p[3], const Bary3& k) {
    V4 accu = v4_mul(p[0], k.c[0]);
    accu = v4_add(accu, v4_mul(p[1], k.c[1]));
    accu = v4_add(accu, v4_mul(p[2], k.c[2]));
    return accu;
}
// Barycentric<3> composed with clip barycentrics: points are Barycentric<3> values
// (raster.rs:338-343 -> interpolation.rs:149-163 with T = Barycentric<3>, whose Mul<f32> and
// Add are component-wise, interpolation.rs:165-183).
static inline Bary3 compose_bary(const Bary3 pts[3], const Bary3& k) {
    Bary3 r;
    for (int j = 0; j < 3; ++j) {
        float accu = pts[0].c[j] * k.c[0];
        accu = accu + pts[1].c[j] * k.c[1];
        accu = accu + pts[2].c[j] * k.c[2];
        r.c[j] = accu;
    }
    return r;
}

// `lerp(x0, x1, t) = x0 * (1.0 - t) + x1 * t` (interpolation.rs:84-89)
static inline float lerpf(float x0, float x1, float t) { return x0 * (1.0f - t) + x1 * t; }

// ------------------------------------------------------------------------------------------
// Clip volume (render_pass/clipper.rs:150-163): point is outside a plane if dot(point, n) < 0.
static const V4 kClipPlanes[6] = {
    {1.0f, 0.0f, 0.0f, 1.0f},   // left:   x < -w
    {-1.0f, 0.0f, 0.0f, 1.0f},  // right:  x >  w
    {0.0f, 1.0f, 0.0f, 1.0f},   // bottom: y < -w
    {0.0f, -1.0f, 0.0f, 1.0f},  // top:    y >  w
    {0.0f, 0.0f, 1.0f, 0.0f},   // front:  z <  0
    {0.0f, 0.0f, -1.0f, 1.0f},  // back:   z >  w
};

// tri_clip::Vertex (clipper.rs:590-613)
struct ClipVertex {
    V4 position;
    Bary3 bary;
};
// lerp(vertices[i], vertices[j], t) on tri_clip::Vertex: Mul<f32> and Add act on position and
// barycentric component-wise (clipper.rs:593-613, interpolation.rs:84-89).
static inline ClipVertex clip_vertex_lerp(const ClipVertex& a, const ClipVertex& b, float t) {
    float omt = 1.0f - t;
    ClipVertex r;
    r.position = v4_add(v4_mul(a.position, omt), v4_mul(b.position, t));
    for (int k = 0; k < 3; ++k) r.bary.c[k] = a.bary.c[k] * omt + b.bary.c[k] * t;
    return r;
}

struct ClipTri {
    ClipVertex v[3];
};

// clip_tri_against_plane (clipper.rs:625-728): the case table and output vertex orders.
static inline int clip_tri_against_plane(const ClipTri& tri, V4 plane, ClipTri out[2]) {
    float d[3];
    for (int i = 0; i < 3; ++i) d[i] = dot4(tri.v[i].position, plane);
    bool o0 = d[0] < 0.0f, o1 = d[1] < 0.0f, o2 = d[2] < 0.0f;
    auto clip = [&](int i, int j) {
        float t = d[i] / (d[i] - d[j]);
        return clip_vertex_lerp(tri.v[i], tri.v[j], t);
    };
    const ClipVertex& A = tri.v[0];
    const ClipVertex& B = tri.v[1];
    const ClipVertex& C = tri.v[2];
    if (o0 && o1 && o2) return 0;
    if (!o0 && !o1 && !o2) {
        out[0] = tri;
        return 1;
    }
    if (o0 && o1 && !o2) {  // A out, B out, C in: [A', B', C], A' = clip(2,0), B' = clip(1,2)
        ClipVertex a_new = clip(2, 0);
        ClipVertex b_new = clip(1, 2);
        out[0] = {{a_new, b_new, C}};
        return 1;
    }
    if (!o0 && o1 && o2) {  // A in: [A, B', C'], B' = clip(0,1), C' = clip(2,0)
        ClipVertex b_new = clip(0, 1);
        ClipVertex c_new = clip(2, 0);
        out[0] = {{A, b_new, c_new}};
        return 1;
    }
    if (o0 && !o1 && o2) {  // B in: [A', B, C'], A' = clip(0,1), C' = clip(1,2)
        ClipVertex a_new = clip(0, 1);
        ClipVertex c_new = clip(1, 2);
        out[0] = {{a_new, B, c_new}};
        return 1;
    }
    if (o0 && !o1 && !o2) {  // A out: [B', B, C'], [B, C, C'], B' = clip(0,1), C' = clip(0,2)
        ClipVertex b_new = clip(0, 1);
        ClipVertex c_new = clip(0, 2);
        out[0] = {{b_new, B, c_new}};
        out[1] = {{B, C, c_new}};
        return 2;
    }
    if (!o0 && o1 && !o2) {  // B out: [A, A', C'], [A, C', C], A' = clip(0,1), C' = clip(1,2)
        ClipVertex a_new = clip(0, 1);
        ClipVertex c_new = clip(1, 2);
        out[0] = {{A, a_new, c_new}};
        out[1] = {{A, c_new, C}};
        return 2;
    }
    // C out: [A, B, B'], [A, B', A'], B' = clip(1,2), A' = clip(0,2)
    ClipVertex b_new = clip(1, 2);
    ClipVertex a_new = clip(0, 2);
    out[0] = {{A, B, b_new}};
    out[1] = {{A, b_new, a_new}};
    return 2;
}

// TriClipper::clip_tri (clipper.rs:756-776): a FIFO queue, planes in order L,R,B,T,Front,Back.
static inline void clip_tri(const V4 pos[3], std::vector<ClipTri>& result) {
    std::deque<ClipTri> queue;
    ClipTri first;
    for (int i = 0; i < 3; ++i) first.v[i] = {pos[i], bary_at_vertex(i)};
    queue.push_back(first);
    for (int p = 0; p < 6; ++p) {
        size_t n = queue.size();
        for (size_t k = 0; k < n; ++k) {
            ClipTri t = queue.front();
            queue.pop_front();
            ClipTri out[2];
            int m = clip_tri_against_plane(t, kClipPlanes[p], out);
            for (int j = 0; j < m; ++j) queue.push_back(out[j]);
        }
    }
    result.assign(queue.begin(), queue.end());
}

// Cohen–Sutherland line clip (clipper.rs:268-356).  Returns false for "None".
static inline bool clip_line(V4 pts[2], float alphas_out[2]) {
    float dist[2][6];
    unsigned outcode[2] = {0, 0};
    for (int i = 0; i < 2; ++i)
        for (int p = 0; p < 6; ++p) {
            dist[i][p] = dot4(pts[i], kClipPlanes[p]);
            if (dist[i][p] < 0.0f) outcode[i] |= 1u << p;
        }
    unsigned o_or = outcode[0] | outcode[1], o_and = outcode[0] & outcode[1];
    if (o_or == 0) {
        alphas_out[0] = 0.0f;
        alphas_out[1] = 1.0f;
        return true;
    }
    if (o_and != 0) return false;
    float alphas[2] = {0.0f, 1.0f};
    for (int p = 0; p < 6; ++p) {
        unsigned bit = 1u << p;
        if (o_or & bit) {
            float a = dist[0][p], b = dist[1][p];
            float alpha = a / (a - b);
            if (outcode[0] & bit) {
                if (alpha > alphas[0]) alphas[0] = alpha;
            } else {
                if (alpha < alphas[1]) alphas[1] = alpha;
            }
            if (alphas[0] > alphas[1]) return false;
        }
    }
    V4 p0 = pts[0], p1 = pts[1];
    auto update = [&](int i) {
        float t = alphas[i];
        float omt = 1.0f - t;
        pts[i] = v4_add(v4_mul(p0, omt), v4_mul(p1, t));
    };
    // Note: update_point reads points[0]/points[1] at call time; point 0 is updated first, so
    // updating point 1 uses the *updated* point 0 (clipper.rs:337-352).
    if (outcode[0] != 0) {
        update(0);
        p0 = pts[0];
    }
    if (outcode[1] != 0) update(1);
    alphas_out[0] = alphas[0];
    alphas_out[1] = alphas[1];
    return true;
}

// ------------------------------------------------------------------------------------------
// TriFace (primitive.rs:159-198).  Returns false if some w == 0 (the reference panics).
// front = true for Ccw (vector_area.z > 0).
static inline bool tri_face_ccw(const V4 pos[3], bool* ccw) {
    float n[3][3];
    for (int i = 0; i < 3; ++i) {
        if (pos[i].w == 0.0f) return false;
        n[i][0] = pos[i].x / pos[i].w;
        n[i][1] = pos[i].y / pos[i].w;
        n[i][2] = pos[i].z / pos[i].w;
    }
    float abx = n[1][0] - n[0][0], aby = n[1][1] - n[0][1];
    float acx = n[2][0] - n[0][0], acy = n[2][1] - n[0][1];
    float z = abx * acy - aby * acx;
    *ccw = z > 0.0f;
    return true;
}

// ------------------------------------------------------------------------------------------
// ToRaster (raster.rs:122-168)
struct ToRaster {
    float tx, ty, sx, sy;
    uint32_t s0x, s0y, s1x, s1y;  // scissor [s0, s1)
};
static inline ToRaster make_to_raster(const float vp[4] /*x,y,w,h*/, const uint32_t sc[4]) {
    ToRaster r;
    // translation = offset + 0.5 * size; scaling = 0.5 * size; scaling.y *= -1.0
    r.tx = vp[0] + 0.5f * vp[2];
    r.ty = vp[1] + 0.5f * vp[3];
    r.sx = 0.5f * vp[2];
    r.sy = (0.5f * vp[3]) * -1.0f;
    r.s0x = sc[0];
    r.s0y = sc[1];
    r.s1x = sc[0] + sc[2];
    r.s1y = sc[1] + sc[3];
    return r;
}

struct RasterPoint {
    uint32_t fbx, fby;
    V4 frag;  // (viewport.x, viewport.y, ndc.z, 1/w)
};

// to_raster (raster.rs:145-160); false on w == 0 (the reference panics "w=0").
static inline bool to_raster(const ToRaster& r, V4 clip, RasterPoint* out) {
    if (clip.w == 0.0f) return false;
    float nx = clip.x / clip.w, ny = clip.y / clip.w, nz = clip.z / clip.w;
    float pd = 1.0f / clip.w;
    float vx = nx * r.sx + r.tx;
    float vy = ny * r.sy + r.ty;
    vx = rust_max0(vx);
    vy = rust_max0(vy);
    out->fbx = rust_f32_to_u32(vx);
    out->fby = rust_f32_to_u32(vy);
    out->frag = {vx, vy, nz, pd};
    return true;
}

static inline bool in_scissor(const ToRaster& r, uint32_t x, uint32_t y) {  // raster.rs:162-167
    return x >= r.s0x && x < r.s1x && y >= r.s0y && y < r.s1y;
}

// ------------------------------------------------------------------------------------------
// bubblesort3 (util/sort.rs:3-22): compare-and-swap (0,1), (0,2), (1,2), swapping on Greater.
template <class T, class Key>
static inline void bubblesort3(T v[3], Key key) {
    auto cas = [&](int l, int r) {
        if (key(v[l]) > key(v[r])) {
            T t = v[l];
            v[l] = v[r];
            v[r] = t;
        }
    };
    cas(0, 1);
    cas(0, 2);
    cas(1, 2);
}

struct IPoint {
    int64_t x, y;
};
struct Scanline {
    int64_t y, x1, x2;  // inclusive span, x1 <= x2 (scanline.rs:156-170)
};

// scanlines (util/scanline.rs:14-146): the tinyrenderer state machine, iterated exactly.
// Calls emit(Scanline) for each row.  Returns false if a coordinate would not fit u32 (the
// reference panics).
template <class Emit>
static inline bool scanlines(const uint32_t fx[3], const uint32_t fy[3], Emit emit) {
    IPoint tri[3];
    for (int i = 0; i < 3; ++i) tri[i] = {(int64_t)fx[i], (int64_t)fy[i]};
    bubblesort3(tri, [](const IPoint& p) { return p.y; });
    IPoint a = tri[0], b = tri[1], c = tri[2];
    IPoint ac = {c.x - a.x, c.y - a.y}, ab = {b.x - a.x, b.y - a.y}, bc = {c.x - b.x, c.y - b.y};
    auto mk = [&](int64_t y, int64_t x1, int64_t x2) -> bool {
        if (x1 > x2) {
            int64_t t = x1;
            x1 = x2;
            x2 = t;
        }
        if (y < 0 || x1 < 0 || x2 < 0 || y > 0xFFFFFFFFll || x1 > 0xFFFFFFFFll || x2 > 0xFFFFFFFFll) return false;
        emit(Scanline{y, x1, x2});
        return true;
    };
    if (ac.y == 0) {  // DegenerateLine
        bubblesort3(tri, [](const IPoint& p) { return p.x; });
        return mk(a.y, tri[0].x, tri[2].x);
    }
    int64_t y = a.y, i = 0;
    bool first = ab.y != 0;
    if (first) {
        while (y < b.y) {
            int64_t x1 = a.x + (ac.x * i) / ac.y;
            int64_t x2 = a.x + (ab.x * i) / ab.y;
            if (!mk(y, x1, x2)) return false;
            ++y;
            ++i;
        }
        if (bc.y == 0) return true;  // Done: the row y == c.y is not emitted
    }
    int64_t i2 = 0;
    while (y <= c.y) {
        int64_t x1 = a.x + (ac.x * i) / ac.y;
        int64_t x2 = b.x + (bc.x * i2) / bc.y;
        ++i2;
        if (!mk(y, x1, x2)) return false;
        ++y;
        ++i;
    }
    return true;
}

// ------------------------------------------------------------------------------------------
// Extension profile, edge-function rule (no reference counterpart): vertices snapped to 1/256
// pixel (round to nearest even), coverage of pixel centres by three integer edge functions with
// the top-left rule.  The kernels' span_edge (raster.cuh) follows the same steps.
static inline int64_t floor_div64(int64_t a, int64_t b) {  // b > 0
    int64_t q = a / b;
    if ((a % b) != 0 && a < 0) --q;
    return q;
}
static inline int64_t ceil_div64(int64_t a, int64_t b) { return -floor_div64(-a, b); }

// Snapped vertices ordered to a positive doubled area, which is returned (0: nothing covered).
static inline int64_t snap_triangle(const float vx[3], const float vy[3], int64_t X[3], int64_t Y[3]) {
    for (int i = 0; i < 3; ++i) {
        X[i] = (int64_t)std::nearbyint(vx[i] * 256.0f);
        Y[i] = (int64_t)std::nearbyint(vy[i] * 256.0f);
    }
    int64_t a2 = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
    if (a2 < 0) {
        std::swap(X[1], X[2]);
        std::swap(Y[1], Y[2]);
        a2 = -a2;
    }
    return a2;
}

// Covered pixels [x1, x2] of row y: every edge i -> j (d = (dx, dy)) needs
// E = dx (P.y - Y_i) - dy (P.x - X_i) > 0 at the centre P = (256 x + 128, 256 y + 128), or E == 0 on
// a top (dy == 0, dx > 0) or left (dy < 0) edge.
static inline void span_edge(const int64_t X[3], const int64_t Y[3], int64_t y, int64_t* x1, int64_t* x2) {
    const int64_t py = y * 256 + 128;
    int64_t lo = -(int64_t(1) << 30), hi = int64_t(1) << 30;
    for (int e = 0; e < 3; ++e) {
        const int i = e, j = (e + 1) % 3;
        const int64_t dx = X[j] - X[i], dy = Y[j] - Y[i];
        const bool owns_on_edge = dy < 0 || (dy == 0 && dx > 0);
        // E(x) = -dy * (256 x + 128) + dx * (py - Y_i) + dy * X_i, needed >= (owns ? 0 : 1)
        const int64_t a = -256 * dy;
        const int64_t b = -128 * dy + dx * (py - Y[i]) + dy * X[i] - (owns_on_edge ? 0 : 1);
        if (a > 0) lo = std::max(lo, ceil_div64(-b, a));
        else if (a < 0) hi = std::min(hi, floor_div64(b, -a));
        else if (b < 0) {
            lo = 1;
            hi = 0;
        }
    }
    *x1 = lo;
    *x2 = hi;
}

// shoelace (raster.rs:294-298), evaluated left to right.
struct P2 {
    float x, y;
};
static inline float shoelace(P2 a, P2 b, P2 c) {
    return (b.y - a.y) * (b.x + a.x) + (c.y - b.y) * (c.x + b.x) + (a.y - c.y) * (a.x + c.x);
}

// ------------------------------------------------------------------------------------------
// Bresenham (util/bresenham.rs:17-153).  Emits (x, y, t) for each point, end point excluded.
template <class Emit>
static inline void bresenham(uint32_t sx, uint32_t sy, uint32_t ex, uint32_t ey, Emit emit) {
    int64_t s[2] = {(int64_t)sx, (int64_t)sy}, e[2] = {(int64_t)ex, (int64_t)ey};
    int64_t dx = e[0] - s[0], dy = e[1] - s[1];
    int oct = 0;
    if (dy < 0) {
        dx = -dx;
        dy = -dy;
        oct += 4;
    }
    if (dx < 0) {
        int64_t tmp = dx;
        dx = dy;
        dy = -tmp;
        oct += 2;
    }
    if (dx < dy) oct += 1;
    auto to0 = [&](int64_t x, int64_t y, int64_t* ox, int64_t* oy) {
        switch (oct) {
            case 0: *ox = x; *oy = y; break;
            case 1: *ox = y; *oy = x; break;
            case 2: *ox = y; *oy = -x; break;
            case 3: *ox = -x; *oy = y; break;
            case 4: *ox = -x; *oy = -y; break;
            case 5: *ox = -y; *oy = -x; break;
            case 6: *ox = -y; *oy = x; break;
            default: *ox = x; *oy = -y; break;
        }
    };
    auto from0 = [&](int64_t x, int64_t y, int64_t* ox, int64_t* oy) {
        switch (oct) {
            case 0: *ox = x; *oy = y; break;
            case 1: *ox = y; *oy = x; break;
            case 2: *ox = -y; *oy = x; break;
            case 3: *ox = -x; *oy = y; break;
            case 4: *ox = -x; *oy = -y; break;
            case 5: *ox = -y; *oy = -x; break;
            case 6: *ox = y; *oy = -x; break;
            default: *ox = x; *oy = -y; break;
        }
    };
    int64_t px, py, qx, qy;
    to0(s[0], s[1], &px, &py);
    to0(e[0], e[1], &qx, &qy);
    int64_t Dx = qx - px, Dy = qy - py;
    float dt = 1.0f / (float)Dx;
    int64_t diff = Dy - Dx;
    float t = 0.0f;
    while (px < qx) {
        int64_t cx = px, cy = py;
        if (diff >= 0) {
            py += 1;
            diff -= Dx;
        }
        diff += Dy;
        float tt = t;
        t += dt;
        px += 1;
        int64_t ox, oy;
        from0(cx, cy, &ox, &oy);
        emit((uint32_t)ox, (uint32_t)oy, tt);
    }
}

// ------------------------------------------------------------------------------------------
// Triangle-strip assembly (primitive.rs:360-392): primitive p of a strip uses stream positions
// [p, p+1, p+2] for even p and [p+1, p, p+2] for odd p.
static inline void strip_tri(uint32_t p, uint32_t out[3]) {
    if ((p & 1u) == 0) {
        out[0] = p;
        out[1] = p + 1;
    } else {
        out[0] = p + 1;
        out[1] = p;
    }
    out[2] = p + 2;
}

// f32 -> binary16, round to nearest even (IEEE 754), used by the extension profile for
// Rgba16Float targets and Float16 vertex formats.
static inline uint16_t f32_to_f16_rne(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t absx = x & 0x7FFFFFFFu;
    if (absx > 0x7F800000u) return (uint16_t)(sign | 0x7E00u | ((absx >> 13) & 0x3FFu));  // NaN
    if (absx >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // overflow (>= 65520) -> inf
    if (absx >= 0x38800000u) {                                    // normal half
        uint32_t mant = absx & 0x7FFFFFu;
        uint32_t exp = (absx >> 23) - 127 + 15;
        uint32_t h = (exp << 10) | (mant >> 13);
        uint32_t rem = mant & 0x1FFFu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1;
        return (uint16_t)(sign | h);
    }
    if (absx < 0x33000000u) return (uint16_t)sign;  // < 2^-25: rounds to zero
    // subnormal half
    uint32_t exp = absx >> 23;
    uint32_t mant = (absx & 0x7FFFFFu) | 0x800000u;
    uint32_t shift = 126 - exp;  // 14 + (113 - exp) ... number of bits dropped beyond 13
    uint32_t h = mant >> (shift);
    uint32_t rem = mant & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1);
    if (rem > half || (rem == half && (h & 1u))) h += 1;
    return (uint16_t)(sign | h);
}
static inline float f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1Fu;
    uint32_t mant = h & 0x3FFu;
    uint32_t x;
    if (exp == 0) {
        if (mant == 0) {
            x = sign;
        } else {
            int e = -1;
            do {
                ++e;
                mant <<= 1;
            } while ((mant & 0x400u) == 0);
            mant &= 0x3FFu;
            x = sign | ((uint32_t)(127 - 15 - e) << 23) | (mant << 13);
        }
    } else if (exp == 31) {
        x = sign | 0x7F800000u | (mant << 13);
    } else {
        x = sign | ((exp - 15 + 127) << 23) | (mant << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

}  // namespace orc
