// sampling.cuh — extension-profile texturing: sRGB decode/encode, mip LOD from analytic
// derivatives, nearest / bilinear / trilinear filtering with WebGPU addressing.
//
// The reference has none of this (image_sample, render_pass/binding.rs:93-140, reads mip 0 with
// its own nearest rule and treats Srgb formats as Unorm); the parity profile keeps that
// behaviour.  The extension profile follows the WebGPU sampling model, with every float step
// spelled out so that the CPU oracle (oracle/orc_device.cpp, sample_ext / lod_from_grad) gives
// the same bits:
//   * texel decode: RGB of an Rgba8UnormSrgb texture through kSrgbToLinear, everything else
//     `k / 255` (correctly rounded);
//   * LOD per primitive: the varyings are interpolated affinely in screen space (raster.rs:313-346),
//     so d(uv)/dx and d(uv)/dy are constant per record; lambda = 0.5 * log2(max(|d/dx|^2,
//     |d/dy|^2)) in level-0 texels, clamped to the sampler's [lod_min, lod_max];
//   * lambda <= 0 magnifies (mag filter, level 0); otherwise the min filter, and the mip filter
//     picks level ceil(lambda + 0.5) - 1 (nearest) or blends floor(lambda) and the next level
//     (linear); levels are clamped to the texture's last mip;
//   * nearest texel floor(u * w); linear taps at u * w - 0.5 with weights from the fraction;
//     integer texel coordinates wrap per address mode (repeat: Euclidean modulo, mirror: period
//     2w, clamp: [0, w-1]);
//   * lerp(a, b, t) = a + (b - a) * t per channel.
#pragma once

#include "exact.cuh"
#include "gbr_types.h"

#define GBR_TABLE_QUAL static __device__ const
#include "srgb_tables.h"

namespace gbr {

// ------------------------------------------------------------------------------ sRGB
__device__ __forceinline__ float srgb_to_linear(uint32_t k) { return __ldg(&kSrgbToLinear[k & 0xFFu]); }

// Linear -> unorm8 sRGB: the number of thresholds at or below v (binary search over 255 sorted
// values); NaN and v < threshold[1] give 0, v >= threshold[255] (including v > 1) gives 255.
__device__ __forceinline__ uint32_t linear_to_srgb8(float v) {
    uint32_t k = 0;
#pragma unroll
    for (uint32_t step = 128; step > 0; step >>= 1)
        if (k + step <= 255u && v >= __ldg(&kSrgbEncodeThreshold[k + step])) k += step;
    return k;
}

// ------------------------------------------------------------------------------ LOD
// log2 of a binary32 value with basic IEEE operations only (same sequence in the oracle):
// r = m * 2^e with m in [sqrt(1/2), sqrt(2)), ln(m) = 2 atanh(s), s = (m - 1) / (m + 1), from the
// series s + s^3/3 + s^5/5 + s^7/7 (|s| < 0.172: truncation below 3e-8 relative).  0, negative and
// NaN give -inf; +inf gives +inf.
__device__ __forceinline__ float log2_spec(float r) {
    if (!(r > 0.0f)) return -__int_as_float(0x7F800000);
    if (r == __int_as_float(0x7F800000)) return r;
    uint32_t bits = __float_as_uint(r);
    int e = (int)((bits >> 23) & 0xFFu);
    if (e == 0) {  // subnormal: scale by 2^24 first (exact)
        bits = __float_as_uint(fmul(r, 0x1p24f));
        e = (int)((bits >> 23) & 0xFFu) - 24;
    }
    e -= 127;
    float m = __uint_as_float((bits & 0x7FFFFFu) | 0x3F800000u);
    if (m > 0x1.6a09e6p+0f) {  // sqrt(2) rounded to binary32
        m = fmul(m, 0.5f);
        e += 1;
    }
    const float s = fdiv(fsub(m, 1.0f), fadd(m, 1.0f));
    const float z = fmul(s, s);
    float p = 0x1.249250p-3f;           // 1/7
    p = fadd(fmul(p, z), 0x1.99999ap-3f);  // 1/5
    p = fadd(fmul(p, z), 0x1.555556p-2f);  // 1/3
    p = fadd(fmul(p, z), 1.0f);
    const float ln = fmul(fmul(2.0f, s), p);
    return fadd((float)e, fmul(ln, 0x1.715476p+0f));  // 1/ln(2)
}

// Sampler-clamped LOD from the screen-space derivatives of (u, v) and the level-0 size.
__device__ __forceinline__ float lod_from_grad(float dudx, float dvdx, float dudy, float dvdy, uint32_t w, uint32_t h,
                                               float lod_min, float lod_max) {
    const float sx = fmul(dudx, (float)w), tx = fmul(dvdx, (float)h);
    const float sy = fmul(dudy, (float)w), ty = fmul(dvdy, (float)h);
    const float px2 = fadd(fmul(sx, sx), fmul(tx, tx)), py2 = fadd(fmul(sy, sy), fmul(ty, ty));
    const float r2 = px2 >= py2 ? px2 : py2;
    float lod = fmul(0.5f, log2_spec(r2));
    if (!(lod >= lod_min)) lod = lod_min;
    if (lod > lod_max) lod = lod_max;
    return lod;
}

// Screen-space derivatives of the composed barycentrics of a record (raster.rs:313-343):
// lambda_0 = S(p, b, c) / A gives d/dx = (b.y - c.y) / A, d/dy = (c.x - b.x) / A (cyclically for
// lambda_1, lambda_2); the clip barycentrics cb (row i = vertex i) compose them like the
// barycentrics themselves.
__device__ __forceinline__ void bary_gradients(const float vx[3], const float vy[3], float area, const float cb[9],
                                               float dcx[3], float dcy[3]) {
    const float lx[3] = {fdiv(fsub(vy[1], vy[2]), area), fdiv(fsub(vy[2], vy[0]), area), fdiv(fsub(vy[0], vy[1]), area)};
    const float ly[3] = {fdiv(fsub(vx[2], vx[1]), area), fdiv(fsub(vx[0], vx[2]), area), fdiv(fsub(vx[1], vx[0]), area)};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        dcx[j] = fadd(fadd(fmul(cb[j], lx[0]), fmul(cb[3 + j], lx[1])), fmul(cb[6 + j], lx[2]));
        dcy[j] = fadd(fadd(fmul(cb[j], ly[0]), fmul(cb[3 + j], ly[1])), fmul(cb[6 + j], ly[2]));
    }
}

// ------------------------------------------------------------------------------ filtering
__device__ __forceinline__ int wrap_texel(int i, int n, uint32_t mode) {
    if (mode == 1) {  // Repeat
        const int r = i % n;
        return r < 0 ? r + n : r;
    }
    if (mode == 2) {  // MirrorRepeat
        const int p = 2 * n;
        int t = i % p;
        if (t < 0) t += p;
        return t < n ? t : p - 1 - t;
    }
    return i < 0 ? 0 : (i >= n ? n - 1 : i);  // ClampToEdge (and ClampToBorder, unsupported)
}

// u * size, clamped to +-2^24 (NaN -> 0) so the integer conversion is defined.
__device__ __forceinline__ float texel_space(float u, uint32_t size, float bias) {
    float x = fsub(fmul(u, (float)size), bias);
    if (!(x >= -16777216.0f)) x = x != x ? 0.0f : -16777216.0f;
    if (x > 16777216.0f) x = 16777216.0f;
    return x;
}

struct TexelDecode {
    const float* unorm;  // `k / 255` table (shared memory of the raster kernels)
    bool srgb;
};
__device__ __forceinline__ V4 decode_texel(uint32_t px, const TexelDecode& td) {
    if (td.srgb)
        return {srgb_to_linear(px & 0xFFu), srgb_to_linear((px >> 8) & 0xFFu), srgb_to_linear((px >> 16) & 0xFFu),
                td.unorm[px >> 24]};
    return {td.unorm[px & 0xFFu], td.unorm[(px >> 8) & 0xFFu], td.unorm[(px >> 16) & 0xFFu], td.unorm[px >> 24]};
}
__device__ __forceinline__ V4 lerp4(V4 a, V4 b, float t) {
    return {fadd(a.x, fmul(fsub(b.x, a.x), t)), fadd(a.y, fmul(fsub(b.y, a.y), t)), fadd(a.z, fmul(fsub(b.z, a.z), t)),
            fadd(a.w, fmul(fsub(b.w, a.w), t))};
}

// One mip level of an Rgba8 texture, nearest or linear.
__device__ __forceinline__ V4 sample_level(const TexDesc& t, const SamplerDescDev& s, uint32_t level, bool linear,
                                           float u, float v, const TexelDecode& td) {
    const int w = (int)max(1u, t.width >> level), h = (int)max(1u, t.height >> level);
    const uint32_t* texels = reinterpret_cast<const uint32_t*>(t.data + t.mip_offset[level]);
    if (!linear) {
        const int x = wrap_texel((int)floorf(texel_space(u, (uint32_t)w, 0.0f)), w, s.address_u);
        const int y = wrap_texel((int)floorf(texel_space(v, (uint32_t)h, 0.0f)), h, s.address_v);
        return decode_texel(__ldg(texels + (size_t)y * w + x), td);
    }
    const float xs = texel_space(u, (uint32_t)w, 0.5f), ys = texel_space(v, (uint32_t)h, 0.5f);
    const float xf = floorf(xs), yf = floorf(ys);
    const float fx = fsub(xs, xf), fy = fsub(ys, yf);
    const int x0 = wrap_texel((int)xf, w, s.address_u), x1 = wrap_texel((int)xf + 1, w, s.address_u);
    const int y0 = wrap_texel((int)yf, h, s.address_v), y1 = wrap_texel((int)yf + 1, h, s.address_v);
    const V4 t00 = decode_texel(__ldg(texels + (size_t)y0 * w + x0), td);
    const V4 t10 = decode_texel(__ldg(texels + (size_t)y0 * w + x1), td);
    const V4 t01 = decode_texel(__ldg(texels + (size_t)y1 * w + x0), td);
    const V4 t11 = decode_texel(__ldg(texels + (size_t)y1 * w + x1), td);
    return lerp4(lerp4(t00, t10, fx), lerp4(t01, t11, fx), fy);
}

// Extension-profile sample of an Rgba8 / Rgba8UnormSrgb texture at (u, v) with the record's LOD.
__device__ __forceinline__ V4 sample_ext(const TexDesc& t, const SamplerDescDev& s, float u, float v, float lod,
                                         const float* unorm_lut) {
    const TexelDecode td{unorm_lut, t.format == TEXFMT_RGBA8_UNORM_SRGB};
    const uint32_t last = t.mip_count > 0 ? t.mip_count - 1 : 0;
    if (lod <= 0.0f) return sample_level(t, s, 0, s.mag_filter == 1, u, v, td);
    const bool lin = s.min_filter == 1;
    if (s.mip_filter != 1) {
        float lv = fsub(ceilf(fadd(lod, 0.5f)), 1.0f);
        const uint32_t level = lv >= (float)last ? last : (uint32_t)lv;
        return sample_level(t, s, level, lin, u, v, td);
    }
    const float lc = lod < (float)last ? lod : (float)last;
    const float lf = floorf(lc);
    const uint32_t l0 = (uint32_t)lf;
    const float f = fsub(lc, lf);
    const V4 c0 = sample_level(t, s, l0, lin, u, v, td);
    if (f == 0.0f || l0 >= last) return c0;
    return lerp4(c0, sample_level(t, s, l0 + 1, lin, u, v, td), f);
}

}  // namespace gbr
