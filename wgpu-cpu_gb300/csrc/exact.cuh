// exact.cuh — IEEE binary32 building blocks that reproduce wgpu-cpu's scalar arithmetic bit for
// bit on the GPU.  Every operation is an explicitly rounded intrinsic (__fadd_rn, __fmul_rn,
// ...), which the compiler never contracts into FMA, and the library is also built with
// --fmad=false.  The order of operations in each helper is the reference's order.
#pragma once

#include <cuda_fp16.h>
#ifndef __CUDACC_RTC__
#include <stdint.h>
#endif

#include "gbr_types.h"

namespace gbr {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

struct V4 {
    float x, y, z, w;
};

__device__ __forceinline__ V4 v4_mul(V4 a, float s) { return {fmul(a.x, s), fmul(a.y, s), fmul(a.z, s), fmul(a.w, s)}; }
__device__ __forceinline__ V4 v4_add(V4 a, V4 b) { return {fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z), fadd(a.w, b.w)}; }

// nalgebra 0.34 `Matrix::dot` for 4-vectors (blas.rs `dotx`): (p0 + p2) + (p1 + p3).
__device__ __forceinline__ float dot4(V4 a, V4 b) {
    float p0 = fmul(a.x, b.x), p1 = fmul(a.y, b.y), p2 = fmul(a.z, b.z), p3 = fmul(a.w, b.w);
    return fadd(fadd(p0, p2), fadd(p1, p3));
}

// Rust f32::max(v, 0.0) as used by to_raster (raster.rs:150-151); NaN -> 0, -0 -> +0.
__device__ __forceinline__ float rust_max0(float v) { return v > 0.0f ? v : 0.0f; }

// Rust `v as u32` (saturating, NaN -> 0).
__device__ __forceinline__ uint32_t rust_f2u32(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xFFFFFFFFu;
    return __float2uint_rz(v);
}

// f32_to_u8 of TexelWriter::from_color (texture.rs:378-381): (v*255).clamp(0,255) as u8.
__device__ __forceinline__ uint32_t unorm8_trunc(float v) {
    float s = fmul(v, 255.0f);
    if (s < 0.0f) s = 0.0f;
    if (s > 255.0f) s = 255.0f;
    if (!(s > 0.0f)) return 0u;  // NaN and zero
    return __float2uint_rz(s);
}

// Extension profile: float -> unorm8 as WebGPU converts, clamp to [0, 1] then round to nearest
// (ties to even) of v * 255; NaN -> 0.  (The alpha of sRGB-encoded targets.)
__device__ __forceinline__ uint32_t unorm8_round(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 1.0f) return 255u;
    return (uint32_t)__float2int_rn(fmul(v, 255.0f));
}

// shoelace (raster.rs:294-298), left to right.
__device__ __forceinline__ float shoelace(float ax, float ay, float bx, float by, float cx, float cy) {
    float t1 = fmul(fsub(by, ay), fadd(bx, ax));
    float t2 = fmul(fsub(cy, by), fadd(cx, bx));
    float t3 = fmul(fsub(ay, cy), fadd(ax, cx));
    return fadd(fadd(t1, t2), t3);
}

// Integer division truncating toward zero for d > 0 (Rust isize `/`), 32-bit fast path.
__device__ __forceinline__ int64_t div_trunc(int64_t n, int64_t d) {
    if (n >= -2147483647ll && n <= 2147483647ll && d <= 2147483647ll) return (int64_t)((int32_t)n / (int32_t)d);
    return n / d;
}

// div_trunc with a binary32 fast path for |n|, d < 2^22 (every span of a target up to 2048
// pixels a side): q0 = trunc(n * RN(1/d)) has relative error below 2^-22.4 against n / d, so
// |q0 - trunc(n / d)| <= 1, and the exact remainder n - q0 d (|.| < 2^24) says which way to step.
__device__ __forceinline__ int64_t div_trunc_span(int64_t n, int64_t d) {
    if (n > -4194304ll && n < 4194304ll && d < 4194304ll) {
        const int32_t ni = (int32_t)n, di = (int32_t)d;
        int32_t q = __float2int_rz(__fmul_rn((float)ni, __frcp_rn((float)di)));
        const int32_t r = ni - q * di;
        if (ni >= 0) q += r < 0 ? -1 : (r >= di ? 1 : 0);
        else q += r > 0 ? 1 : (r <= -di ? -1 : 0);
        return q;
    }
    return div_trunc(n, d);
}

// a / b correctly rounded (round to nearest even), given y = RN(1/b) from __frcp_rn.
//
// Method: P. Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor" (IBM J. Res. Dev. 34(1), 1990), Theorem: if y is within half an ulp of 1/b and q is
// within one ulp of a/b, then with r = a - b*q computed exactly by one fused multiply-add,
// RN(q + r*y) is the correctly rounded quotient (see also Muller et al., Handbook of Floating-Point
// Arithmetic, §4.7).  q0 = RN(a*y) can be up to ~1.5 ulp away, so one correction step first makes
// it faithful; the second step then rounds correctly.  The theorem assumes no underflow or
// overflow: the fast path is taken only for 2^-60 <= |a|, |b| <= 2^60 (quotients, remainders and
// products then stay far inside the normal range); zeros, NaNs, infinities and everything outside
// go to __fdiv_rn.  tests/test_gpu_parity.py checks the result against __fdiv_rn bit for bit.
__device__ __forceinline__ bool div_fast_ok(float v) {
    const float m = fabsf(v);
    return m >= 0x1p-60f && m <= 0x1p60f;
}
__device__ __forceinline__ float div_by_recip(float a, float b, float y, bool b_ok) {
    if (!(b_ok && div_fast_ok(a))) return __fdiv_rn(a, b);
    const float q0 = __fmul_rn(a, y);
    const float r0 = __fmaf_rn(-b, q0, a);
    const float q1 = __fmaf_rn(r0, y, q0);
    const float r1 = __fmaf_rn(-b, q1, a);
    return __fmaf_rn(r1, y, q1);
}

// Packed f32x2 arithmetic (sm_100+): two IEEE binary32 operations per instruction, each lane
// rounded to nearest even exactly like the scalar op.
//
// Hazard: ptxas fuses a packed product whose only use is a packed sum into one fused
// multiply-add (a single rounding), whatever the .rn modifiers and --fmad=false say; it also
// sees through fma(a, b, -0) as the product and fma(p, 1, c) as the sum.  So a product that must
// be rounded on its own before a sum is always a scalar __fmul_rn (f2mul_rn below: two scalar
// products, which then feed a packed sum exactly).  Packed f2mul / f2fma are for the
// correction steps of a division, where every product feeds fused multiply-adds anyway.
__device__ __forceinline__ float2 f2add(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
// packed product: only where no sum consumes it (see above)
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
// a * b + c with one rounding per lane, as __fmaf_rn
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mov.b64 pc, {%6, %7};\n\tfma.rn.f32x2 pd, pa, pb, pc;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// two separately rounded scalar products, safe to feed a packed sum
__device__ __forceinline__ float2 f2mul_rn(float2 a, float2 b) {
    return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}

__device__ __forceinline__ uint16_t f32_to_f16_bits(float f) { return __half_as_ushort(__float2half_rn(f)); }
__device__ __forceinline__ float f16_bits_to_f32(uint16_t h) { return __half2float(__ushort_as_half(h)); }

}  // namespace gbr
