// wgsl_rt.cuh — value types and operators for CUDA emitted from WGSL (wgsl.cpp).
//
// Every f32 operator is one correctly rounded IEEE operation (__fadd_rn & co.), as Cranelift
// emits them for naga-cranelift (expression/binary.rs:421-447); integer arithmetic wraps;
// integer division and remainder by zero (and i32::MIN / -1) set the trap flag, which fails the
// draw as the reference's EntryPointError::DivisionByZero does; casts follow Rust's `as`
// (expression/as.rs:60-160): float -> int saturates and maps NaN to 0.
#pragma once

#include "exact.cuh"
#include "programs.cuh"

namespace gbr {

template <class T, int N>
struct WV {
    T c[N];
};
template <int C, int R>
struct WM {
    WV<float, R> col[C];
};
template <class T, int N>
struct WA {
    T e[N];
};

// ---- scalar operators
__device__ __forceinline__ float w_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float w_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float w_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float w_div(float a, float b, bool&) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float w_rem(float a, float b, bool&) { return fmodf(a, b); }  // Rust f32 `%`
__device__ __forceinline__ int w_add(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
__device__ __forceinline__ int w_sub(int a, int b) { return (int)((unsigned)a - (unsigned)b); }
__device__ __forceinline__ int w_mul(int a, int b) { return (int)((unsigned)a * (unsigned)b); }
__device__ __forceinline__ int w_div(int a, int b, bool& tr) {
    if (b == 0 || (a == (int)0x80000000 && b == -1)) {
        tr = true;
        return 0;
    }
    return a / b;
}
__device__ __forceinline__ int w_rem(int a, int b, bool& tr) {
    if (b == 0 || (a == (int)0x80000000 && b == -1)) {
        tr = true;
        return 0;
    }
    return a % b;
}
__device__ __forceinline__ unsigned w_add(unsigned a, unsigned b) { return a + b; }
__device__ __forceinline__ unsigned w_sub(unsigned a, unsigned b) { return a - b; }
__device__ __forceinline__ unsigned w_mul(unsigned a, unsigned b) { return a * b; }
__device__ __forceinline__ unsigned w_div(unsigned a, unsigned b, bool& tr) {
    if (b == 0) {
        tr = true;
        return 0;
    }
    return a / b;
}
__device__ __forceinline__ unsigned w_rem(unsigned a, unsigned b, bool& tr) {
    if (b == 0) {
        tr = true;
        return 0;
    }
    return a % b;
}
__device__ __forceinline__ int w_and(int a, int b) { return a & b; }
__device__ __forceinline__ int w_or(int a, int b) { return a | b; }
__device__ __forceinline__ int w_xor(int a, int b) { return a ^ b; }
__device__ __forceinline__ unsigned w_and(unsigned a, unsigned b) { return a & b; }
__device__ __forceinline__ unsigned w_or(unsigned a, unsigned b) { return a | b; }
__device__ __forceinline__ unsigned w_xor(unsigned a, unsigned b) { return a ^ b; }
__device__ __forceinline__ bool w_and(bool a, bool b) { return a && b; }
__device__ __forceinline__ bool w_or(bool a, bool b) { return a || b; }
__device__ __forceinline__ bool w_xor(bool a, bool b) { return a != b; }
// shift amounts are taken modulo the bit width (Cranelift ishl / sshr / ushr)
__device__ __forceinline__ int w_shl(int a, unsigned b) { return (int)((unsigned)a << (b & 31u)); }
__device__ __forceinline__ int w_shr(int a, unsigned b) { return a >> (b & 31u); }
__device__ __forceinline__ unsigned w_shl(unsigned a, unsigned b) { return a << (b & 31u); }
__device__ __forceinline__ unsigned w_shr(unsigned a, unsigned b) { return a >> (b & 31u); }

__device__ __forceinline__ float w_neg(float a) { return -a; }
__device__ __forceinline__ int w_neg(int a) { return (int)(0u - (unsigned)a); }
__device__ __forceinline__ bool w_lnot(bool a) { return !a; }
__device__ __forceinline__ int w_bnot(int a) { return ~a; }
__device__ __forceinline__ unsigned w_bnot(unsigned a) { return ~a; }

template <class T>
__device__ __forceinline__ bool w_eq(T a, T b) { return a == b; }
template <class T>
__device__ __forceinline__ bool w_ne(T a, T b) { return a != b; }
template <class T>
__device__ __forceinline__ bool w_lt(T a, T b) { return a < b; }
template <class T>
__device__ __forceinline__ bool w_le(T a, T b) { return a <= b; }
template <class T>
__device__ __forceinline__ bool w_gt(T a, T b) { return a > b; }
template <class T>
__device__ __forceinline__ bool w_ge(T a, T b) { return a >= b; }

// ---- conversions (Rust `as`)
__device__ __forceinline__ float w_f32(float a) { return a; }
__device__ __forceinline__ float w_f32(int a) { return __int2float_rn(a); }
__device__ __forceinline__ float w_f32(unsigned a) { return __uint2float_rn(a); }
__device__ __forceinline__ float w_f32(bool a) { return a ? 1.0f : 0.0f; }
__device__ __forceinline__ int w_i32(float a) {
    if (a != a) return 0;
    if (a >= 2147483648.0f) return 0x7FFFFFFF;
    if (a < -2147483648.0f) return (int)0x80000000;
    return (int)a;
}
__device__ __forceinline__ int w_i32(int a) { return a; }
__device__ __forceinline__ int w_i32(unsigned a) { return (int)a; }
__device__ __forceinline__ int w_i32(bool a) { return a ? 1 : 0; }
__device__ __forceinline__ unsigned w_u32(float a) {
    if (!(a > 0.0f)) return 0u;  // NaN, zero and negatives
    if (a >= 4294967296.0f) return 0xFFFFFFFFu;
    return (unsigned)a;
}
__device__ __forceinline__ unsigned w_u32(int a) { return (unsigned)a; }
__device__ __forceinline__ unsigned w_u32(unsigned a) { return a; }
__device__ __forceinline__ unsigned w_u32(bool a) { return a ? 1u : 0u; }
__device__ __forceinline__ bool w_bool(float a) { return a != 0.0f; }
__device__ __forceinline__ bool w_bool(int a) { return a != 0; }
__device__ __forceinline__ bool w_bool(unsigned a) { return a != 0u; }
__device__ __forceinline__ bool w_bool(bool a) { return a; }

// ---- component-wise forms
#define GBR_W_VV(NAME)                                                                  \
    template <class T, int N>                                                           \
    __device__ __forceinline__ WV<T, N> NAME(WV<T, N> a, WV<T, N> b) {                  \
        WV<T, N> r;                                                                     \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b.c[i]);    \
        return r;                                                                       \
    }                                                                                   \
    template <class T, int N>                                                           \
    __device__ __forceinline__ WV<T, N> NAME(WV<T, N> a, T b) {                         \
        WV<T, N> r;                                                                     \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b);         \
        return r;                                                                       \
    }                                                                                   \
    template <class T, int N>                                                           \
    __device__ __forceinline__ WV<T, N> NAME(T a, WV<T, N> b) {                         \
        WV<T, N> r;                                                                     \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a, b.c[i]);         \
        return r;                                                                       \
    }
GBR_W_VV(w_add)
GBR_W_VV(w_sub)
GBR_W_VV(w_mul)
GBR_W_VV(w_and)
GBR_W_VV(w_or)
GBR_W_VV(w_xor)
#undef GBR_W_VV
#define GBR_W_VV_TRAP(NAME)                                                                   \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<T, N> NAME(WV<T, N> a, WV<T, N> b, bool& tr) {              \
        WV<T, N> r;                                                                           \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b.c[i], tr);      \
        return r;                                                                             \
    }                                                                                         \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<T, N> NAME(WV<T, N> a, T b, bool& tr) {                     \
        WV<T, N> r;                                                                           \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b, tr);           \
        return r;                                                                             \
    }                                                                                         \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<T, N> NAME(T a, WV<T, N> b, bool& tr) {                     \
        WV<T, N> r;                                                                           \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a, b.c[i], tr);           \
        return r;                                                                             \
    }
GBR_W_VV_TRAP(w_div)
GBR_W_VV_TRAP(w_rem)
#undef GBR_W_VV_TRAP
#define GBR_W_SHIFT(NAME)                                                                     \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<T, N> NAME(WV<T, N> a, WV<unsigned, N> b) {                 \
        WV<T, N> r;                                                                           \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b.c[i]);          \
        return r;                                                                             \
    }                                                                                         \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<T, N> NAME(WV<T, N> a, unsigned b) {                        \
        WV<T, N> r;                                                                           \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b);               \
        return r;                                                                             \
    }
GBR_W_SHIFT(w_shl)
GBR_W_SHIFT(w_shr)
#undef GBR_W_SHIFT
#define GBR_W_CMP(NAME)                                                                       \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<bool, N> NAME(WV<T, N> a, WV<T, N> b) {                     \
        WV<bool, N> r;                                                                        \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b.c[i]);          \
        return r;                                                                             \
    }                                                                                         \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<bool, N> NAME(WV<T, N> a, T b) {                            \
        WV<bool, N> r;                                                                        \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i], b);               \
        return r;                                                                             \
    }                                                                                         \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<bool, N> NAME(T a, WV<T, N> b) {                            \
        WV<bool, N> r;                                                                        \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a, b.c[i]);               \
        return r;                                                                             \
    }
GBR_W_CMP(w_eq)
GBR_W_CMP(w_ne)
GBR_W_CMP(w_lt)
GBR_W_CMP(w_le)
GBR_W_CMP(w_gt)
GBR_W_CMP(w_ge)
#undef GBR_W_CMP
#define GBR_W_UN(NAME, RT)                                                                     \
    template <class T, int N>                                                                 \
    __device__ __forceinline__ WV<RT, N> NAME(WV<T, N> a) {                                   \
        WV<RT, N> r;                                                                          \
        _Pragma("unroll") for (int i = 0; i < N; ++i) r.c[i] = NAME(a.c[i]);                  \
        return r;                                                                             \
    }
GBR_W_UN(w_neg, T)
GBR_W_UN(w_lnot, T)
GBR_W_UN(w_bnot, T)
GBR_W_UN(w_f32, float)
GBR_W_UN(w_i32, int)
GBR_W_UN(w_u32, unsigned)
GBR_W_UN(w_bool, bool)
#undef GBR_W_UN

// abstract-literal vectors given a concrete element type
template <class T, class S, int N>
__device__ __forceinline__ WV<T, N> w_cast(WV<S, N> a) {
    WV<T, N> r;
#pragma unroll
    for (int i = 0; i < N; ++i) r.c[i] = (T)a.c[i];
    return r;
}
template <class T, int N>
__device__ __forceinline__ WV<T, N> w_splat(T a) {
    WV<T, N> r;
#pragma unroll
    for (int i = 0; i < N; ++i) r.c[i] = a;
    return r;
}

template <class T>
__device__ __forceinline__ T w_select(T f, T t, bool c) { return c ? t : f; }
template <class T, int N>
__device__ __forceinline__ WV<T, N> w_select(WV<T, N> f, WV<T, N> t, WV<bool, N> c) {
    WV<T, N> r;
#pragma unroll
    for (int i = 0; i < N; ++i) r.c[i] = c.c[i] ? t.c[i] : f.c[i];
    return r;
}

// ---- matrices: M * v as the column sum ((v0*c0 + v1*c1) + v2*c2) + v3*c3, lane by lane
template <int C, int R>
__device__ __forceinline__ WV<float, R> w_mulmv(const WM<C, R>& m, WV<float, C> v) {
    WV<float, R> r;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        float s = __fmul_rn(v.c[0], m.col[0].c[j]);
#pragma unroll
        for (int i = 1; i < C; ++i) s = __fadd_rn(s, __fmul_rn(v.c[i], m.col[i].c[j]));
        r.c[j] = s;
    }
    return r;
}
template <int C, int R>
__device__ __forceinline__ WM<C, R> w_mul(WM<C, R> m, float s) {
#pragma unroll
    for (int i = 0; i < C; ++i) m.col[i] = w_mul(m.col[i], s);
    return m;
}
template <int C, int R>
__device__ __forceinline__ WM<C, R> w_mul(float s, WM<C, R> m) {
#pragma unroll
    for (int i = 0; i < C; ++i) m.col[i] = w_mul(s, m.col[i]);
    return m;
}
template <int C, int R>
__device__ __forceinline__ WM<C, R> w_add(WM<C, R> a, const WM<C, R>& b) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.col[i] = w_add(a.col[i], b.col[i]);
    return a;
}
template <int C, int R>
__device__ __forceinline__ WM<C, R> w_sub(WM<C, R> a, const WM<C, R>& b) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.col[i] = w_sub(a.col[i], b.col[i]);
    return a;
}

// ---- dynamic indexing (an out-of-range index is clamped)
template <class T, int N, class I>
__device__ __forceinline__ T w_index(const WV<T, N>& v, I i) { return v.c[(unsigned)i < (unsigned)N ? (unsigned)i : N - 1]; }
template <class T, int N, class I>
__device__ __forceinline__ T& w_index_ref(WV<T, N>& v, I i) { return v.c[(unsigned)i < (unsigned)N ? (unsigned)i : N - 1]; }
template <int C, int R, class I>
__device__ __forceinline__ WV<float, R> w_col(const WM<C, R>& m, I i) { return m.col[(unsigned)i < (unsigned)C ? (unsigned)i : C - 1]; }
template <int C, int R, class I>
__device__ __forceinline__ WV<float, R>& w_col_ref(WM<C, R>& m, I i) { return m.col[(unsigned)i < (unsigned)C ? (unsigned)i : C - 1]; }
template <class T, int N, class I>
__device__ __forceinline__ T w_elem(const WA<T, N>& a, I i) { return a.e[(unsigned)i < (unsigned)N ? (unsigned)i : N - 1]; }
template <class T, int N, class I>
__device__ __forceinline__ T& w_elem_ref(WA<T, N>& a, I i) { return a.e[(unsigned)i < (unsigned)N ? (unsigned)i : N - 1]; }

// ---- textureSample: the reference's nearest sampler on mip 0 (render_pass/binding.rs:93-164)
__device__ __forceinline__ WV<float, 4> w_sample(const DrawDesc& d, WV<float, 2> uv) {
    const V4 t = sample_nearest_rgba8(d.tex, d.samp, uv.c[0], uv.c[1]);
    return WV<float, 4>{t.x, t.y, t.z, t.w};
}

}  // namespace gbr
