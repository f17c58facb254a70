// df64.cuh -- double-float ("float-float") arithmetic on the FP32 pipe.
//
// GB300 runs FP32 FMAs about 74x faster than FP64 ones (measured 77 vs
// 1.05 TFLOP/s).  A value held as an unevaluated sum hi + lo of two floats
// carries a ~48-bit significand; each operation costs a handful of FP32
// instructions, built from the error-free transformations of Dekker (1971,
// two-product, here through fmaf) and Knuth (TAOCP vol. 2, two-sum).  This is
// the "emulated FP64" form of the Fock build: about 1e-14 relative accuracy
// per operation, float exponent range (values below ~1e-30 lose the low word;
// below 1.2e-38 they flush to zero -- far below anything that reaches J or K).
#pragma once
#include <cuda_runtime.h>

#include "boys.cuh"

struct df64 {
    float hi, lo;
    __host__ __device__ constexpr df64() : hi(0.f), lo(0.f) {}
    __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr df64(int k) : hi((float)k), lo(0.f) {}
    __host__ __device__ constexpr explicit df64(float h) : hi(h), lo(0.f) {}
    // exact split of a double (used on compile-time constants and on the host)
    __host__ __device__ constexpr df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

__device__ __forceinline__ df64 df_quick_two_sum(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return df64(s, b - (s - a));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
    const float s = a.hi + b.hi;
    const float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);  // two-sum error of the high words
    e += a.lo + b.lo;
    return df_quick_two_sum(s, e);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);  // two-product error, exact through the FMA
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_quick_two_sum(p, e);
}

__device__ __forceinline__ df64 &operator+=(df64 &a, df64 b) {
    a = a + b;
    return a;
}

// a*b + c with one renormalisation
__device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const float s = p + c.hi;
    const float v = s - p;
    e += (p - (s - v)) + (c.hi - v);
    e += c.lo;
    return df_quick_two_sum(s, e);
}

// 1/sqrt(x): single-precision seed, one Newton step in df64 (23 -> ~46 bits)
__device__ __forceinline__ df64 df_rsqrt(df64 x) {
    const float y0 = rsqrtf(x.hi);
    const df64 y(y0, 0.f);
    const df64 r = df64(1) - x * (y * y);  // 1 - x y^2, tiny
    return df_fma(y * df64(0.5f, 0.f), r, y);
}

__device__ __forceinline__ df64 &operator*=(df64 &a, df64 b) {
    a = a * b;
    return a;
}
__device__ __forceinline__ bool rchem_lt(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool boys_small(df64 T) { return rchem_lt(T, df64(40.0f)); }
__device__ __forceinline__ float rchem_tofloat(df64 a) { return a.hi; }
__device__ __forceinline__ df64 rchem_fma(df64 a, df64 b, df64 c) { return df_fma(a, b, c); }
__device__ __forceinline__ df64 rchem_rsqrt(df64 x) { return df_rsqrt(x); }
__device__ __forceinline__ df64 rchem_ldg(const df64 *p) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return df64(v.x, v.y);
}
// nearest grid row from the high word (the low word cannot move it by more
// than an ulp of T, far inside the Taylor radius); x = T_i - T exactly in df64
__device__ __forceinline__ void boys_grid(df64 T, int &i, df64 &x) {
    const float magic = 12582912.0f;  // 2^23 + 2^22
    const float t = fmaf(T.hi, (float)BOYS_INVH64, magic);
    i = __float_as_int(t) - __float_as_int(magic);
    x = df64((t - magic) * (float)BOYS_H64, 0.f) - T;
}
__device__ __forceinline__ df64 __shfl_xor_sync(unsigned mask, df64 v, int lane) {
    return df64(__shfl_xor_sync(mask, v.hi, lane), __shfl_xor_sync(mask, v.lo, lane));
}
