// boys.cuh -- Boys function F_m(T) = int_0^1 t^(2m) exp(-T t^2) dt, FP64 and FP32.
//
// The reference evaluates F_m with a Numerical-Recipes incomplete gamma
// function (libpyquante2/cints.c:302-373, relative error ~1e-7).  Here:
//   T < BOYS_TMAX: Taylor expansion about the nearest grid point T_i = i*h,
//     F_m(T_i + d) = sum_k F_{m+k}(T_i) (-d)^k / k!,  |d| <= h/2,
//     with NTAY terms (6 in FP64: remainder < 3e-16 F; 4 in FP32: < 2e-10 F).
//     The tables hold the coefficients already divided by k!, one sub-table per
//     m (and one for e^{-T} = e^{-T_i} e^{-d}), so an evaluation is a pure
//     Horner chain in x = -d: NTAY-1 fused multiply-adds.  Small L evaluates
//     every F_m that way ("direct"); larger L evaluates F_L and e^{-T} and runs
//     the downward recursion F_m = (2T F_{m+1} + e^{-T}) / (2m+1).
//   T >= BOYS_TMAX: F_0 = sqrt(pi/T)/2 (erfc(sqrt T) < 4e-19 there) and the
//     upward recursion F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T), stable for T > m.
// All F values come out multiplied by the caller's prefactor.
// The FP64 grid index and the T < TMAX test use integer operations on T's bits,
// so only the Taylor chains and one subtraction run on the (narrow) FP64 pipe.
#pragma once
#include <math.h>
#include <string.h>

#include "rchem_types.h"

// h = 1/64 is exact in binary, so T_i = i*h and d = T - T_i are exact in both
// precisions and the host tables are built at exactly the device's grid points.
// With |d| <= h/2 the Taylor remainder after NT terms is below
// F_m (h/2)^NT / NT!: 3e-16 relative for the 6 FP64 terms, 2e-10 for the 4 FP32 ones.
#define BOYS_NGRID 2561  // rows i = 0..2560 (nearest-point rounding reaches 2560 just below T = 40)
#define BOYS_MMAX 16     // F_0 .. F_16
#define BOYS_NSUB (BOYS_MMAX + 2)  // sub-table 0 = e^{-T}, sub-table m+1 = F_m
#define BOYS_TMAX 40.0
#define BOYS_INVH 64.0
#define BOYS_H 0.015625
#define BOYS_NT64 6
#define BOYS_NT32 4

template <typename R> struct BoysPrec { static constexpr int NTAY = BOYS_NT64; };  // double, double-float
template <> struct BoysPrec<float> { static constexpr int NTAY = BOYS_NT32; };

// 1/k for a small integer k, as a compile-time constant of type R
template <typename R> RCHEM_HD constexpr R rchem_recip(int k) { return R(1.0 / (double)k); }
template <> RCHEM_HD constexpr float rchem_recip<float>(int k) { return 1.0f / (float)k; }
RCHEM_HD inline bool rchem_lt(double a, double b) { return a < b; }
// T < BOYS_TMAX for T >= 0 (or -0), compared on the bit pattern: an integer
// compare keeps the test off the narrow FP64 pipe (NaN goes to the T >= TMAX
// branch, as with the floating-point compare)
RCHEM_HD inline bool boys_small(double T) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(T) < 0x4044000000000000LL;  // bits of 40.0
#else
    return T < BOYS_TMAX;
#endif
}
RCHEM_HD inline bool boys_small(float T) { return T < (float)BOYS_TMAX; }
RCHEM_HD inline bool rchem_lt(float a, float b) { return a < b; }
RCHEM_HD inline float rchem_tofloat(double a) { return (float)a; }
RCHEM_HD inline float rchem_tofloat(float a) { return a; }

// table element (sub-table s, grid row i, Taylor order k)
RCHEM_HD inline int boys_idx(int s, int i, int k, int nt) { return (s * BOYS_NGRID + i) * nt + k; }

RCHEM_HD inline double rchem_rsqrt(double x) {
#ifdef __CUDA_ARCH__
    return rsqrt(x);
#else
    return 1.0 / sqrt(x);
#endif
}
RCHEM_HD inline float rchem_rsqrt(float x) {
#ifdef __CUDA_ARCH__
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}

// e^{-T} only enters the T >= 40 branch as a correction below 1e-9 of F_m,
// so single precision is ample there (and it underflows harmlessly past 87).
RCHEM_HD inline float rchem_expf(float x) { return expf(x); }

RCHEM_HD inline double rchem_fma(double a, double b, double c) { return fma(a, b, c); }
RCHEM_HD inline float rchem_fma(float a, float b, float c) { return fmaf(a, b, c); }

template <typename R>
RCHEM_HD inline R rchem_ldg(const R *p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

// nearest grid row i and x = T_i - T, for 0 <= T < BOYS_TMAX.  On the device
// the row comes from T's bits with integer operations (T = m 2^(e-52), so
// T/h = m 2^(e-46), rounded half up) and T_i = i h is assembled as a double
// from i's bits, leaving one FP64 subtraction; the host rounds with the
// 2^52 + 2^51 addition.  Either rounding keeps |x| <= h/2.
RCHEM_HD inline void boys_grid(double T, int &i, double &x) {
#ifdef __CUDA_ARCH__
    const long long bits = __double_as_longlong(T);
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;  // T < 40: e <= 5
    const int sh = 46 - e;                              // >= 41
    const long long m = (bits & 0xfffffffffffffLL) | 0x10000000000000LL;
    i = (e < -1022 || sh >= 63) ? 0 : (int)((m + (1LL << (sh - 1))) >> sh);
    double Ti = 0.0;
    if (i > 0) {
        const int msb = 31 - __clz(i);  // i h = i 2^-6: exponent msb - 6, mantissa i's lower bits
        Ti = __longlong_as_double(((long long)(msb - 6 + 1023) << 52) |
                                  (((long long)i << (52 - msb)) & 0xfffffffffffffLL));
    }
    x = Ti - T;
#else
    const double magic = 6755399441055744.0;  // 2^52 + 2^51
    const double t = fma(T, BOYS_INVH, magic);
    long long bits;
    memcpy(&bits, &t, sizeof(bits));
    i = (int)(bits & 0xffffffffLL);
    x = fma(t - magic, BOYS_H, -T);
#endif
}
RCHEM_HD inline void boys_grid(float T, int &i, float &x) {
    const float magic = 12582912.0f;  // 2^23 + 2^22
    const float t = fmaf(T, (float)BOYS_INVH, magic);
#ifdef __CUDA_ARCH__
    i = __float_as_int(t) - __float_as_int(magic);
#else
    int bits, mb;
    memcpy(&bits, &t, sizeof(bits));
    memcpy(&mb, &magic, sizeof(mb));
    i = bits - mb;
#endif
    x = fmaf(t - magic, (float)BOYS_H, -T);
}

template <typename R>
RCHEM_HD inline R boys_horner(const R *__restrict__ tab, int s, int i, R x) {
    constexpr int NT = BoysPrec<R>::NTAY;
    const R *c = tab + boys_idx(s, i, 0, NT);
    R acc = rchem_ldg(c + NT - 1);
#pragma unroll
    for (int k = NT - 2; k >= 0; --k) acc = rchem_fma(acc, x, rchem_ldg(c + k));
    return acc;
}

// Direct evaluation of every F_m is cheaper up to this L.
#define BOYS_DIRECT_MAXL 1

// F[0..L] = pref * F_m(T); with SCALE false, F[0..L] = F_m(T) (pref unused), for
// callers that fold the prefactor into their own products.
template <int L, typename R, bool SCALE = true>
RCHEM_HD inline void boys_eval(R T, R pref, const R *__restrict__ tab, R *F) {
    auto sc = [&](R v) { return SCALE ? v * pref : v; };
    if (boys_small(T)) {
        int i;
        R x;
        boys_grid(T, i, x);
        if (L <= BOYS_DIRECT_MAXL) {
#pragma unroll
            for (int m = 0; m <= L; ++m) F[m] = sc(boys_horner(tab, m + 1, i, x));
        } else {
            const R ex = sc(boys_horner(tab, 0, i, x));
            F[L] = sc(boys_horner(tab, L + 1, i, x));
            const R T2 = T + T;
#pragma unroll
            for (int m = L - 1; m >= 0; --m) F[m] = rchem_fma(T2, F[m + 1], ex) * rchem_recip<R>(2 * m + 1);
        }
    } else {
        const R rs = rchem_rsqrt(T);
        const R inv2T = R(0.5) * rs * rs;
        F[0] = sc(R(0.88622692545275801365) * rs);
        if (L <= 1) {
            // e^{-T} / F_0 < 3e-17 for T >= 40: the correction is below FP64 rounding
#pragma unroll
            for (int m = 1; m <= L; ++m) F[m] = F[m - 1] * inv2T;
        } else {
            const R ex = sc(R(rchem_expf(-rchem_tofloat(T))));
#pragma unroll
            for (int m = 1; m <= L; ++m) F[m] = (R(2 * m - 1) * F[m - 1] - ex) * inv2T;
        }
    }
}

// Runtime-L variant for the generic (non-class) kernels; L <= BOYS_MMAX.
template <typename R>
RCHEM_HD inline void boys_eval_rt(int L, R T, R pref, const R *__restrict__ tab, R *F) {
    if (rchem_lt(T, R(BOYS_TMAX))) {
        int i;
        R x;
        boys_grid(T, i, x);
        for (int m = 0; m <= L; ++m) F[m] = boys_horner(tab, m + 1, i, x) * pref;
    } else {
        const R rs = rchem_rsqrt(T);
        const R inv2T = R(0.5) * rs * rs;
        const R ex = R(rchem_expf(-rchem_tofloat(T))) * pref;
        F[0] = R(0.88622692545275801365) * rs * pref;
        for (int m = 1; m <= L; ++m) F[m] = (R(2 * m - 1) * F[m - 1] - ex) * inv2T;
    }
}

// Host: fill the FP64 and FP32 tables (sizes boys_table_size(nt)).
inline size_t boys_table_size(int nt) { return (size_t)BOYS_NSUB * BOYS_NGRID * nt; }

inline double boys_series_host(int m, double x) {
    // F_m(x) = e^{-x} sum_k (2x)^k / prod_{i=0..k} (2m+2i+1): every term positive
    double term = 1.0 / (2 * m + 1), sum = term;
    for (int k = 1; k < 2000; ++k) {
        term *= 2.0 * x / (2 * m + 2 * k + 1);
        sum += term;
        if (term < sum * 1e-18) break;
    }
    return exp(-x) * sum;
}

inline void boys_fill_tables(double *t64, float *t32) {
    double fk[32];
    fk[0] = 1.0;
    for (int k = 1; k < 32; ++k) fk[k] = fk[k - 1] * k;
    for (int i = 0; i < BOYS_NGRID; ++i) {
        const double T = (double)i * BOYS_H;  // exact: h = 1/64
        double F[BOYS_MMAX + BOYS_NT64 + 1];
        for (int m = 0; m <= BOYS_MMAX + BOYS_NT64; ++m) F[m] = boys_series_host(m, T);
        const double e = exp(-T);
        for (int k = 0; k < BOYS_NT64; ++k) t64[boys_idx(0, i, k, BOYS_NT64)] = e / fk[k];
        for (int k = 0; k < BOYS_NT32; ++k) t32[boys_idx(0, i, k, BOYS_NT32)] = (float)(e / fk[k]);
        for (int m = 0; m <= BOYS_MMAX; ++m) {
            for (int k = 0; k < BOYS_NT64; ++k) t64[boys_idx(m + 1, i, k, BOYS_NT64)] = F[m + k] / fk[k];
            for (int k = 0; k < BOYS_NT32; ++k) t32[boys_idx(m + 1, i, k, BOYS_NT32)] = (float)(F[m + k] / fk[k]);
        }
    }
}
