// boys.cuh -- Boys function F_m(T) = int_0^1 t^(2m) exp(-T t^2) dt, FP64 and FP32.
//
// The reference evaluates F_m with a Numerical-Recipes incomplete gamma
// function (libpyquante2/cints.c:302-373, relative error ~1e-7).  Here:
//   T < BOYS_TMAX: a polynomial in x = T_i - T about the nearest grid point
//     T_i = i*h, from the Taylor expansion
//     F_m(T_i + d) = sum_k F_{m+k}(T_i) (-d)^k / k!,  |d| <= h/2:
//     FP64 (h = 1/128): the 7-term expansion economized to 5 coefficients on
//     |x| <= h/2 (Chebyshev economization: x^6 and x^5 replaced by their
//     best lower-degree approximations, error <= (a_5 + a_6 h/2) (h/2)^5 / 16
//     ~ 5e-16 F); FP32 (h = 1/64): 4 Taylor terms (< 2e-10 F).
//     The tables hold the coefficients, one sub-table per m (and one for
//     e^{-T} = e^{-T_i} e^{-d}), so an evaluation is a pure Horner chain in x:
//     NTAY-1 fused multiply-adds.  Small L evaluates
//     every F_m that way ("direct"); larger L evaluates F_L and e^{-T} and runs
//     the downward recursion F_m = (2T F_{m+1} + e^{-T}) / (2m+1).
//   T >= BOYS_TMAX: F_0 = sqrt(pi/T)/2 (erfc(sqrt T) < 4e-19 there) and the
//     upward recursion F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T), stable for T > m.
// All F values come out multiplied by the caller's prefactor.
// The FP64 grid index and the T < TMAX test use integer operations on T's bits,
// so only the Taylor chains and one subtraction run on the (narrow) FP64 pipe.
// boys_eval_u, the FP64 ERI kernels' form, removes the branch: below a switch
// point (40 for L <= 1, 80 above, the FP64 table extended to T < 80) a lane
// takes a Taylor row, above it a row of a power-law table, both chosen with
// integer operations, so a warp whose lanes straddle the switch issues one
// instruction stream.
#pragma once
#include <math.h>
#include <string.h>

#include <type_traits>

#include "rchem_types.h"

// h = 1/128 (FP64) and 1/64 (FP32) are exact in binary, so T_i = i*h and
// T_i - T are exact and the host tables are built at exactly the device's grid
// points.  Rows i = 0..T_end/h (nearest-point rounding reaches the last one
// just below T_end: 80 for the FP64 table, 40 for the FP32 one).
#define BOYS_MMAX 16     // F_0 .. F_16
#define BOYS_NSUB (BOYS_MMAX + 2)  // sub-table 0 = e^{-T}, sub-table m+1 = F_m
#define BOYS_TMAX 40.0
#define BOYS_NGRID64 10241  // T < 80: the branch-free evaluation (boys_eval_u) uses rows past T = 40
#define BOYS_INVH64 128.0
#define BOYS_H64 0.0078125
#define BOYS_NT64 5
// Power-law table of boys_eval_u for T beyond the Taylor range: F_m(T) =
// Gamma(m+1/2)/2 T^-(m+1/2) (the e^{-T} terms are below 1e-17 of F_m for m <= 1
// at T >= 40 and for m <= 8 at T >= 80).  T = 2^(2k+par) v with v in [1, 2];
// sub-table (par, m) holds, at v_j = 1 + j/BOYS_FAR_R, 5 coefficients of
// Gamma(m+1/2)/2 2^-(par (m+1/2)) v^-(m+1/2) in x = v_j - v (7 Taylor terms
// economized on |x| <= 1/(2 BOYS_FAR_R)); the factor 2^-(k (2m+1)) goes on
// by the exponent field.  A row of zeros (the far e^{-T}) follows the rows.
#define BOYS_FAR_R 2048
#define BOYS_FAR_ROWS (BOYS_FAR_R + 1)
#define BOYS_FAR_M 9  // m = 0..8 (the class kernels' L <= 8)
#define BOYS_FAR_ZERO (2 * BOYS_FAR_M * BOYS_FAR_ROWS * BOYS_NT64)
#define BOYS_FAR_SIZE (BOYS_FAR_ZERO + BOYS_NT64)
#define BOYS_NGRID32 2561
#define BOYS_INVH32 64.0
#define BOYS_H32 0.015625
#define BOYS_NT32 4

template <typename R> struct BoysPrec {  // double, double-float
    static constexpr int NTAY = BOYS_NT64, NGRID = BOYS_NGRID64;
};
template <> struct BoysPrec<float> { static constexpr int NTAY = BOYS_NT32, NGRID = BOYS_NGRID32; };

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

// table element (sub-table s, grid row i, coefficient k) of a table of ngrid rows
RCHEM_HD inline int boys_idx(int s, int i, int k, int nt, int ngrid) { return (s * ngrid + i) * nt + k; }

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

// nearest FP64 grid row i and x = T_i - T, for 0 <= T < BOYS_TMAX.  On the
// device the row comes from T's bits with integer operations (T = m 2^(e-52),
// so T/h = m 2^(e-45), rounded half up) and T_i = i h is assembled as a double
// from i's bits, leaving one FP64 subtraction; the host rounds with the
// 2^52 + 2^51 addition.  Either rounding keeps |x| <= h/2.
RCHEM_HD inline void boys_grid(double T, int &i, double &x) {
#ifdef __CUDA_ARCH__
    const long long bits = __double_as_longlong(T);
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;  // T < 40: e <= 5
    const int sh = 45 - e;                              // >= 40
    const long long m = (bits & 0xfffffffffffffLL) | 0x10000000000000LL;
    i = (e < -1022 || sh >= 63) ? 0 : (int)((m + (1LL << (sh - 1))) >> sh);
    double Ti = 0.0;
    if (i > 0) {
        const int msb = 31 - __clz(i);  // i h = i 2^-7: exponent msb - 7, mantissa i's lower bits
        Ti = __longlong_as_double(((long long)(msb - 7 + 1023) << 52) |
                                  (((long long)i << (52 - msb)) & 0xfffffffffffffLL));
    }
    x = Ti - T;
#else
    const double magic = 6755399441055744.0;  // 2^52 + 2^51
    const double t = fma(T, BOYS_INVH64, magic);
    long long bits;
    memcpy(&bits, &t, sizeof(bits));
    i = (int)(bits & 0xffffffffLL);
    x = fma(t - magic, BOYS_H64, -T);
#endif
}
RCHEM_HD inline void boys_grid(float T, int &i, float &x) {
    const float magic = 12582912.0f;  // 2^23 + 2^22
    const float t = fmaf(T, (float)BOYS_INVH32, magic);
#ifdef __CUDA_ARCH__
    i = __float_as_int(t) - __float_as_int(magic);
#else
    int bits, mb;
    memcpy(&bits, &t, sizeof(bits));
    memcpy(&mb, &magic, sizeof(mb));
    i = bits - mb;
#endif
    x = fmaf(t - magic, (float)BOYS_H32, -T);
}

template <typename R>
RCHEM_HD inline R boys_horner(const R *__restrict__ tab, int s, int i, R x) {
    constexpr int NT = BoysPrec<R>::NTAY;
    const R *c = tab + boys_idx(s, i, 0, NT, BoysPrec<R>::NGRID);
#ifdef __CUDA_ARCH__
    if constexpr (std::is_same<R, float>::value && NT == 4) {
        // an FP32 row is 16 aligned bytes: one vector load (the FP32 kernels
        // are bound by their global-load instructions, not their arithmetic)
        const float4 v = __ldg(reinterpret_cast<const float4 *>(c));
        return fmaf(fmaf(fmaf(v.w, x, v.z), x, v.y), x, v.x);
    }
#endif
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

#ifdef __CUDACC__
// v 2^k by the exponent field (integer operations; k = 0 leaves v as it is):
// zero, subnormals, infinities and NaN unchanged, results below the normal
// range flushed to zero.
__device__ __forceinline__ double boys_ldexp(double v, int k) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((u >> 52) & 0x7ff), f = e + k;
    if (e == 0 || e == 0x7ff) return v;
    if (f <= 0) return 0.0;
    return __longlong_as_double((long long)((u & ~(0x7ffULL << 52)) | ((unsigned long long)f << 52)));
}

template <int NT>
__device__ __forceinline__ double boys_horner_at(const double *__restrict__ c, double x) {
    double acc = __ldg(c + NT - 1);
#pragma unroll
    for (int k = NT - 2; k >= 0; --k) acc = fma(acc, x, __ldg(c + k));
    return acc;
}

// F[0..L] (times pref with SCALE) in FP64 for the class kernels, with one FP64
// instruction stream for every T: below the switch point (40 for L <= 1, 80
// above) a row of the Taylor table at T_i = i/128, above it a row of the
// power-law table at v_j, T = 2^(2k+par) v; the row, its grid point and the
// argument are chosen with integer operations, so the lanes of a warp with T
// on either side run the same x = grid - argument, the same Horner chains and,
// for L >= 2, the same downward recursion (e^{-T} from the zero row above the
// switch), instead of both branches of boys_eval.
template <int L, bool SCALE>
__device__ __forceinline__ void boys_eval_u(double T, double pref, const double *__restrict__ tab,
                                            const double *__restrict__ far, double *F) {
    constexpr int NT = BOYS_NT64, NG = BOYS_NGRID64;
    const long long bits = __double_as_longlong(T);
    const bool nr = bits < (L <= 1 ? 0x4044000000000000LL : 0x4054000000000000LL);  // T < 40 / T < 80
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    const long long man = bits & 0xfffffffffffffLL;
    // Taylor row: i = T 128 rounded half up (clamped, so far lanes hold an unused valid row)
    int sh = 45 - e;
    sh = sh < 1 ? 1 : sh;
    int i = (e < -1022 || sh >= 63) ? 0 : (int)min((long long)(NG - 1), ((man | (1LL << 52)) + (1LL << (sh - 1))) >> sh);
    long long gb_near = 0;
    if (i > 0) {
        const int msb = 31 - __clz(i);  // i/128: exponent msb - 7, mantissa i's lower bits
        gb_near = ((long long)(msb - 7 + 1023) << 52) | (((long long)i << (52 - msb)) & 0xfffffffffffffLL);
    }
    // power-law row: v = T 2^-e in [1, 2), j = (v - 1) BOYS_FAR_R rounded, v_j = 1 + j/BOYS_FAR_R
    // (j = BOYS_FAR_R carries into the exponent: v_j = 2)
    const int par = e & 1, k = e >> 1;
    const int j = (int)((man + (1LL << 40)) >> 41);
    const long long gb_far = (1023LL << 52) + ((long long)j << 41);
    const long long ab_far = man | (1023LL << 52);
    const double x = __longlong_as_double(nr ? gb_near : gb_far) - __longlong_as_double(nr ? bits : ab_far);
    auto row = [&](int m) {  // F_m's row (m <= L)
        return nr ? tab + boys_idx(m + 1, i, 0, NT, NG) : far + ((par * BOYS_FAR_M + m) * BOYS_FAR_ROWS + j) * NT;
    };
    auto sc = [&](double v) { return SCALE ? v * pref : v; };
    if (L <= BOYS_DIRECT_MAXL) {
#pragma unroll
        for (int m = 0; m <= L; ++m) F[m] = sc(boys_ldexp(boys_horner_at<NT>(row(m), x), nr ? 0 : -k * (2 * m + 1)));
    } else {
        const double *pex = nr ? tab + boys_idx(0, i, 0, NT, NG) : far + BOYS_FAR_ZERO;
        const double ex = sc(boys_horner_at<NT>(pex, x));
        F[L] = sc(boys_ldexp(boys_horner_at<NT>(row(L), x), nr ? 0 : -k * (2 * L + 1)));
        const double T2 = T + T;
#pragma unroll
        for (int m = L - 1; m >= 0; --m) F[m] = fma(T2, F[m + 1], ex) * rchem_recip<double>(2 * m + 1);
    }
}
#endif

#ifdef __CUDACC__
// FP32 quartets with the recursion in FP64 (RCHEM_JK_FP32_REC64): the Taylor
// values F_L and e^{-T} (T < 40) or F_0 and e^{-T} (above) in FP32 as in
// boys_eval, the downward (upward) recursion over m in FP64, the results
// rounded to FP32 (times pref with SCALE).
template <int L, bool SCALE>
__device__ __forceinline__ void boys_eval_rec64(float T, float pref, const float *__restrict__ tab, float *F) {
    double Fd[L + 1];
    if (boys_small(T)) {
        int i;
        float x;
        boys_grid(T, i, x);
        const double ex = (double)boys_horner<float>(tab, 0, i, x);
        Fd[L] = (double)boys_horner<float>(tab, L + 1, i, x);
        const double T2 = 2.0 * (double)T;
#pragma unroll
        for (int m = L - 1; m >= 0; --m) Fd[m] = fma(T2, Fd[m + 1], ex) * rchem_recip<double>(2 * m + 1);
    } else {
        const float rs = rsqrtf(T);
        const double inv2T = (double)(0.5f * rs * rs), ex = (double)expf(-T);
        Fd[0] = (double)(0.88622692545275801365f * rs);
#pragma unroll
        for (int m = 1; m <= L; ++m) Fd[m] = (double(2 * m - 1) * Fd[m - 1] - ex) * inv2T;
    }
#pragma unroll
    for (int m = 0; m <= L; ++m) F[m] = SCALE ? (float)Fd[m] * pref : (float)Fd[m];
}
#endif

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

// Host: fill the FP64 and FP32 tables (sizes boys_table_size(nt, ngrid)).
inline size_t boys_table_size(int nt, int ngrid) { return (size_t)BOYS_NSUB * ngrid * nt; }

// F_0..F_mtop at x (host, long double: a 64- or 113-bit significand, so the
// tables carry each F_m rounded once to double): F_mtop from its series
// e^{-x} sum_k (2x)^k / prod_{i=0..k} (2m+2i+1) (every term positive), the
// rest by the stable downward recursion F_m = (2x F_{m+1} + e^{-x}) / (2m+1).
inline void boys_row_host(double x, int mtop, double *F) {
    long double term = 1.0L / (2 * mtop + 1), sum = term;
    const long double x2 = 2.0L * x, ex = expl(-(long double)x);
    for (int k = 1; k < 4000; ++k) {
        term *= x2 / (2 * mtop + 2 * k + 1);
        sum += term;
        if (term < sum * 1e-24L) break;
    }
    long double f = ex * sum;
    F[mtop] = (double)f;
    for (int m = mtop - 1; m >= 0; --m) {
        f = (x2 * f + ex) / (2 * m + 1);
        F[m] = (double)f;
    }
}
// FP64: a_k = F_{m+k}(T_i) / k! for k = 0..6 economized on |x| <= d = h/2
// (u = x/d; u^5 -> (20 u^3 - 5 u)/16, u^6 -> (48 u^4 - 18 u^2 + 1)/32, the
// Chebyshev polynomials T_5 and T_6 dropped); FP32: a_0..a_3.
inline void boys_econ5(const double *a, double *b) {
    const double d2 = 0.25 * BOYS_H64 * BOYS_H64, d4 = d2 * d2, d6 = d4 * d2;
    b[0] = a[0] + d6 / 32.0 * a[6];
    b[1] = a[1] - 5.0 / 16.0 * d4 * a[5];
    b[2] = a[2] - 9.0 / 16.0 * d4 * a[6];
    b[3] = a[3] + 5.0 / 4.0 * d2 * a[5];
    b[4] = a[4] + 3.0 / 2.0 * d2 * a[6];
}
// The power-law table (BOYS_FAR_SIZE doubles), coefficients in long double.
inline void boys_fill_far(double *far) {
    const long double d = 0.5L / BOYS_FAR_R, d2 = d * d, d4 = d2 * d2, d6 = d4 * d2;
    long double g_half = sqrtl(3.14159265358979323846264338327950288L);  // Gamma(1/2)
    for (int m = 0; m < BOYS_FAR_M; ++m) {
        const long double al = m + 0.5L, C0 = g_half / 2;  // Gamma(m+1/2)/2
        for (int par = 0; par < 2; ++par) {
            const long double C = par ? C0 * powl(2.0L, -al) : C0;
            for (int j = 0; j < BOYS_FAR_ROWS; ++j) {
                const long double g = 1.0L + (long double)j / BOYS_FAR_R, ig = 1.0L / g;
                long double a[7], rf = 1.0L, fk = 1.0L, gp = powl(g, -al);
                for (int q = 0; q < 7; ++q) {
                    a[q] = C * rf * gp / fk;  // C (al)_q g^-(al+q) / q!
                    rf *= al + q;
                    fk *= q + 1;
                    gp *= ig;
                }
                const long double b[5] = {a[0] + d6 / 32 * a[6], a[1] - 5.0L / 16 * d4 * a[5],
                                          a[2] - 9.0L / 16 * d4 * a[6], a[3] + 5.0L / 4 * d2 * a[5],
                                          a[4] + 3.0L / 2 * d2 * a[6]};
                for (int q = 0; q < BOYS_NT64; ++q)
                    far[((par * BOYS_FAR_M + m) * BOYS_FAR_ROWS + j) * BOYS_NT64 + q] = (double)b[q];
            }
        }
        g_half *= al;  // Gamma(m+3/2) = (m+1/2) Gamma(m+1/2)
    }
    for (int q = 0; q < BOYS_NT64; ++q) far[BOYS_FAR_ZERO + q] = 0.0;
}

inline void boys_fill_tables(double *t64, float *t32) {
    double fk[32];
    fk[0] = 1.0;
    for (int k = 1; k < 32; ++k) fk[k] = fk[k - 1] * k;
    constexpr int NA = 7;  // Taylor terms before the economization
    for (int i = 0; i < BOYS_NGRID64; ++i) {
        const double T = (double)i * BOYS_H64;  // exact
        double F[BOYS_MMAX + NA + 1], a[NA], b[BOYS_NT64];
        boys_row_host(T, BOYS_MMAX + NA, F);
        const double e = (double)expl(-(long double)T);
        for (int k = 0; k < NA; ++k) a[k] = e / fk[k];
        boys_econ5(a, b);
        for (int k = 0; k < BOYS_NT64; ++k) t64[boys_idx(0, i, k, BOYS_NT64, BOYS_NGRID64)] = b[k];
        for (int m = 0; m <= BOYS_MMAX; ++m) {
            for (int k = 0; k < NA; ++k) a[k] = F[m + k] / fk[k];
            boys_econ5(a, b);
            for (int k = 0; k < BOYS_NT64; ++k) t64[boys_idx(m + 1, i, k, BOYS_NT64, BOYS_NGRID64)] = b[k];
        }
    }
    for (int i = 0; i < BOYS_NGRID32; ++i) {
        const double T = (double)i * BOYS_H32;
        double F[BOYS_MMAX + BOYS_NT32 + 1];
        boys_row_host(T, BOYS_MMAX + BOYS_NT32, F);
        const double e = exp(-T);
        for (int k = 0; k < BOYS_NT32; ++k) t32[boys_idx(0, i, k, BOYS_NT32, BOYS_NGRID32)] = (float)(e / fk[k]);
        for (int m = 0; m <= BOYS_MMAX; ++m)
            for (int k = 0; k < BOYS_NT32; ++k)
                t32[boys_idx(m + 1, i, k, BOYS_NT32, BOYS_NGRID32)] = (float)(F[m + k] / fk[k]);
    }
}
