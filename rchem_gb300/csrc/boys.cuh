// boys.cuh -- Boys function F_m(T) = int_0^1 t^(2m) exp(-T t^2) dt, FP64 and FP32.
//
// The reference evaluates F_m with a Numerical-Recipes incomplete gamma
// function (libpyquante2/cints.c:302-373, relative error ~1e-7).  Here:
//   T < BOYS_TMAX: Taylor expansion about the nearest grid point T_i = i*h,
//     F_m(T_i + d) = sum_k F_{m+k}(T_i) (-d)^k / k!,  |d| <= h/2,
//     with NTAY terms (8 in FP64: remainder < 3e-17 F; 4 in FP32: < 5e-8 F);
//     either for every m ("direct") or for m = L only, followed by the
//     downward recursion F_m = (2T F_{m+1} + e^{-T}) / (2m+1), with
//     e^{-T} = e^{-T_i} e^{-d} from the same Taylor multipliers;
//   T >= BOYS_TMAX: F_0 = sqrt(pi/T)/2 (erfc(sqrt T) < 4e-19 there) and the
//     upward recursion F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T), stable for T > m.
// All F values come out multiplied by the caller's prefactor.
// The grid tables are filled on the host (rchem_gpu.cu) from the exact power
// series, in double, at exactly the T_i values used here.
#pragma once
#include "rchem_types.h"

// h = 1/16 is exact in binary, so T_i = i*h and d = T - T_i are exact in both
// precisions and the host tables are built at exactly the device's grid points.
#define BOYS_NGRID 641   // rows i = 0..640 (nearest-point rounding reaches 640 just below T = 40)
#define BOYS_NCOL 24
#define BOYS_TMAX 40.0
#define BOYS_INVH 16.0
#define BOYS_H 0.0625

template <typename R> struct BoysPrec;
template <> struct BoysPrec<double> { static constexpr int NTAY = 8; };
template <> struct BoysPrec<float> { static constexpr int NTAY = 4; };

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

template <typename R>
RCHEM_HD inline R rchem_ldg(const R *p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

// F[0..L] = pref * F_m(T).
template <int L, bool DIRECT, typename R>
RCHEM_HD inline void boys_eval(R T, R pref, const R *__restrict__ tab, const R *__restrict__ etab, R *F) {
    constexpr int NT = BoysPrec<R>::NTAY;
    if (T < R(BOYS_TMAX)) {
        const int i = (int)(T * R(BOYS_INVH) + R(0.5));
        const R d = T - R(i) * R(BOYS_H);
        const R *row = tab + i * BOYS_NCOL;
        R mult[NT];
#pragma unroll
        for (int k = 1; k < NT; ++k) mult[k] = -d * (R(1) / R(k));
        if (DIRECT) {
#pragma unroll
            for (int m = 0; m <= L; ++m) {
                R acc = rchem_ldg(row + m + NT - 1);
#pragma unroll
                for (int k = NT - 1; k >= 1; --k) acc = rchem_ldg(row + m + k - 1) + acc * mult[k];
                F[m] = acc * pref;
            }
        } else {
            R acc = rchem_ldg(row + L + NT - 1);
#pragma unroll
            for (int k = NT - 1; k >= 1; --k) acc = rchem_ldg(row + L + k - 1) + acc * mult[k];
            // e^{-T} = e^{-T_i} * e^{-d}; Taylor of e^{-d} with the multipliers mult[k] = -d/k
            R ex = R(1);
#pragma unroll
            for (int k = NT - 1; k >= 1; --k) ex = R(1) + ex * mult[k];
            ex *= rchem_ldg(etab + i) * pref;
            F[L] = acc * pref;
            const R T2 = T + T;
#pragma unroll
            for (int m = L - 1; m >= 0; --m) F[m] = (T2 * F[m + 1] + ex) * (R(1) / R(2 * m + 1));
        }
    } else {
        const R rs = rchem_rsqrt(T);
        const R inv2T = R(0.5) * rs * rs;
        const R ex = R(rchem_expf(-(float)T)) * pref;
        F[0] = R(0.88622692545275801365) * rs * pref;
#pragma unroll
        for (int m = 1; m <= L; ++m) F[m] = (R(2 * m - 1) * F[m - 1] - ex) * inv2T;
    }
}

// Runtime-L variant for the generic (non-class) kernels.
template <typename R>
RCHEM_HD inline void boys_eval_rt(int L, R T, R pref, const R *__restrict__ tab, R *F) {
    constexpr int NT = BoysPrec<R>::NTAY;
    if (T < R(BOYS_TMAX)) {
        const int i = (int)(T * R(BOYS_INVH) + R(0.5));
        const R d = T - R(i) * R(BOYS_H);
        const R *row = tab + i * BOYS_NCOL;
        R mult[NT];
        for (int k = 1; k < NT; ++k) mult[k] = -d * (R(1) / R(k));
        for (int m = 0; m <= L; ++m) {
            R acc = rchem_ldg(row + m + NT - 1);
            for (int k = NT - 1; k >= 1; --k) acc = rchem_ldg(row + m + k - 1) + acc * mult[k];
            F[m] = acc * pref;
        }
    } else {
        const R rs = rchem_rsqrt(T);
        const R inv2T = R(0.5) * rs * rs;
        const R ex = R(rchem_expf(-(float)T)) * pref;
        F[0] = R(0.88622692545275801365) * rs * pref;
        for (int m = 1; m <= L; ++m) F[m] = (R(2 * m - 1) * F[m - 1] - ex) * inv2T;
    }
}
