// pq_table.cuh -- per primitive quartet factors of the two exponents p, q.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "boys.cuh"
#include "df64.cuh"

// The factors of a primitive quartet that depend only on the two exponents p
// and q: rs = 1/sqrt(p+q), ipq = 1/(p+q), rho = pq/(p+q), qi = q/(p+q),
// pi = p/(p+q).  With a table (a.npq > 0; FP64 and double-float) they are two
// loads indexed by the primitive pairs' exponent numbers, which takes the
// reciprocal square root and four products off the FP64 pipe; FP32 computes them.
template <typename R> struct PqLoad;
template <> struct PqLoad<double> {
    template <typename A>
    static __device__ __forceinline__ void get(const A &a, int e, double &rs, double &rho, double &qi, double &pi) {
        const double2 v0 = __ldg(a.pq64 + 2 * e), v1 = __ldg(a.pq64 + 2 * e + 1);
        rs = v0.x; rho = v0.y; qi = v1.x; pi = v1.y;
    }
};
template <> struct PqLoad<df64> {
    template <typename A>
    static __device__ __forceinline__ void get(const A &a, int e, df64 &rs, df64 &rho, df64 &qi, df64 &pi) {
        const float4 v0 = __ldg(a.pqdf + 2 * e), v1 = __ldg(a.pqdf + 2 * e + 1);
        rs = df64(v0.x, v0.y); rho = df64(v0.z, v0.w); qi = df64(v1.x, v1.y); pi = df64(v1.z, v1.w);
    }
};
// (A: any argument block with the npq, prim_eid, pq64 and pqdf members;
// TAB = false: always computed, for kernels that the table's loads in flight
// would push past the register file)
template <typename R, bool TAB = true, typename A>
__device__ __forceinline__ void pq_factors(const A &a, int ib, int ik, R p, R q, R &rs, R &ipq, R &rho, R &qi,
                                           R &pi) {
    if constexpr (TAB && !std::is_same<R, float>::value) {
        if (a.npq) {  // launch-uniform
            PqLoad<R>::get(a, __ldg(a.prim_eid + ib) * a.npq + __ldg(a.prim_eid + ik), rs, rho, qi, pi);
            ipq = rs * rs;
            return;
        }
    }
    rs = rchem_rsqrt(p + q);
    ipq = rs * rs;
    qi = q * ipq;
    pi = p * ipq;
    rho = p * qi;
}
