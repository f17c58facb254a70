// eri_kernel.cuh -- the HGP ERI class kernel and its fused epilogues.
//
// Work unit: one warp = 32 consecutive quartets of one (bra pair group, ket
// pair group) combination -- same angular momenta and primitive-pair counts on
// both sides, so every lane runs the same primitive-loop trip counts; lanes
// may straddle bra pairs.  Per primitive quartet: Boys function, the generated
// Obara--Saika VRR into the [e0|f0] contraction accumulators (held in
// registers); per contracted quartet: the generated HRR, then
//   EPI_JK    -- the 8-fold-symmetric J/K scatter (contracted with D in
//                registers, then added with FP64 atomics into J-hat / K-hat:
//                the additions run in L2, not on the SM's narrow FP64 pipe),
//   EPI_STORE -- the dense ERI tensor (all 8 index permutations),
//   EPI_DIAG  -- the Schwarz diagonal max |(ab|ab)| (bra = ket = lane's pair).
//
// The reference computes the same quantities with no symmetry and no
// screening, one primitive ERI per call (src/basis.rs:383-428,
// libpyquante2/cints.c:72-115).
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "rchem_types.h"
#include "df64.cuh"
#include "boys.cuh"
#include "pq_table.cuh"

template <int LA, int LB, int LC, int LD> struct EriClass;

enum { EPI_JK = 0, EPI_STORE = 1, EPI_DIAG = 2 };

// Position of (ij|kl) in the 8-fold packed ERI array (the ordering of
// libpyquante2/cints.c:375-387): ij = i(i+1)/2 + j with i >= j, kl likewise,
// then the pair index of (max(ij,kl), min(ij,kl)).  64-bit: n = 608 reaches 1.7e10.
__host__ __device__ __forceinline__ size_t rchem_eri_pack8(size_t i, size_t j, size_t k, size_t l) {
    const size_t ij = i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
    const size_t kl = k >= l ? k * (k + 1) / 2 + l : l * (l + 1) / 2 + k;
    return ij >= kl ? ij * (ij + 1) / 2 + kl : kl * (kl + 1) / 2 + ij;
}

// One contracted integral into the ERI-tensor output: its 8 symmetric
// positions of the dense n^4 array, or its one packed position.
__device__ __forceinline__ void eri_put(const EriArgs &a, size_t N1, size_t i, size_t j, size_t k, size_t l,
                                        double v) {
    if (a.eri_packed) {
        a.eri[rchem_eri_pack8(i, j, k, l)] = v;
        return;
    }
    const size_t N2 = N1 * N1, N3 = N2 * N1;
    a.eri[i * N3 + j * N2 + k * N1 + l] = v;
    a.eri[j * N3 + i * N2 + k * N1 + l] = v;
    a.eri[i * N3 + j * N2 + l * N1 + k] = v;
    a.eri[j * N3 + i * N2 + l * N1 + k] = v;
    a.eri[k * N3 + l * N2 + i * N1 + j] = v;
    a.eri[l * N3 + k * N2 + i * N1 + j] = v;
    a.eri[k * N3 + l * N2 + j * N1 + i] = v;
    a.eri[l * N3 + k * N2 + j * N1 + i] = v;
}

template <typename R> struct PrimLoad;
template <> struct PrimLoad<double> {
    static __device__ __forceinline__ void get(const EriArgs &a, int idx, double &p, double &ohp, double *P,
                                               double *PA, double &K) {
        const double2 *q = reinterpret_cast<const double2 *>(a.prims + idx);
        const double2 v0 = __ldg(q), v1 = __ldg(q + 1), v2 = __ldg(q + 2), v3 = __ldg(q + 3), v4 = __ldg(q + 4);
        p = v0.x; ohp = v0.y; P[0] = v1.x; P[1] = v1.y; P[2] = v2.x; PA[0] = v2.y; PA[1] = v3.x; PA[2] = v3.y; K = v4.x;
    }
};
template <> struct PrimLoad<float> {
    static __device__ __forceinline__ void get(const EriArgs &a, int idx, float &p, float &ohp, float *P, float *PA,
                                               float &K) {
        const float4 *q = reinterpret_cast<const float4 *>(a.prims32 + idx);
        const float4 v0 = __ldg(q), v1 = __ldg(q + 1), v2 = __ldg(q + 2);
        p = v0.x; ohp = v0.y; P[0] = v0.z; P[1] = v0.w; P[2] = v1.x; PA[0] = v1.y; PA[1] = v1.z; PA[2] = v1.w; K = v2.x;
    }
};

// Widen a contribution to double for the FP64 atomic.  float -> double by
// rebuilding the bit pattern with integer operations, so the FP32 kernels put
// nothing on the narrow FP64 pipe (subnormal floats, below 1.2e-38, flush to 0).
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu, sgn = u & 0x80000000u;
    const unsigned ed = (e == 0xffu) ? 0x7ffu : e + 896u;  // rebias 127 -> 1023 (inf/nan kept)
    const unsigned hi = (e == 0u) ? sgn : (sgn | (ed << 20) | (m >> 3));
    const unsigned lo = (e == 0u) ? 0u : (m << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// v 2^k for the degeneracy weights of the J/K scatter (k = -3..1): the
// exponent field is adjusted with integer operations, so the weights cost no
// FP64 instruction.  Exact for normal v; zero, subnormals (below 2.2e-308,
// never a J/K contribution), infinities and NaN are returned unchanged, and a
// result below the normal range is flushed to zero.
__device__ __forceinline__ double scale_pow2(double v, int k) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((u >> 52) & 0x7ff), f = e + k;
    if (e == 0 || e == 0x7ff) return v;
    if (f <= 0) return 0.0;
    return __longlong_as_double((long long)((u & ~(0x7ffULL << 52)) | ((unsigned long long)f << 52)));
}
// one weighted J/K contribution s 2^k as the FP64 atomic's operand: FP32 scales
// on its own (wide) pipe, FP64 and double-float by the exponent field
__device__ __forceinline__ double jk_term(double s, int k) { return scale_pow2(s, k); }
__device__ __forceinline__ double jk_term(float s, int k) { return widen(s * __int_as_float((127 + k) << 23)); }

template <> struct PrimLoad<df64> {
    static __device__ __forceinline__ void get(const EriArgs &a, int idx, df64 &p, df64 &ohp, df64 *P, df64 *PA,
                                               df64 &K) {
        const float4 *q = reinterpret_cast<const float4 *>(a.primsdf + idx);
        const float4 v0 = __ldg(q), v1 = __ldg(q + 1), v2 = __ldg(q + 2), v3 = __ldg(q + 3), v4 = __ldg(q + 4);
        p = df64(v0.x, v0.y); ohp = df64(v0.z, v0.w);
        P[0] = df64(v1.x, v1.y); P[1] = df64(v1.z, v1.w); P[2] = df64(v2.x, v2.y);
        PA[0] = df64(v2.z, v2.w); PA[1] = df64(v3.x, v3.y); PA[2] = df64(v3.z, v3.w);
        K = df64(v4.x, v4.y);
    }
};

// double-float to double: both words widened exactly, one FP64 add per atomic
__device__ __forceinline__ double widen(df64 x) { return widen(x.hi) + widen(x.lo); }
__device__ __forceinline__ double jk_term(df64 s, int k) { return scale_pow2(widen(s), k); }

template <typename R> struct Tabs;
template <> struct Tabs<double> {
    static __device__ __forceinline__ const double *boys(const EriArgs &a) { return a.boys64; }
    static __device__ __forceinline__ double dens(const EriArgs &a, int i) { return __ldg(a.D + i); }
    static __device__ __forceinline__ void ab(const ShellPair &s, double *v) { v[0] = s.AB[0]; v[1] = s.AB[1]; v[2] = s.AB[2]; }
};
template <> struct Tabs<df64> {
    static __device__ __forceinline__ const df64 *boys(const EriArgs &a) {
        return reinterpret_cast<const df64 *>(a.boysdf);
    }
    static __device__ __forceinline__ df64 dens(const EriArgs &a, int i) {
        const float2 v = __ldg(a.Ddf + i);
        return df64(v.x, v.y);
    }
    static __device__ __forceinline__ void ab(const ShellPair &s, df64 *v) {
        v[0] = df64(s.AB32[0], s.ABlo[0]); v[1] = df64(s.AB32[1], s.ABlo[1]); v[2] = df64(s.AB32[2], s.ABlo[2]);
    }
};
template <> struct Tabs<float> {
    static __device__ __forceinline__ const float *boys(const EriArgs &a) { return a.boys32; }
    static __device__ __forceinline__ float dens(const EriArgs &a, int i) { return __ldg(a.D32 + i); }
    static __device__ __forceinline__ void ab(const ShellPair &s, float *v) { v[0] = s.AB32[0]; v[1] = s.AB32[1]; v[2] = s.AB32[2]; }
};

// Scaled Boys values F[0..L] of one primitive quartet.  The FP32 kernels take
// them in FP32 (a.f32_boys64 = 0), entirely in FP64 from the FP32 argument and
// prefactor (1), or with FP32 table values and the recursion over m in FP64
// (2), rounding the results to FP32.
// FP64 (and the FP64 Boys function of the FP32 quartets
// with f32_boys64 = 1) runs boys_eval_u, one instruction stream for T on either
// side of the Taylor range: those kernels are bound by the narrow FP64 pipe,
// where a diverged warp issuing both branches cost 12 % of the build.  The
// FP32 and double-float kernels keep boys_eval's two branches: they are bound
// by instruction issue, and the branch-free form's extra integer selects and
// loads cost them more than the divergence (measured: mixed 21.2 -> 22.3 ms,
// emulated 24.1 -> 27.2 ms on the (H2O)32 build).
template <int L, typename R, bool SCALE = true>
__device__ __forceinline__ void eri_boys(const EriArgs &a, R T, R pref, const R *btab, R *F) {
    static_assert(L <= BOYS_FAR_M - 1, "the power-law table holds m <= 8");
    if constexpr (std::is_same<R, float>::value) {
        if (a.f32_boys64 == 1) {  // values and recursion in FP64
            double Fd[L + 1];
            boys_eval_u<L, SCALE>((double)T, (double)pref, a.boys64, a.boysfar, Fd);
#pragma unroll
            for (int m = 0; m <= L; ++m) F[m] = (float)Fd[m];
            return;
        }
        if constexpr (L >= 2) {  // the recursion in FP64 (L <= 1 evaluates every F_m directly)
            if (a.f32_boys64 == 2) {
                boys_eval_rec64<L, SCALE>(T, pref, btab, F);
                return;
            }
        }
        boys_eval<L, R, SCALE>(T, pref, btab, F);
    } else if constexpr (std::is_same<R, double>::value) {
        boys_eval_u<L, SCALE>(T, pref, btab, a.boysfar, F);
    } else {
        boys_eval<L, R, SCALE>(T, pref, btab, F);
    }
}

template <int LA, int LB, int LC, int LD, typename R, int EPI>
__global__ void __launch_bounds__(128) eri_class_kernel(EriArgs a) {
    using C = EriClass<LA, LB, LC, LD>;
    constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND, L = C::L;
    const int lane = threadIdx.x & 31;
    const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (w >= a.ntasks) return;  // warp-uniform
    const EriTask t = a.tasks[w];
    const int lg = (t.nq_lg >> 8) & 7, nq = t.nq_lg & 255;
    const int G = 1 << lg, r = lane & (G - 1), qi = lane >> lg;
    const bool active = qi < nq;
    // walk the segment chain to this lane's quartet (inactive lanes repeat lane 0's)
    int sg = t.seg, off = t.off + (active ? qi : 0);
    EriSeg seg = a.segs[sg];
    while (off >= seg.count) {
        off -= seg.count;
        seg = a.segs[++sg];
    }
    const int bidx = seg.bra;
    const int kidx = seg.ket0 + off;
    const ShellPair bp = a.pairs[bidx];
    const ShellPair kp = a.pairs[kidx];

    R acc[C::NE * C::NF];
#pragma unroll
    for (int i = 0; i < C::NE * C::NF; ++i) acc[i] = R(0);

    const R *btab = Tabs<R>::boys(a);
    // one primitive quartet: Boys function, then the VRR into acc
    auto prim = [&](const R ohp, const R *P, const R *PA, const R Kab, const R ohq, const R *Q, const R *QC,
                    const R Kcd, const R rs, const R ipq, const R rho, const R qi_, const R pi_) {
        const R PQx = P[0] - Q[0], PQy = P[1] - Q[1], PQz = P[2] - Q[2];
        const R T = rho * (PQx * PQx + PQy * PQy + PQz * PQz);
        const R pref = Kab * Kcd * rs;
        R F[L + 1];
        if constexpr (L == 0) {
            // (ss|ss): the integral is pref F_0; the prefactor goes into the accumulating FMA
            eri_boys<0, R, false>(a, T, pref, btab, F);
            acc[0] = rchem_fma(F[0], pref, acc[0]);
        } else if constexpr (LA == 1 && LB == 0 && LC == 0 && LD == 0) {
            // (ps|ss): (PA_i F_0 + WP_i F_1) pref with WP = -q/(p+q) PQ, as
            // PA_i (pref F_0) + PQ_i (-pref q/(p+q) F_1)
            eri_boys<1, R, false>(a, T, pref, btab, F);
            const R f0 = F[0] * pref, f1 = F[1] * (pref * -qi_);
            acc[0] = rchem_fma(PQx, f1, rchem_fma(PA[0], f0, acc[0]));
            acc[1] = rchem_fma(PQy, f1, rchem_fma(PA[1], f0, acc[1]));
            acc[2] = rchem_fma(PQz, f1, rchem_fma(PA[2], f0, acc[2]));
        } else {
            eri_boys<L, R>(a, T, pref, btab, F);
            C::template vrr<R>(acc, F, PA[0], PA[1], PA[2], -qi_ * PQx, -qi_ * PQy, -qi_ * PQz, QC[0], QC[1], QC[2],
                               pi_ * PQx, pi_ * PQy, pi_ * PQz, ohp, ohq, R(0.5) * ipq, qi_, pi_);
        }
    };
    // the G lanes of a quartet split its npp_bra x npp_ket primitive quartets
    // (one flat loop: a single inlined copy of the VRR), then reduce
    const int nk = kp.npp, ntot = bp.npp * nk;
    for (int tq = r; tq < ntot; tq += G) {
        const int ia = tq / nk, ic = tq - ia * nk;
        R p, ohp, P[3], PA[3], Kab, q, ohq, Q[3], QC[3], Kcd, rs, ipq, rho, qi_, pi_;
        PrimLoad<R>::get(a, bp.prim0 + ia, p, ohp, P, PA, Kab);
        PrimLoad<R>::get(a, kp.prim0 + ic, q, ohq, Q, QC, Kcd);
        pq_factors<R>(a, bp.prim0 + ia, kp.prim0 + ic, p, q, rs, ipq, rho, qi_, pi_);
        prim(ohp, P, PA, Kab, ohq, Q, QC, Kcd, rs, ipq, rho, qi_, pi_);
    }
    for (int o = G >> 1; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < C::NE * C::NF; ++i) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
    // one lane per quartet finishes it
    const bool lead = active && r == 0;

    R AB[3], CD[3];
    Tabs<R>::ab(bp, AB);
    Tabs<R>::ab(kp, CD);
    R out[NA * NB * NC * ND];
    C::template hrr<R>(acc, out, AB[0], AB[1], AB[2], CD[0], CD[1], CD[2]);

#define IDX(ia, ib, ic, id) ((((ia) * NB + (ib)) * NC + (ic)) * ND + (id))
    if constexpr (EPI == EPI_DIAG) {
        if constexpr (LA == LC && LB == LD) {
            if (lead) {
                double m = 0.0;
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int ib = 0; ib < NB; ++ib) m = fmax(m, fabs((double)out[IDX(ia, ib, ia, ib)]));
                a.J[kidx] = sqrt(m);
            }
        }
        return;
    }
    // bra and ket belong to one geometry: its block of the packed matrices
    const int n = bp.mn;
    const int m0 = bp.aoA, n0 = bp.aoB, l0 = kp.aoA, s0 = kp.aoB;
    const int mo = bp.moff;
    if constexpr (EPI == EPI_STORE) {
        if (lead) {
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                    for (int ic = 0; ic < NC; ++ic)
#pragma unroll
                        for (int id = 0; id < ND; ++id)
                            eri_put(a, (size_t)n, m0 + ia, n0 + ib, l0 + ic, s0 + id, (double)out[IDX(ia, ib, ic, id)]);
        }
        return;
    }

    // ---- EPI_JK: degeneracy-weighted 8-fold scatter -------------------------
    // weight 2^kK (1/2 per diagonal pair and for bra = ket); J carries a factor 2
    const int kK = -(bp.diag + kp.diag + (bidx == kidx ? 1 : 0)), kJ = kK + 1;

    if (!lead) return;
    // J-hat bra block: 2 (ab|cd) D_cd
    {
        R Dcd[NC * ND];
#pragma unroll
        for (int ic = 0; ic < NC; ++ic)
#pragma unroll
            for (int id = 0; id < ND; ++id) Dcd[ic * ND + id] = Tabs<R>::dens(a, mo + (l0 + ic) * n + s0 + id);
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ib = 0; ib < NB; ++ib) {
                R s = R(0);
#pragma unroll
                for (int ic = 0; ic < NC; ++ic)
#pragma unroll
                    for (int id = 0; id < ND; ++id) s += out[IDX(ia, ib, ic, id)] * Dcd[ic * ND + id];
                atomicAdd(a.J + mo + (m0 + ia) * n + n0 + ib, jk_term(s, kJ));
            }
    }
    // J-hat ket block: 2 (ab|cd) D_ab
    {
        R Dab[NA * NB];
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ib = 0; ib < NB; ++ib) Dab[ia * NB + ib] = Tabs<R>::dens(a, mo + (m0 + ia) * n + n0 + ib);
#pragma unroll
        for (int ic = 0; ic < NC; ++ic)
#pragma unroll
            for (int id = 0; id < ND; ++id) {
                R s = R(0);
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int ib = 0; ib < NB; ++ib) s += out[IDX(ia, ib, ic, id)] * Dab[ia * NB + ib];
                atomicAdd(a.J + mo + (l0 + ic) * n + s0 + id, jk_term(s, kJ));
            }
    }
    // K-hat[a][c] += (ab|cd) D_bd
    {
        R Dbd[NB * ND];
#pragma unroll
        for (int ib = 0; ib < NB; ++ib)
#pragma unroll
            for (int id = 0; id < ND; ++id) Dbd[ib * ND + id] = Tabs<R>::dens(a, mo + (n0 + ib) * n + s0 + id);
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) {
                R s = R(0);
#pragma unroll
                for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                    for (int id = 0; id < ND; ++id) s += out[IDX(ia, ib, ic, id)] * Dbd[ib * ND + id];
                atomicAdd(a.K + mo + (m0 + ia) * n + l0 + ic, jk_term(s, kK));
            }
    }
    // K-hat[b][c] += (ab|cd) D_ad
    {
        R Dad[NA * ND];
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int id = 0; id < ND; ++id) Dad[ia * ND + id] = Tabs<R>::dens(a, mo + (m0 + ia) * n + s0 + id);
#pragma unroll
        for (int ib = 0; ib < NB; ++ib)
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) {
                R s = R(0);
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int id = 0; id < ND; ++id) s += out[IDX(ia, ib, ic, id)] * Dad[ia * ND + id];
                atomicAdd(a.K + mo + (n0 + ib) * n + l0 + ic, jk_term(s, kK));
            }
    }
    // K-hat[a][d] += (ab|cd) D_bc
    {
        R Dbc[NB * NC];
#pragma unroll
        for (int ib = 0; ib < NB; ++ib)
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) Dbc[ib * NC + ic] = Tabs<R>::dens(a, mo + (n0 + ib) * n + l0 + ic);
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int id = 0; id < ND; ++id) {
                R s = R(0);
#pragma unroll
                for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                    for (int ic = 0; ic < NC; ++ic) s += out[IDX(ia, ib, ic, id)] * Dbc[ib * NC + ic];
                atomicAdd(a.K + mo + (m0 + ia) * n + s0 + id, jk_term(s, kK));
            }
    }
    // K-hat[b][d] += (ab|cd) D_ac
    {
        R Dac[NA * NC];
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) Dac[ia * NC + ic] = Tabs<R>::dens(a, mo + (m0 + ia) * n + l0 + ic);
#pragma unroll
        for (int ib = 0; ib < NB; ++ib)
#pragma unroll
            for (int id = 0; id < ND; ++id) {
                R s = R(0);
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int ic = 0; ic < NC; ++ic) s += out[IDX(ia, ib, ic, id)] * Dac[ia * NC + ic];
                atomicAdd(a.K + mo + (n0 + ib) * n + s0 + id, jk_term(s, kK));
            }
    }
#undef IDX
}

// prec: 0 = FP64, 1 = FP32 (mixed form), 2 = double-float on the FP32 pipe
// (emulated FP64): the one-lane-group-per-quartet kernel has a double-float
// instantiation up to l_a+l_b+l_c+l_d = 4; the larger classes have one in the
// warp-cooperative kernel below (a list of those classes that runs the
// one-lane-group kernel stays FP64).
// ---------------------------------------------------------------------------
// Warp-cooperative J/K kernel for the large classes (EriClass::WC, total
// angular momentum 4 and up; double, float and double-float): one warp
// per contracted shell quartet, the recurrence intermediates in shared
// memory.  The generated program (EriProg) lists the VRR terms and the HRR
// terms level by level of their DAG; within a level the terms are independent
// (no term reads a slot another term of its level writes) and the 32 lanes
// take them in turn, one __syncwarp between levels.  Slots of dead values are
// reused from one level to the next, so a warp's array holds the live values
// of a level, not the whole DAG; terms are sorted by branch shape inside a
// level so lanes mostly agree on it.
// With QL = 16 or 8 lanes per quartet a warp runs 2 or 4 quartets of the list
// side by side, each in its own array: the per-primitive-quartet set-up and
// Boys function, which every lane of a quartet evaluates, then cost a warp
// instruction per 2 or 4 quartets, and levels and contractions smaller than 32
// terms leave fewer lanes idle (the classes whose shell quartets have one or
// two primitive quartets).
template <int LA, int LB, int LC, int LD> struct EriProg;

#define WC_U 4  // independent recurrence terms per lane and pass

// Shared memory of an SM and of one block (sm_103: 228 KB per SM, at most 227 KB
// per block, 1 KB of each block's share reserved by the runtime); the warps a
// kernel of ~128 registers per thread can keep resident (65536 / (32 * 128)).
#define RCHEM_SM_SMEM (228 * 1024)
#define RCHEM_BLOCK_SMEM (227 * 1024)
#define RCHEM_WC_MAX_WARPS 16

template <int LA, int LB, int LC, int LD, typename R, int QL = 32>
struct WcShape {
    using P = EriProg<LA, LB, LC, LD>;
    static_assert(QL == 32 || QL == 16 || QL == 8, "8, 16 or 32 lanes per quartet");
    static constexpr int QW = 32 / QL;  // quartets per warp
    // one quartet's array (elements of R); with several quartets per warp the
    // stride is 4 mod 16 elements, so the arrays start on different banks
    static constexpr int STRIDE = QW == 1 ? P::SCR : P::SCR + (20 - P::SCR % 16) % 16;
    static constexpr int PER_WARP = QW * STRIDE;
    static constexpr size_t BYTES = (size_t)PER_WARP * sizeof(R);
    // warps per block that keep the most warps resident on an SM (ties: the
    // larger block, so a block's warps spread over the SM's four schedulers)
    static constexpr int pick() {
        int best = 1, best_res = 0;
        for (int w = 1; w <= 8; ++w) {
            const size_t blk = (size_t)w * BYTES;
            if (blk > RCHEM_BLOCK_SMEM) break;
            int nb = (int)(RCHEM_SM_SMEM / (blk + 1024));
            int res = nb * w;
            if (res > RCHEM_WC_MAX_WARPS) res = RCHEM_WC_MAX_WARPS;
            if (res >= best_res) {
                best_res = res;
                best = w;
            }
        }
        return best;
    }
    static constexpr int WARPS = pick();
    static constexpr size_t SMEM = (size_t)WARPS * BYTES;
    static_assert(BYTES <= RCHEM_BLOCK_SMEM, "a warp's recurrence values exceed a block's shared memory");
};

// lanes per target of a warp-cooperative contraction of ntg sums of nl terms
// over the ql lanes of a quartet
constexpr int wc_split(int ntg, int nl, int ql) {
    int p = 1;
    while (2 * p * ntg <= ql && 2 * p <= nl) p *= 2;
    return p;
}

template <typename R>
__device__ __forceinline__ R wc_sel3(int i, R a, R b, R c) { return i == 0 ? a : (i == 1 ? b : c); }
template <typename R>
__device__ __forceinline__ R wc_sel4(int n, const R *v) {  // v[0..3] = 1..4 times a coefficient
    return n == 1 ? v[0] : (n == 2 ? v[1] : (n == 3 ? v[2] : v[3]));
}

template <int LA, int LB, int LC, int LD, typename R, int EPI = EPI_JK, int QL = 32>
__global__ void __launch_bounds__(256, 2) eri_wc_kernel(EriArgs a) {  // <= 128 registers
    using C = EriClass<LA, LB, LC, LD>;
    using P = EriProg<LA, LB, LC, LD>;
    using W = WcShape<LA, LB, LC, LD, R, QL>;
    static_assert(QL == 32 || EPI == EPI_JK, "the ERI-store and Schwarz epilogues run one quartet per warp");
    constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND, L = C::L, QW = W::QW;
    extern __shared__ __align__(16) unsigned char wc_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int sub = lane & (QL - 1), qs = lane / QL;  // lane within the quartet, quartet within the warp
    // the quartet's array: accumulators [0, NT), Boys values and VRR terms
    // above them; after the HRR the integrals (ab|cd) in their own slots
    R *S = reinterpret_cast<R *>(wc_smem) + wib * W::PER_WARP + qs * W::STRIDE;
    const int w = blockIdx.x * W::WARPS + wib;
    if (w * QW >= a.ntasks) return;  // warp-uniform
    // quartets past the end of the list (the last warp's) run on the list's
    // last task with no primitive quartets and no stores
    const bool valid = w * QW + qs < a.ntasks;
    const EriTask tk = a.tasks[valid ? w * QW + qs : a.ntasks - 1];
    int sg = tk.seg, off = tk.off;
    EriSeg seg = a.segs[sg];
    while (off >= seg.count) {
        off -= seg.count;
        seg = a.segs[++sg];
    }
    const int bidx = seg.bra, kidx = seg.ket0 + off;
    const ShellPair bp = a.pairs[bidx], kp = a.pairs[kidx];
    for (int k = sub; k < P::NT; k += QL) S[k] = R(0);
    const R *btab = Tabs<R>::boys(a);
    const uint4 *vprog = P::vrr();
    const int *vlev = P::vrrlv();
    const int nk = kp.npp, ntot = valid ? bp.npp * nk : 0;
    int nmax = ntot;  // the warp runs its quartets' primitive loops side by side
    if constexpr (QW > 1) nmax = __reduce_max_sync(0xffffffffu, ntot);
    for (int tq = 0; tq < nmax; ++tq) {
        // a quartet past its last primitive quartet computes on zeros and stores nothing
        const bool live = tq < ntot;
        R p = R(0), ohp = R(0), Pc[3] = {R(0), R(0), R(0)}, PA[3] = {R(0), R(0), R(0)}, Kab = R(0);
        R q = R(0), ohq = R(0), Qc[3] = {R(0), R(0), R(0)}, QC[3] = {R(0), R(0), R(0)}, Kcd = R(0);
        R rs = R(0), ipq = R(0), rho = R(0), qi_ = R(0), pi_ = R(0);
        if (QW == 1 || live) {
            const int ia = tq / nk, ic = tq - ia * nk;
            PrimLoad<R>::get(a, bp.prim0 + ia, p, ohp, Pc, PA, Kab);
            PrimLoad<R>::get(a, kp.prim0 + ic, q, ohq, Qc, QC, Kcd);
            pq_factors<R>(a, bp.prim0 + ia, kp.prim0 + ic, p, q, rs, ipq, rho, qi_, pi_);
        }
        const R PQx = Pc[0] - Qc[0], PQy = Pc[1] - Qc[1], PQz = Pc[2] - Qc[2];
        const R T = rho * (PQx * PQx + PQy * PQy + PQz * PQz);
        R F[L + 1];
        eri_boys<L, R>(a, T, Kab * Kcd * rs, btab, F);
        const R WP[3] = {-qi_ * PQx, -qi_ * PQy, -qi_ * PQz}, WQ[3] = {pi_ * PQx, pi_ * PQy, pi_ * PQz};
        const R ohpq = R(0.5) * ipq;
        const R cp[4] = {ohp, ohp + ohp, R(3) * ohp, R(4) * ohp};
        const R cq[4] = {ohq, ohq + ohq, R(3) * ohq, R(4) * ohq};
        const R cpq[4] = {ohpq, ohpq + ohpq, R(3) * ohpq, R(4) * ohpq};
        __syncwarp();  // the previous primitive quartet's terms have been read
#pragma unroll
        for (int m = 0; m <= L; ++m)
            if ((m & (QL - 1)) == sub) S[P::NT + m] = F[m];
        __syncwarp();
        // one term: X a + Y b [+ n1 c (c_ - rho d)] [+ n2 ohpq g]
        auto term = [&](const unsigned wd, R ta, R tb, R tc, R td, R tg) {
            const int dir = wd & 3, ket = (wd >> 2) & 1, n1 = (wd >> 3) & 7, n2 = (wd >> 6) & 7;
            const R X = ket ? wc_sel3(dir, QC[0], QC[1], QC[2]) : wc_sel3(dir, PA[0], PA[1], PA[2]);
            const R Y = ket ? wc_sel3(dir, WQ[0], WQ[1], WQ[2]) : wc_sel3(dir, WP[0], WP[1], WP[2]);
            R v = rchem_fma(Y, tb, X * ta);
            if (n1) v = rchem_fma(ket ? wc_sel4(n1, cq) : wc_sel4(n1, cp), rchem_fma(-(ket ? pi_ : qi_), td, tc), v);
            if (n2) v = rchem_fma(wc_sel4(n2, cpq), tg, v);
            return v;
        };
        // one pass: NS <= WC_U independent terms per lane, every program word,
        // then every operand, loaded before any result is stored (latency overlap)
        auto vpass = [&](const int t, const int e, auto nsc) {
            constexpr int NS = decltype(nsc)::value;
            uint4 o[NS];
            R ta[NS], tb[NS], tc[NS], td[NS], tg[NS];
#pragma unroll
            for (int u = 0; u < NS; ++u) o[u] = t + QL * u < e ? __ldg(vprog + t + QL * u) : make_uint4(0, 0, 0, 0);
#pragma unroll
            for (int u = 0; u < NS; ++u) {
                const unsigned n1 = (o[u].w >> 3) & 7, n2 = (o[u].w >> 6) & 7;
                ta[u] = S[o[u].x >> 16];
                tb[u] = S[o[u].y & 0xffff];
                tc[u] = n1 ? S[o[u].y >> 16] : R(0);
                td[u] = n1 ? S[o[u].z & 0xffff] : R(0);
                tg[u] = n2 ? S[o[u].z >> 16] : R(0);
            }
#pragma unroll
            for (int u = 0; u < NS; ++u) {
                const R v = term(o[u].w, ta[u], tb[u], tc[u], td[u], tg[u]);
                if (t + QL * u < e && (QW == 1 || live)) {
                    const unsigned dest = o[u].x & 0xffff, tg1 = o[u].w >> 9;
                    if (dest != 0xffffu) S[dest] = v;
                    if (tg1) S[tg1 - 1] += v;  // a target: into its contraction accumulator
                }
            }
        };
        for (int lv = 0; lv < P::NVL; ++lv) {
            const int e = __ldg(vlev + lv + 1);
            // passes over the level (warp-uniform): each takes only the term slots
            // that hold a term for some lane, so a small level's empty slots cost nothing
            for (int b = __ldg(vlev + lv); b < e; b += QL * WC_U) {
                const int ns = min(WC_U, (e - b + QL - 1) / QL);
                if (ns == 4) vpass(b + sub, e, std::integral_constant<int, 4>{});
                else if (ns == 3) vpass(b + sub, e, std::integral_constant<int, 3>{});
                else if (ns == 2) vpass(b + sub, e, std::integral_constant<int, 2>{});
                else vpass(b + sub, e, std::integral_constant<int, 1>{});
            }
            __syncwarp();
        }
    }
    // HRR on the contracted [e0|f0], in place
    R AB[3], CD[3];
    Tabs<R>::ab(bp, AB);
    Tabs<R>::ab(kp, CD);
    const uint2 *hprog = P::hrr();
    const int *hlev = P::hrrlv();
    auto hcoef = [&](const uint2 op) {
        const int dir = (op.y >> 16) & 255, side = op.y >> 24;
        return side ? wc_sel3(dir, CD[0], CD[1], CD[2]) : wc_sel3(dir, AB[0], AB[1], AB[2]);
    };
    auto hpass = [&](const int t, const int e, auto nsc) {
        constexpr int NS = decltype(nsc)::value;
        uint2 o[NS];
        R tx[NS], ty[NS];
#pragma unroll
        for (int u = 0; u < NS; ++u) o[u] = t + QL * u < e ? __ldg(hprog + t + QL * u) : make_uint2(0, 0);
#pragma unroll
        for (int u = 0; u < NS; ++u) {
            tx[u] = S[o[u].x >> 16];
            ty[u] = S[o[u].y & 0xffff];
        }
#pragma unroll
        for (int u = 0; u < NS; ++u) {
            const R v = rchem_fma(hcoef(o[u]), ty[u], tx[u]);
            if (t + QL * u < e) S[o[u].x & 0xffff] = v;
        }
    };
    for (int lv = 0; lv < P::NHL; ++lv) {
        const int e = __ldg(hlev + lv + 1);
        for (int b = __ldg(hlev + lv); b < e; b += QL * WC_U) {
            const int ns = min(WC_U, (e - b + QL - 1) / QL);
            if (ns == 4) hpass(b + sub, e, std::integral_constant<int, 4>{});
            else if (ns == 3) hpass(b + sub, e, std::integral_constant<int, 3>{});
            else if (ns == 2) hpass(b + sub, e, std::integral_constant<int, 2>{});
            else hpass(b + sub, e, std::integral_constant<int, 1>{});
        }
        __syncwarp();
    }
    // the integrals (ab|cd) scaled by their component norms, in place (every
    // output has a slot of its own); A(k) reads integral k
    const unsigned short *oslot = P::out();
    for (int k = sub; k < P::NOUT; k += QL) {
        const int sk = __ldg(oslot + k);
        S[sk] = R(__ldg(P::onorm() + k)) * S[sk];
    }
    __syncwarp();
    auto A = [&](int k) { return S[__ldg(oslot + k)]; };
    if constexpr (EPI == EPI_DIAG) {  // Schwarz bound sqrt(max |(ab|ab)|) of a diagonal quartet
        if constexpr (LA == LC && LB == LD) {
            double m = 0.0;
            for (int t = lane; t < NA * NB; t += 32) {
                const int ia = t / NB, ib = t - ia * NB;
                m = fmax(m, fabs((double)A(((ia * NB + ib) * NC + ia) * ND + ib)));
            }
            for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) a.J[kidx] = sqrt(m);
        }
        return;
    }
    if constexpr (EPI == EPI_STORE) {  // the ERI tensor: dense (8 positions) or packed (one)
        const int i0 = bp.aoA, j0 = bp.aoB, k0 = kp.aoA, l0s = kp.aoB;
        for (int t = lane; t < NA * NB * NC * ND; t += 32) {
            const int id = t % ND, ic = (t / ND) % NC, ib = (t / (ND * NC)) % NB, ia = t / (ND * NC * NB);
            eri_put(a, (size_t)bp.mn, i0 + ia, j0 + ib, k0 + ic, l0s + id, (double)A(t));
        }
        return;
    }

    // degeneracy-weighted 8-fold scatter: each of the six contractions is a
    // set of NTG target sums of NL terms; SPL lanes share a target (each a
    // strided part of its sum, then a shuffle reduction), SPL the largest power
    // of two with NTG SPL <= QL and SPL <= NL, so a contraction with few
    // targets still keeps the quartet's lanes busy
    const int kK = -(bp.diag + kp.diag + (bidx == kidx ? 1 : 0)), kJ = kK + 1;
    const int n = bp.mn, mo = bp.moff;
    const int m0 = bp.aoA, n0 = bp.aoB, l0 = kp.aoA, s0 = kp.aoB;
#define WIDX(ia, ib, ic, id) ((((ia) * NB + (ib)) * NC + (ic)) * ND + (id))
    auto contract = [&](auto ntg_c, auto nl_c, double *M, int kw, auto tgt, auto term) {
        constexpr int NTG = decltype(ntg_c)::value, NL = decltype(nl_c)::value;
        constexpr int SPL = wc_split(NTG, NL, QL), PER = QL / SPL;
        const int sl = sub & (SPL - 1);
        for (int t0 = 0; t0 < NTG; t0 += PER) {
            const int t = t0 + sub / SPL;
            R sum = R(0);
            if (t < NTG)
                for (int i = sl; i < NL; i += SPL) {
                    int ai, di;
                    term(t, i, ai, di);
                    sum = rchem_fma(A(ai), Tabs<R>::dens(a, di), sum);
                }
#pragma unroll
            for (int o = SPL >> 1; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            if (valid && t < NTG && sl == 0) atomicAdd(M + tgt(t), jk_term(sum, kw));
        }
    };
    using std::integral_constant;
    // J-hat bra: 2 (ab|cd) D_cd
    contract(integral_constant<int, NA * NB>{}, integral_constant<int, NC * ND>{}, a.J, kJ,
             [&](int t) { return mo + (m0 + t / NB) * n + n0 + t % NB; },
             [&](int t, int i, int &ai, int &di) {
                 const int ic = i / ND, id = i % ND;
                 ai = WIDX(t / NB, t % NB, ic, id);
                 di = mo + (l0 + ic) * n + s0 + id;
             });
    // J-hat ket: 2 (ab|cd) D_ab
    contract(integral_constant<int, NC * ND>{}, integral_constant<int, NA * NB>{}, a.J, kJ,
             [&](int t) { return mo + (l0 + t / ND) * n + s0 + t % ND; },
             [&](int t, int i, int &ai, int &di) {
                 const int ia = i / NB, ib = i % NB;
                 ai = WIDX(ia, ib, t / ND, t % ND);
                 di = mo + (m0 + ia) * n + n0 + ib;
             });
    // K-hat[a][c] += (ab|cd) D_bd
    contract(integral_constant<int, NA * NC>{}, integral_constant<int, NB * ND>{}, a.K, kK,
             [&](int t) { return mo + (m0 + t / NC) * n + l0 + t % NC; },
             [&](int t, int i, int &ai, int &di) {
                 const int ib = i / ND, id = i % ND;
                 ai = WIDX(t / NC, ib, t % NC, id);
                 di = mo + (n0 + ib) * n + s0 + id;
             });
    // K-hat[b][c] += (ab|cd) D_ad
    contract(integral_constant<int, NB * NC>{}, integral_constant<int, NA * ND>{}, a.K, kK,
             [&](int t) { return mo + (n0 + t / NC) * n + l0 + t % NC; },
             [&](int t, int i, int &ai, int &di) {
                 const int ia = i / ND, id = i % ND;
                 ai = WIDX(ia, t / NC, t % NC, id);
                 di = mo + (m0 + ia) * n + s0 + id;
             });
    // K-hat[a][d] += (ab|cd) D_bc
    contract(integral_constant<int, NA * ND>{}, integral_constant<int, NB * NC>{}, a.K, kK,
             [&](int t) { return mo + (m0 + t / ND) * n + s0 + t % ND; },
             [&](int t, int i, int &ai, int &di) {
                 const int ib = i / NC, ic = i % NC;
                 ai = WIDX(t / ND, ib, ic, t % ND);
                 di = mo + (n0 + ib) * n + l0 + ic;
             });
    // K-hat[b][d] += (ab|cd) D_ac
    contract(integral_constant<int, NB * ND>{}, integral_constant<int, NA * NC>{}, a.K, kK,
             [&](int t) { return mo + (n0 + t / ND) * n + s0 + t % ND; },
             [&](int t, int i, int &ai, int &di) {
                 const int ia = i / NC, ic = i % NC;
                 ai = WIDX(ia, t / ND, ic, t % ND);
                 di = mo + (m0 + ia) * n + l0 + ic;
             });
#undef WIDX
}

// Raise the shared-memory limit of the warp-cooperative kernels (once per
// device, outside any stream capture).
template <int LA, int LB, int LC, int LD, typename R, int EPI, int QL>
cudaError_t wc_set_smem() {
    return cudaFuncSetAttribute(eri_wc_kernel<LA, LB, LC, LD, R, EPI, QL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)WcShape<LA, LB, LC, LD, R, QL>::SMEM);
}
template <int LA, int LB, int LC, int LD, typename R>
cudaError_t wc_set_smem_jk() {
    cudaError_t e = wc_set_smem<LA, LB, LC, LD, R, EPI_JK, 32>();
    if (e == cudaSuccess) e = wc_set_smem<LA, LB, LC, LD, R, EPI_JK, 16>();
    if (e == cudaSuccess) e = wc_set_smem<LA, LB, LC, LD, R, EPI_JK, 8>();
    return e;
}

template <int LA, int LB, int LC, int LD>
cudaError_t prepare_eri_class() {
    if constexpr (EriClass<LA, LB, LC, LD>::WC) {
        cudaError_t e = wc_set_smem_jk<LA, LB, LC, LD, double>();
        if (e == cudaSuccess) e = wc_set_smem_jk<LA, LB, LC, LD, df64>();
        if (e == cudaSuccess) e = wc_set_smem_jk<LA, LB, LC, LD, float>();
        if (e != cudaSuccess) return e;
        if constexpr (EriClass<LA, LB, LC, LD>::WC_ONLY) {
            e = wc_set_smem<LA, LB, LC, LD, double, EPI_STORE, 32>();
            if (e != cudaSuccess) return e;
            if constexpr (LA == LC && LB == LD) e = wc_set_smem<LA, LB, LC, LD, double, EPI_DIAG, 32>();
        }
        return e;
    }
    return cudaSuccess;
}

// A warp-cooperative list: ceil(ntasks / QW) warps of QW quartets each.
template <int LA, int LB, int LC, int LD, typename R, int EPI, int QL>
void launch_wc(const EriArgs &a, cudaStream_t s) {
    using W = WcShape<LA, LB, LC, LD, R, QL>;
    const int warps = (a.ntasks + W::QW - 1) / W::QW;
    eri_wc_kernel<LA, LB, LC, LD, R, EPI, QL><<<(warps + W::WARPS - 1) / W::WARPS, 32 * W::WARPS, W::SMEM, s>>>(a);
}
template <int LA, int LB, int LC, int LD, typename R>
void launch_wc_jk(const EriArgs &a, cudaStream_t s) {
    if (a.wc == 8) launch_wc<LA, LB, LC, LD, R, EPI_JK, 8>(a, s);
    else if (a.wc == 16) launch_wc<LA, LB, LC, LD, R, EPI_JK, 16>(a, s);
    else launch_wc<LA, LB, LC, LD, R, EPI_JK, 32>(a, s);
}

// The one-lane-group-per-quartet kernel of a class list.  The classes of total
// angular momentum 6 build it in a translation unit of its own (compiled with
// ptxas -O1, see build.py) and reach it through launch_eri_class's ext.
template <int LA, int LB, int LC, int LD>
void launch_eri_cls_only(const EriArgs &a, int prec, int epi, cudaStream_t s) {
    if constexpr (!EriClass<LA, LB, LC, LD>::WC_ONLY) {
        if (a.ntasks <= 0) return;
        const int threads = 128;
        const long long nthreads = (long long)a.ntasks * 32;
        const int blocks = (int)((nthreads + threads - 1) / threads);
        if (epi == EPI_JK) {
            if (prec == 1) eri_class_kernel<LA, LB, LC, LD, float, EPI_JK><<<blocks, threads, 0, s>>>(a);
            else if constexpr (LA + LB + LC + LD <= 4) {
                if (prec == 2) eri_class_kernel<LA, LB, LC, LD, df64, EPI_JK><<<blocks, threads, 0, s>>>(a);
                else eri_class_kernel<LA, LB, LC, LD, double, EPI_JK><<<blocks, threads, 0, s>>>(a);
            } else {
                eri_class_kernel<LA, LB, LC, LD, double, EPI_JK><<<blocks, threads, 0, s>>>(a);
            }
        } else if (epi == EPI_STORE) {
            eri_class_kernel<LA, LB, LC, LD, double, EPI_STORE><<<blocks, threads, 0, s>>>(a);
        } else if constexpr (LA == LC && LB == LD) {
            eri_class_kernel<LA, LB, LC, LD, double, EPI_DIAG><<<blocks, threads, 0, s>>>(a);
        }
    }
}

using EriClsLaunch = void (*)(const EriArgs &, int, int, cudaStream_t);

template <int LA, int LB, int LC, int LD, bool EXT_CLS = false>
void launch_eri_class(const EriArgs &a, int prec, int epi, cudaStream_t s, EriClsLaunch ext = nullptr) {
    if (a.ntasks <= 0) return;
    if constexpr (EriClass<LA, LB, LC, LD>::WC_ONLY) {
        // the largest class, (dd|dd), exists only as warp-cooperative kernels (one
        // quartet per task in every plan); its straight-line code would take
        // minutes to compile
        if (epi == EPI_STORE) {
            launch_wc<LA, LB, LC, LD, double, EPI_STORE, 32>(a, s);
            return;
        }
        if (epi == EPI_DIAG) {
            if constexpr (LA == LC && LB == LD) launch_wc<LA, LB, LC, LD, double, EPI_DIAG, 32>(a, s);
            return;
        }
    }
    if constexpr (EriClass<LA, LB, LC, LD>::WC) {
        if (epi == EPI_JK && (a.wc || EriClass<LA, LB, LC, LD>::WC_ONLY)) {  // one quartet per task
            if (prec == 1) launch_wc_jk<LA, LB, LC, LD, float>(a, s);
            else if (prec == 2) launch_wc_jk<LA, LB, LC, LD, df64>(a, s);
            else launch_wc_jk<LA, LB, LC, LD, double>(a, s);
            return;
        }
    }
    if constexpr (EXT_CLS) ext(a, prec, epi, s);
    else launch_eri_cls_only<LA, LB, LC, LD>(a, prec, epi, s);
}
