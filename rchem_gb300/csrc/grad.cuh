// grad.cuh -- adjoint kernels for the nuclear gradient of the RHF energy.
//
// E = 2 sum D.H + sum D_mn D_ls [2(mn|ls) - (ml|ns)] + E_nuc  (the energy of
// src/bin/rchem.rs:106-108, D = C_occ C_occ^T without the factor 2).  With the
// energy-weighted density W = sum_i eps_i C_i C_i^T,
//   dE/dX = 2 sum D dH/dX + sum Gamma d(mn|ls)/dX - 2 sum W dS/dX + dE_nuc/dX,
//   Gamma_mnls = 2 D_mn D_ls - (D_ml D_ns + D_ms D_nl)/2.
// Derivatives of a Cartesian Gaussian centred on A (the shifted-angular-
// momentum relation): d/dA_x [x_A^l e^{-a r_A^2}] = 2a x_A^{l+1}(...) - l x_A^{l-1}(...).
// Integrals are evaluated by McMurchie--Davidson (Hermite) recursions with
// run-time angular momenta: compact code for every class up to (dd|dd)
// (shifted to l = 3 on one centre).  The derivative integrals are never
// stored: each contracted shell quartet is contracted with Gamma on the fly
// and only the 9 centre derivatives leave the warp (translational invariance
// gives the fourth centre).
#pragma once
#include <type_traits>

#include "boys.cuh"
#include "df64.cuh"
#include "md.cuh"
#include "pq_table.cuh"
#include "rchem_types.h"

#define GR_NI 4    // powers 0..3 per centre and direction (l <= 2, shifted by one)
#define GR_NT 7    // Hermite index t <= 6
#define GR_LMAX 9  // largest total L of a shifted quartet
#define GR_NR 220  // (t,u,v) with t+u+v <= 9

struct GradArgs {
    const EriTask *tasks;  // warp tasks over the surviving unique quartets
    const EriSeg *segs;
    int ntasks;
    const ShellPair *pairs;
    const PairPrim *prims;
    const PairPrim32 *prims32;    // the same in FP32 (mixed form) ...
    const PairPrimDF *primsdf;    // ... and double-float (emulated form)
    const float *boys32;
    const float2 *boysdf;
    const int *shell_atom;
    const int *shell_l;
    const double *boys64;
    const double *boysfar;  // the FP64 power-law table of boys_eval_u
    const double *D;
    double *grad;  // 3 * natoms
    int npq;       // exponent-pair factor table (EriArgs::npq and the three after it)
    const int *prim_eid;
    const double2 *pq64;
    const float4 *pqdf;
};

// E[i][j][t] of x_A^i x_B^j for i <= imax, j <= jmax (no exponential factor)
template <typename R, int NJ = GR_NI, int NT = GR_NT>
__device__ __forceinline__ void gr_herm(int imax, int jmax, R PA, R AB, R ohp, R (*E)[NJ][NT]) {
    const R PB = PA + AB;  // P - B = (P - A) + (A - B)
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j <= jmax; ++j)
            for (int t = 0; t < NT; ++t) E[i][j][t] = R(0);
    E[0][0][0] = R(1);
    for (int i = 0; i <= imax; ++i) {
        if (i > 0)
            for (int t = 0; t <= i; ++t) {
                R v = PA * E[i - 1][0][t];
                if (t > 0) v = rchem_fma(ohp, E[i - 1][0][t - 1], v);
                if (t + 1 <= i - 1) v = rchem_fma(R(t + 1), E[i - 1][0][t + 1], v);
                E[i][0][t] = v;
            }
        for (int j = 1; j <= jmax; ++j)
            for (int t = 0; t <= i + j; ++t) {
                R v = PB * E[i][j - 1][t];
                if (t > 0) v = rchem_fma(ohp, E[i][j - 1][t - 1], v);
                if (t + 1 <= i + j - 1) v = rchem_fma(R(t + 1), E[i][j - 1][t + 1], v);
                E[i][j][t] = v;
            }
    }
}

// R^0_tuv for t+u+v <= L (md_tuv order) into out, NR >= (L+1)(L+2)(L+3)/6
// values; the recursion alternates between out and one scratch table, starting
// in the one that makes the last pass land in out
template <typename R, int NR = GR_NR>
__device__ __forceinline__ void gr_R(int L, R a, R X, R Y, R Z, const R *F, R *out) {
    R buf[NR];
    R *cur = (L & 1) ? buf : out, *nxt = (L & 1) ? out : buf;
    const R m2a = R(-2) * a;
    R pw[GR_LMAX + 1];
    pw[0] = R(1);
    for (int n = 1; n <= L; ++n) pw[n] = pw[n - 1] * m2a;
    cur[0] = pw[L] * F[L];
    for (int n = L - 1; n >= 0; --n) {
        const int top = L - n;
        for (int N = 0; N <= top; ++N)
            for (int t = N; t >= 0; --t)
                for (int u = N - t; u >= 0; --u) {
                    const int v = N - t - u;
                    R r;
                    if (N == 0) r = pw[n] * F[n];
                    else if (t > 0) r = X * cur[md_tuv(t - 1, u, v)] + (t > 1 ? R(t - 1) * cur[md_tuv(t - 2, u, v)] : R(0));
                    else if (u > 0) r = Y * cur[md_tuv(0, u - 1, v)] + (u > 1 ? R(u - 1) * cur[md_tuv(0, u - 2, v)] : R(0));
                    else r = Z * cur[md_tuv(0, 0, v - 1)] + (v > 1 ? R(v - 1) * cur[md_tuv(0, 0, v - 2)] : R(0));
                    nxt[md_tuv(t, u, v)] = r;
                }
        R *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
}

__device__ __forceinline__ void gr_comp(int l, int k, int *lmn) {
    int idx = 0;
    for (int a = 1; a <= l + 1; ++a)
        for (int b = 1; b <= a; ++b, ++idx)
            if (idx == k) {
                lmn[0] = l + 1 - a;
                lmn[1] = a - b;
                lmn[2] = b - 1;
                return;
            }
}

__device__ __forceinline__ double gr_cnorm(const int *p) {
    // N(alpha,l,m,n) / N(alpha,L,0,0) = sqrt((2L-1)!! / ((2l-1)!!(2m-1)!!(2n-1)!!))
    const double f2[7] = {1.0, 1.0, 3.0, 15.0, 105.0, 945.0, 10395.0};  // (2k-1)!! for k = 0..6
    return sqrt(f2[p[0] + p[1] + p[2]] / (f2[p[0]] * f2[p[1]] * f2[p[2]]));
}

// primitive pair in the kernel's arithmetic: p, 1/(2p), P, P-A, K and the
// exponent on the pair's first shell (the derivative weight 2 alpha)
template <typename R> struct GradPrim;
template <> struct GradPrim<double> {
    static __device__ __forceinline__ void get(const GradArgs &g, int i, double &p, double &ohp, double *P, double *PA,
                                               double &K, double &ea) {
        const PairPrim q = g.prims[i];
        p = q.p; ohp = q.ohp; K = q.K; ea = q.pad;
        for (int d = 0; d < 3; ++d) { P[d] = q.P[d]; PA[d] = q.PA[d]; }
    }
    static __device__ __forceinline__ const double *boys(const GradArgs &g) { return g.boys64; }
};
template <> struct GradPrim<float> {
    static __device__ __forceinline__ void get(const GradArgs &g, int i, float &p, float &ohp, float *P, float *PA,
                                               float &K, float &ea) {
        const float4 *q = reinterpret_cast<const float4 *>(g.prims32 + i);
        const float4 v0 = __ldg(q), v1 = __ldg(q + 1), v2 = __ldg(q + 2);
        p = v0.x; ohp = v0.y; P[0] = v0.z; P[1] = v0.w; P[2] = v1.x; PA[0] = v1.y; PA[1] = v1.z; PA[2] = v1.w;
        K = v2.x; ea = v2.y;
    }
    static __device__ __forceinline__ const float *boys(const GradArgs &g) { return g.boys32; }
};
template <> struct GradPrim<df64> {
    static __device__ __forceinline__ void get(const GradArgs &g, int i, df64 &p, df64 &ohp, df64 *P, df64 *PA,
                                               df64 &K, df64 &ea) {
        const float4 *q = reinterpret_cast<const float4 *>(g.primsdf + i);
        const float4 v0 = __ldg(q), v1 = __ldg(q + 1), v2 = __ldg(q + 2), v3 = __ldg(q + 3), v4 = __ldg(q + 4);
        p = df64(v0.x, v0.y); ohp = df64(v0.z, v0.w);
        P[0] = df64(v1.x, v1.y); P[1] = df64(v1.z, v1.w); P[2] = df64(v2.x, v2.y);
        PA[0] = df64(v2.z, v2.w); PA[1] = df64(v3.x, v3.y); PA[2] = df64(v3.z, v3.w);
        K = df64(v4.x, v4.y); ea = df64(v4.z, v4.w);
    }
    static __device__ __forceinline__ const df64 *boys(const GradArgs &g) {
        return reinterpret_cast<const df64 *>(g.boysdf);
    }
};

__device__ __forceinline__ float gt_narrow(double x, float *) { return (float)x; }
__device__ __forceinline__ double gt_narrow(double x, double *) { return x; }
__device__ __forceinline__ df64 gt_narrow(double x, df64 *) { return df64(x); }

// Z_{tuv} = sum_{t'u'v'} (-1)^{t'+u'+v'} E^{cd}_{t'u'v'} R_{t+t',u+u',v+v'} for every bra
// Hermite index with t+u+v <= bmax (stored compactly in md_tuv order): the ket of one component
// contracted with the Coulomb integrals once, reused by every bra component.  The sum is
// nested one direction at a time (one FMA per term instead of a product and an FMA).
template <typename T, int NJ = GR_NI, int NT = GR_NT>
__device__ __forceinline__ void gr_zvec(const T (*Ek)[GR_NI][NJ][NT], const int *c, const int *d, const T *R,
                                        int bmax, T *Z) {
    const T *ex = Ek[0][c[0]][d[0]], *ey = Ek[1][c[1]][d[1]], *ez = Ek[2][c[2]][d[2]];
    const int nx = c[0] + d[0], ny = c[1] + d[1], nz = c[2] + d[2];
    for (int t = 0; t <= bmax; ++t)
        for (int u = 0; u <= bmax - t; ++u)
            for (int v = 0; v <= bmax - t - u; ++v) {
                T z = T(0);
                for (int tt = 0; tt <= nx; ++tt) {
                    T zy = T(0);
                    for (int uu = 0; uu <= ny; ++uu) {
                        T zz = T(0);
                        for (int vv = 0; vv <= nz; ++vv) zz = rchem_fma(ez[vv], R[md_tuv(t + tt, u + uu, v + vv)], zz);
                        zy = rchem_fma(ey[uu], zz, zy);
                    }
                    z = rchem_fma(ex[tt], zy, z);
                }
                Z[md_tuv(t, u, v)] = z;  // compact (t,u,v) order: only t+u+v <= bmax is stored
            }
}

#define GR_ZN 56  // (t,u,v) with t+u+v <= la+lb+1 <= 5
#define GR_ZB 35  // (t,u,v) with t+u+v <= la+lb <= 4
// the per-lane kernel's classes: total L + 1 <= 7 (the two largest classes run
// the warp-cooperative kernel), so its R table holds t+u+v <= 7
#define GR_RT_MAXL1 7
#define GR_RT_NR 120
// ... and its ket pairs have l_d <= 1: ket Hermite tables [i <= 3][j <= 1][t <= 4]
#define GR_RT_NJ 2
#define GR_RT_NTK 5

#define GR_MAXC4 1296  // components of a (dd|dd) quartet

// The smaller classes with a d shell (run-time angular momenta; the larger
// ones run k_grad2e_wc below).  One warp task: up to 32 >> lg unique shell
// quartets, G = 2^lg lanes each (the segment/task layout of the Fock build).  The G lanes split (primitive quartet, ket component
// pair) units; Gamma (degeneracy and component norms folded in) is formed once
// per quartet in FP64 and rounded to R; the 9 centre derivatives are reduced
// over the G lanes with warp shuffles and added to the gradient by one lane.
template <typename R>
__global__ void __launch_bounds__(64) k_grad2e_rt(GradArgs g) {
    const int lane = threadIdx.x & 31;
    const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (w >= g.ntasks) return;  // warp-uniform
    const EriTask tk = g.tasks[w];
    const int lgG = (tk.nq_lg >> 8) & 7, nqt = tk.nq_lg & 255;
    const int G = 1 << lgG, r = lane & (G - 1), qi = lane >> lgG;
    const bool active = qi < nqt;
    int sg = tk.seg, off = tk.off + (active ? qi : 0);
    EriSeg seg = g.segs[sg];
    while (off >= seg.count) {
        off -= seg.count;
        seg = g.segs[++sg];
    }
    const ShellPair bp = g.pairs[seg.bra], kp = g.pairs[seg.ket0 + off];
    const bool same = seg.bra == seg.ket0 + off;
    const int la = g.shell_l[bp.A], lb = g.shell_l[bp.B], lc = g.shell_l[kp.A], ld = g.shell_l[kp.B];
    const int na = (la + 1) * (la + 2) / 2, nb = (lb + 1) * (lb + 2) / 2, nc = (lc + 1) * (lc + 2) / 2,
              nd = (ld + 1) * (ld + 2) / 2;
    const int n = bp.mn;  // the quartet's geometry block of the packed D
    const double *Dg = g.D + bp.moff;
    double deg = 8.0;
    if (bp.diag) deg *= 0.5;
    if (kp.diag) deg *= 0.5;
    if (same) deg *= 0.5;
    // Cartesian components and Gamma, once per quartet
    int cA[6][3], cB[6][3], cC[6][3], cD[6][3];
    double nA[6], nB[6], nC[6], nD[6];
    for (int k = 0; k < na; ++k) {
        gr_comp(la, k, cA[k]);
        nA[k] = gr_cnorm(cA[k]);
    }
    for (int k = 0; k < nb; ++k) {
        gr_comp(lb, k, cB[k]);
        nB[k] = gr_cnorm(cB[k]);
    }
    for (int k = 0; k < nc; ++k) {
        gr_comp(lc, k, cC[k]);
        nC[k] = gr_cnorm(cC[k]);
    }
    for (int k = 0; k < nd; ++k) {
        gr_comp(ld, k, cD[k]);
        nD[k] = gr_cnorm(cD[k]);
    }
    // FP64: Gamma is formed where it is used (five density loads and a few FMAs
    // per bra pair, against a 10 KB local array per thread); the narrower
    // forms keep the array, formed once in FP64 and rounded.
    constexpr bool kGamArray = !std::is_same<R, double>::value;
    R Gam[kGamArray ? GR_MAXC4 : 1];
    if constexpr (kGamArray)
    for (int kc = 0; kc < nc; ++kc)
        for (int kd = 0; kd < nd; ++kd) {
            const int l_ = kp.aoA + kc, s_ = kp.aoB + kd;
            for (int ka = 0; ka < na; ++ka)
                for (int kb = 0; kb < nb; ++kb) {
                    const int mu = bp.aoA + ka, nu = bp.aoB + kb;
                    Gam[((kc * nd + kd) * na + ka) * nb + kb] = gt_narrow(
                        deg * nA[ka] * nB[kb] * nC[kc] * nD[kd] *
                            (2.0 * Dg[mu * n + nu] * Dg[l_ * n + s_] -
                             0.5 * (Dg[mu * n + l_] * Dg[nu * n + s_] + Dg[mu * n + s_] * Dg[nu * n + l_])),
                        (R *)nullptr);
                }
        }
    R AB[3], CD[3];
    Tabs<R>::ab(bp, AB);
    Tabs<R>::ab(kp, CD);
    const R *btab = GradPrim<R>::boys(g);
    R gA[3] = {R(0), R(0), R(0)}, gB[3] = {R(0), R(0), R(0)}, gC[3] = {R(0), R(0), R(0)};
    const int L1 = la + lb + lc + ld + 1;
    R Eb[3][GR_NI][GR_NI][GR_NT], Ek[3][GR_NI][GR_RT_NJ][GR_RT_NTK], Rt[GR_RT_NR], F[GR_RT_MAXL1 + 1];
    R Z0[GR_ZN], Zp[3][GR_ZB], Zm[3][GR_ZB], H0[GR_ZB];
    // work units: (primitive quartet, ket component pair); the G lanes split them
    // (a d-shell quartet's few primitive quartets alone would leave lanes idle)
    const int nk = kp.npp, ntot = bp.npp * nk, ncd = nc * nd;
    const int nunits = active ? ntot * ncd : 0;  // idle lanes only join the reduction
    int cur = -1;
    R a2 = R(0), b2 = R(0), c2 = R(0);
    // each lane a contiguous run of units, so consecutive units mostly share a
    // primitive quartet and its tables are built once per run, not per unit
    const int per = (nunits + G - 1) / G, u0 = r * per, u1 = min(nunits, u0 + per);
    for (int u = u0; u < u1; ++u) {
        const int tq = u / ncd, kcd = u - tq * ncd;
        if (tq != cur) {  // primitive-quartet tables, kept while the lane stays on it
            cur = tq;
            const int ia = tq / nk, ic = tq - ia * nk;
            R p, ohp, Pc[3], PA[3], Kab, aa, q, ohq, Qc[3], QC[3], Kcd, ac;
            GradPrim<R>::get(g, bp.prim0 + ia, p, ohp, Pc, PA, Kab, aa);
            GradPrim<R>::get(g, kp.prim0 + ic, q, ohq, Qc, QC, Kcd, ac);
            a2 = aa + aa;
            b2 = (p - aa) + (p - aa);
            c2 = ac + ac;
            R rs, ipq, rho, qi, pi;
            pq_factors<R>(g, bp.prim0 + ia, kp.prim0 + ic, p, q, rs, ipq, rho, qi, pi);
            const R X = Pc[0] - Qc[0], Y = Pc[1] - Qc[1], Zc = Pc[2] - Qc[2];
            const R T = rho * (X * X + Y * Y + Zc * Zc);
            boys_eval_rt<R>(L1, T, Kab * Kcd * rs, btab, F);
            gr_R<R, GR_RT_NR>(L1, rho, X, Y, Zc, F, Rt);
            for (int dd = 0; dd < 3; ++dd) {
                gr_herm<R>(la + 1, lb + 1, PA[dd], AB[dd], ohp, Eb[dd]);
                gr_herm<R, GR_RT_NJ, GR_RT_NTK>(lc + 1, ld, QC[dd], CD[dd], ohq, Ek[dd]);
                for (int i = 0; i <= lc + 1; ++i)  // ket sign (-1)^t folded in
                    for (int j = 0; j <= ld; ++j)
                        for (int t = 1; t < GR_RT_NTK; t += 2) Ek[dd][i][j][t] = -Ek[dd][i][j][t];
            }
        }
        const int kc = kcd / nd, kd = kcd - kc * nd;
        const R *Gq = Gam + (kGamArray ? (kc * nd + kd) * na * nb : 0);
        const int *Cc = cC[kc];
        const int l_ = kp.aoA + kc, s_ = kp.aoB + kd;
        const double Dls = Dg[l_ * n + s_], wcd = deg * nC[kc] * nD[kd];
        // ket contracted with R: unshifted (the bra may be shifted by one) and C-shifted
        gr_zvec<R, GR_RT_NJ, GR_RT_NTK>(Ek, Cc, cD[kd], Rt, la + lb + 1, Z0);
        for (int x = 0; x < 3; ++x) {
            int s[3] = {Cc[0], Cc[1], Cc[2]};
            s[x] += 1;
            gr_zvec<R, GR_RT_NJ, GR_RT_NTK>(Ek, s, cD[kd], Rt, la + lb, Zp[x]);
            if (Cc[x] > 0) {
                s[x] -= 2;
                gr_zvec<R, GR_RT_NJ, GR_RT_NTK>(Ek, s, cD[kd], Rt, la + lb, Zm[x]);
            }
        }
        // centre C through the bra Hermite density H0_tuv = sum_ab Gamma_ab E^{ab}_tuv
        const int hb = la + lb, nh = (hb + 1) * (hb + 2) * (hb + 3) / 6;
        for (int i = 0; i < nh; ++i) H0[i] = R(0);
        for (int ka = 0; ka < na; ++ka) {
            const int *A = cA[ka];
            for (int kb = 0; kb < nb; ++kb) {
                R Gm;
                if constexpr (kGamArray) {
                    Gm = Gq[ka * nb + kb];
                } else {
                    const int mu = bp.aoA + ka, nu = bp.aoB + kb;
                    Gm = wcd * nA[ka] * nB[kb] *
                         (2.0 * Dg[mu * n + nu] * Dls -
                          0.5 * (Dg[mu * n + l_] * Dg[nu * n + s_] + Dg[mu * n + s_] * Dg[nu * n + l_]));
                }
                const int *B = cB[kb];
                const R *ex = Eb[0][A[0]][B[0]], *ey = Eb[1][A[1]][B[1]], *ez = Eb[2][A[2]][B[2]];
                const int mx = A[0] + B[0], my = A[1] + B[1], mz = A[2] + B[2];
                for (int t = 0; t <= mx; ++t) {
                    const R gx = Gm * ex[t];
                    for (int u = 0; u <= my; ++u) {
                        const R gy = gx * ey[u];
                        for (int v = 0; v <= mz; ++v) H0[md_tuv(t, u, v)] = rchem_fma(gy, ez[v], H0[md_tuv(t, u, v)]);
                    }
                }
                // centres A and B along x, y, z: the derivative shifts one direction's E by one, so
                // the sums over the two other directions are formed once and shared (S_x, S_y, S_z)
                R P[GR_NT][GR_NT], Sx[GR_NT], Sy[GR_NT], Sz[GR_NT];
                for (int t = 0; t <= mx + 1; ++t)
                    for (int u = 0; u <= my + (t <= mx ? 1 : 0); ++u) {
                        R acc = R(0);
                        for (int v = 0; v <= mz; ++v) acc = rchem_fma(ez[v], Z0[md_tuv(t, u, v)], acc);
                        P[t][u] = acc;
                    }
                for (int t = 0; t <= mx + 1; ++t) {
                    R acc = R(0);
                    for (int u = 0; u <= my; ++u) acc = rchem_fma(ey[u], P[t][u], acc);
                    Sx[t] = acc;
                }
                for (int u = 0; u <= my + 1; ++u) {
                    R acc = R(0);
                    for (int t = 0; t <= mx; ++t) acc = rchem_fma(ex[t], P[t][u], acc);
                    Sy[u] = acc;
                }
                for (int v = 0; v <= mz + 1; ++v) {
                    R acc = R(0);
                    for (int t = 0; t <= mx; ++t) {
                        R m = R(0);
                        for (int u = 0; u <= my; ++u) m = rchem_fma(ey[u], Z0[md_tuv(t, u, v)], m);
                        acc = rchem_fma(ex[t], m, acc);
                    }
                    Sz[v] = acc;
                }
                const R *Sd[3] = {Sx, Sy, Sz};
                for (int x = 0; x < 3; ++x) {
                    const R *S = Sd[x];
                    const int ax = A[x], bx = B[x], m = ax + bx;
                    // 2 alpha (a+1|..) - a_x (a-1|..)
                    const R *ep = Eb[x][ax + 1][bx];
                    R v = R(0);
                    for (int t = 0; t <= m + 1; ++t) v = rchem_fma(ep[t], S[t], v);
                    v = a2 * v;
                    if (ax > 0) {
                        const R *em = Eb[x][ax - 1][bx];
                        R w = R(0);
                        for (int t = 0; t <= m - 1; ++t) w = rchem_fma(em[t], S[t], w);
                        v = v - R(ax) * w;
                    }
                    gA[x] = rchem_fma(Gm, v, gA[x]);
                    // 2 beta (..b+1|..) - b_x (..b-1|..)
                    const R *fp = Eb[x][ax][bx + 1];
                    v = R(0);
                    for (int t = 0; t <= m + 1; ++t) v = rchem_fma(fp[t], S[t], v);
                    v = b2 * v;
                    if (bx > 0) {
                        const R *fm = Eb[x][ax][bx - 1];
                        R w = R(0);
                        for (int t = 0; t <= m - 1; ++t) w = rchem_fma(fm[t], S[t], w);
                        v = v - R(bx) * w;
                    }
                    gB[x] = rchem_fma(Gm, v, gB[x]);
                }
            }
        }
        for (int x = 0; x < 3; ++x) {
            R vp = R(0), vm = R(0);
            for (int i = 0; i < nh; ++i) vp = rchem_fma(H0[i], Zp[x][i], vp);
            if (Cc[x] > 0)
                for (int i = 0; i < nh; ++i) vm = rchem_fma(H0[i], Zm[x][i], vm);
            gC[x] = gC[x] + c2 * vp - R(Cc[x]) * vm;
        }
    }
    for (int o = G >> 1; o > 0; o >>= 1)
        for (int x = 0; x < 3; ++x) {
            gA[x] += __shfl_xor_sync(0xffffffffu, gA[x], o);
            gB[x] += __shfl_xor_sync(0xffffffffu, gB[x], o);
            gC[x] += __shfl_xor_sync(0xffffffffu, gC[x], o);
        }
    if (!active || r != 0) return;
    const int atA = g.shell_atom[bp.A], atB = g.shell_atom[bp.B], atC = g.shell_atom[kp.A],
              atD = g.shell_atom[kp.B];
    for (int x = 0; x < 3; ++x) {
        const double a = widen(gA[x]), b = widen(gB[x]), c = widen(gC[x]);
        atomicAdd(g.grad + 3 * atA + x, a);
        atomicAdd(g.grad + 3 * atB + x, b);
        atomicAdd(g.grad + 3 * atC + x, c);
        atomicAdd(g.grad + 3 * atD + x, -(a + b + c));
    }
}

// ---------------------------------------------------------------------------
// The larger classes with a d shell (run-time angular momenta): one contracted
// quartet per warp.
// Per primitive quartet the warp builds the Hermite tables (E of bra and ket,
// the Coulomb table R) once in shared memory; per chunk of ket component
// pairs it builds the ket vectors Z0 = sum E^{cd} R (for the centre-A/B
// derivatives) and W_x = 2 gamma Z(c+1_x) - c_x Z(c-1_x) (centre C) in shared
// memory; then every lane takes (ket pair, bra pair) items: Gamma in place,
// the A/B derivatives through the x/y/z partial sums of E^{ab} against Z0, the
// C derivative as E^{ab} . W_x.  Per-lane state is a few scalars, so nothing
// spills; the tables are formed once per warp instead of once per lane.
#define GW_WARPS 2      // warps per block
#define GW_CHUNK 12     // ket component pairs whose vectors are held at once
#define GW_ZSLOT 161    // Z0 (t+u+v <= 5: 56) + three W_x (t+u+v <= 4: 35 each)
#define GW_ETAB (3 * GR_NI * GR_NI * GR_NT)
#define GW_PER_WARP (2 * GW_ETAB + 2 * GR_NR + GW_CHUNK * GW_ZSLOT)

__device__ __forceinline__ int gr_cnt(int N) { return (N + 1) * (N + 2) * (N + 3) / 6; }
// (t,u,v) of compact Hermite index i (the inverse of md_tuv)
__device__ __forceinline__ void gr_decode(int i, int &t, int &u, int &v) {
    int n = 0;
    while (gr_cnt(n) <= i) ++n;
    const int r = i - (n >= 1 ? gr_cnt(n - 1) : 0);
    int s = 0;
    while ((s + 1) * (s + 2) / 2 <= r) ++s;
    v = r - s * (s + 1) / 2;
    u = s - v;
    t = n - s;
}
// sum_{t'u'v'} E^{cd}_{t'u'v'} R_{t+t',u+u',v+v'} (ket signs folded into E)
template <typename R>
__device__ __forceinline__ R gr_zsum(const R (*Ek)[GR_NI][GR_NI][GR_NT], const int *c, const int *d, const R *Rt,
                                     int t, int u, int v) {
    const R *ex = Ek[0][c[0]][d[0]], *ey = Ek[1][c[1]][d[1]], *ez = Ek[2][c[2]][d[2]];
    R z = R(0);
    for (int tt = 0; tt <= c[0] + d[0]; ++tt) {
        R zy = R(0);
        for (int uu = 0; uu <= c[1] + d[1]; ++uu) {
            R zz = R(0);
            for (int vv = 0; vv <= c[2] + d[2]; ++vv) zz = rchem_fma(ez[vv], Rt[md_tuv(t + tt, u + uu, v + vv)], zz);
            zy = rchem_fma(ey[uu], zz, zy);
        }
        z = rchem_fma(ex[tt], zy, z);
    }
    return z;
}

template <typename R>
__global__ void __launch_bounds__(32 * GW_WARPS) k_grad2e_wc(GradArgs g) {
    extern __shared__ __align__(16) unsigned char gw_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    R *base = reinterpret_cast<R *>(gw_smem) + (size_t)wib * GW_PER_WARP;
    R(*Eb)[GR_NI][GR_NI][GR_NT] = reinterpret_cast<R(*)[GR_NI][GR_NI][GR_NT]>(base);
    R(*Ek)[GR_NI][GR_NI][GR_NT] = reinterpret_cast<R(*)[GR_NI][GR_NI][GR_NT]>(base + GW_ETAB);
    R *Ra = base + 2 * GW_ETAB, *Rb = Ra + GR_NR, *Zc = Rb + GR_NR;
    const int w = blockIdx.x * GW_WARPS + wib;
    if (w >= g.ntasks) return;  // warp-uniform; the kernel has no block-wide barrier
    const EriTask tk = g.tasks[w];
    int sg = tk.seg, off = tk.off;
    EriSeg seg = g.segs[sg];
    while (off >= seg.count) {
        off -= seg.count;
        seg = g.segs[++sg];
    }
    const ShellPair bp = g.pairs[seg.bra], kp = g.pairs[seg.ket0 + off];
    const bool same = seg.bra == seg.ket0 + off;
    const int la = g.shell_l[bp.A], lb = g.shell_l[bp.B], lc = g.shell_l[kp.A], ld = g.shell_l[kp.B];
    const int na = (la + 1) * (la + 2) / 2, nb = (lb + 1) * (lb + 2) / 2, nc = (lc + 1) * (lc + 2) / 2,
              nd = (ld + 1) * (ld + 2) / 2;
    const int n = bp.mn;
    const double *Dg = g.D + bp.moff;
    double deg = 8.0;
    if (bp.diag) deg *= 0.5;
    if (kp.diag) deg *= 0.5;
    if (same) deg *= 0.5;
    R AB[3], CD[3];
    Tabs<R>::ab(bp, AB);
    Tabs<R>::ab(kp, CD);
    const R *btab = GradPrim<R>::boys(g);
    const int L1 = la + lb + lc + ld + 1;
    const int nab = na * nb, ncd = nc * nd;
    const int nz0 = gr_cnt(la + lb + 1), nzb = gr_cnt(la + lb), zs = nz0 + 3 * nzb;
    R gA[3] = {R(0), R(0), R(0)}, gB[3] = {R(0), R(0), R(0)}, gC[3] = {R(0), R(0), R(0)};
    const int nk = kp.npp, ntot = bp.npp * nk;
    for (int tq = 0; tq < ntot; ++tq) {
        const int ia = tq / nk, ic = tq - ia * nk;
        R p, ohp, Pc[3], PA[3], Kab, aa, q, ohq, Qc[3], QC[3], Kcd, ac;
        GradPrim<R>::get(g, bp.prim0 + ia, p, ohp, Pc, PA, Kab, aa);
        GradPrim<R>::get(g, kp.prim0 + ic, q, ohq, Qc, QC, Kcd, ac);
        const R a2 = aa + aa, b2 = (p - aa) + (p - aa), c2 = ac + ac;
        R rs, ipq, rho, qi, pi;
        pq_factors<R>(g, bp.prim0 + ia, kp.prim0 + ic, p, q, rs, ipq, rho, qi, pi);
        const R X = Pc[0] - Qc[0], Y = Pc[1] - Qc[1], Zq = Pc[2] - Qc[2];
        R F[GR_LMAX + 1];
        boys_eval_rt<R>(L1, rho * (X * X + Y * Y + Zq * Zq), Kab * Kcd * rs, btab, F);
        __syncwarp();  // the previous primitive quartet's tables have been read
        // Hermite E tables: lanes 0-2 the bra directions, 3-5 the ket (ket signs folded in)
        if (lane < 3) {
            gr_herm<R>(la + 1, lb + 1, PA[lane], AB[lane], ohp, Eb[lane]);
        } else if (lane < 6) {
            const int dd = lane - 3;
            gr_herm<R>(lc + 1, ld, QC[dd], CD[dd], ohq, Ek[dd]);
            for (int i = 0; i <= lc + 1; ++i)
                for (int j = 0; j <= ld; ++j)
                    for (int t = 1; t < GR_NT; t += 2) Ek[dd][i][j][t] = -Ek[dd][i][j][t];
        }
        // Coulomb table R_tuv (t+u+v <= L1), level by level of the recursion, the
        // entries of a level over the lanes
        const R m2a = R(-2) * rho;
        R *cur = Ra, *nxt = Rb;
        if (lane == 0) {
            R pw = R(1);
            for (int k = 0; k < L1; ++k) pw = pw * m2a;
            cur[0] = pw * F[L1];
        }
        __syncwarp();
        for (int lv = L1 - 1; lv >= 0; --lv) {
            R pw = R(1);
            for (int k = 0; k < lv; ++k) pw = pw * m2a;
            const int cnt = gr_cnt(L1 - lv);
            for (int i = lane; i < cnt; i += 32) {
                int t, u, v;
                gr_decode(i, t, u, v);
                R r;
                if (t + u + v == 0) r = pw * F[lv];
                else if (t > 0) r = rchem_fma(X, cur[md_tuv(t - 1, u, v)], t > 1 ? R(t - 1) * cur[md_tuv(t - 2, u, v)] : R(0));
                else if (u > 0) r = rchem_fma(Y, cur[md_tuv(0, u - 1, v)], u > 1 ? R(u - 1) * cur[md_tuv(0, u - 2, v)] : R(0));
                else r = rchem_fma(Zq, cur[md_tuv(0, 0, v - 1)], v > 1 ? R(v - 1) * cur[md_tuv(0, 0, v - 2)] : R(0));
                nxt[i] = r;
            }
            __syncwarp();
            R *tmp = cur;
            cur = nxt;
            nxt = tmp;
        }
        const R *Rt = cur;
        for (int c0 = 0; c0 < ncd; c0 += GW_CHUNK) {
            const int nch = min(GW_CHUNK, ncd - c0);
            // ket vectors of the chunk: slot k holds Z0 (nz0 values) then W_x (nzb each)
            for (int e = lane; e < nch * zs; e += 32) {
                const int k = e / zs, j = e - k * zs;
                const int kcd = c0 + k, kc = kcd / nd, kd = kcd - kc * nd;
                int cc[3], dd[3];
                gr_comp(lc, kc, cc);
                gr_comp(ld, kd, dd);
                int t, u, v;
                R val;
                if (j < nz0) {
                    gr_decode(j, t, u, v);
                    val = gr_zsum<R>(Ek, cc, dd, Rt, t, u, v);
                } else {
                    const int jj = j - nz0, x = jj / nzb;
                    gr_decode(jj - x * nzb, t, u, v);
                    int s[3] = {cc[0], cc[1], cc[2]};
                    s[x] += 1;
                    val = c2 * gr_zsum<R>(Ek, s, dd, Rt, t, u, v);
                    if (cc[x] > 0) {
                        s[x] -= 2;
                        val = val - R(cc[x]) * gr_zsum<R>(Ek, s, dd, Rt, t, u, v);
                    }
                }
                Zc[e] = val;
            }
            __syncwarp();
            for (int it = lane; it < nch * nab; it += 32) {
                const int k = it / nab, ab = it - k * nab;
                const int kcd = c0 + k, kc = kcd / nd, kd = kcd - kc * nd;
                const int ka = ab / nb, kb = ab - ka * nb;
                int A[3], B[3], Cc[3], Dd[3];
                gr_comp(la, ka, A);
                gr_comp(lb, kb, B);
                gr_comp(lc, kc, Cc);
                gr_comp(ld, kd, Dd);
                // Gamma (degeneracy and component norms folded in), in FP64
                const int mu = bp.aoA + ka, nu = bp.aoB + kb, l_ = kp.aoA + kc, s_ = kp.aoB + kd;
                const double gam = deg * gr_cnorm(A) * gr_cnorm(B) * gr_cnorm(Cc) * gr_cnorm(Dd) *
                                   (2.0 * Dg[mu * n + nu] * Dg[l_ * n + s_] -
                                    0.5 * (Dg[mu * n + l_] * Dg[nu * n + s_] + Dg[mu * n + s_] * Dg[nu * n + l_]));
                const R Gm = gt_narrow(gam, (R *)nullptr);
                const R *Z0 = Zc + k * zs, *W = Z0 + nz0;
                const R *ex = Eb[0][A[0]][B[0]], *ey = Eb[1][A[1]][B[1]], *ez = Eb[2][A[2]][B[2]];
                const int mx = A[0] + B[0], my = A[1] + B[1], mz = A[2] + B[2];
                // centres A and B: for each direction the sum over the two others is
                // formed for every index of this one and dotted with four E vectors
                for (int x = 0; x < 3; ++x) {
                    const int ax = A[x], bx = B[x], m = ax + bx;
                    const R *ep = Eb[x][ax + 1][bx], *fp = Eb[x][ax][bx + 1];
                    const R *em = ax > 0 ? Eb[x][ax - 1][bx] : ep, *fm = bx > 0 ? Eb[x][ax][bx - 1] : fp;
                    R dap = R(0), dam = R(0), dbp = R(0), dbm = R(0);
                    for (int i = 0; i <= m + 1; ++i) {
                        R si = R(0);
                        if (x == 0) {
                            for (int u = 0; u <= my; ++u) {
                                R sv = R(0);
                                for (int v = 0; v <= mz; ++v) sv = rchem_fma(ez[v], Z0[md_tuv(i, u, v)], sv);
                                si = rchem_fma(ey[u], sv, si);
                            }
                        } else if (x == 1) {
                            for (int t = 0; t <= mx; ++t) {
                                R sv = R(0);
                                for (int v = 0; v <= mz; ++v) sv = rchem_fma(ez[v], Z0[md_tuv(t, i, v)], sv);
                                si = rchem_fma(ex[t], sv, si);
                            }
                        } else {
                            for (int t = 0; t <= mx; ++t) {
                                R su = R(0);
                                for (int u = 0; u <= my; ++u) su = rchem_fma(ey[u], Z0[md_tuv(t, u, i)], su);
                                si = rchem_fma(ex[t], su, si);
                            }
                        }
                        dap = rchem_fma(ep[i], si, dap);
                        dbp = rchem_fma(fp[i], si, dbp);
                        if (i < m) {
                            dam = rchem_fma(em[i], si, dam);
                            dbm = rchem_fma(fm[i], si, dbm);
                        }
                    }
                    R va = a2 * dap, vb = b2 * dbp;
                    if (ax > 0) va = va - R(ax) * dam;
                    if (bx > 0) vb = vb - R(bx) * dbm;
                    gA[x] = rchem_fma(Gm, va, gA[x]);
                    gB[x] = rchem_fma(Gm, vb, gB[x]);
                }
                // centre C: E^{ab} . W_x
                for (int x = 0; x < 3; ++x) {
                    const R *Wx = W + x * nzb;
                    R sc = R(0);
                    for (int t = 0; t <= mx; ++t) {
                        R su = R(0);
                        for (int u = 0; u <= my; ++u) {
                            R sv = R(0);
                            for (int v = 0; v <= mz; ++v) sv = rchem_fma(ez[v], Wx[md_tuv(t, u, v)], sv);
                            su = rchem_fma(ey[u], sv, su);
                        }
                        sc = rchem_fma(ex[t], su, sc);
                    }
                    gC[x] = rchem_fma(Gm, sc, gC[x]);
                }
            }
            __syncwarp();  // the chunk's vectors have been read
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int x = 0; x < 3; ++x) {
            gA[x] += __shfl_xor_sync(0xffffffffu, gA[x], o);
            gB[x] += __shfl_xor_sync(0xffffffffu, gB[x], o);
            gC[x] += __shfl_xor_sync(0xffffffffu, gC[x], o);
        }
    if (lane != 0) return;
    const int atA = g.shell_atom[bp.A], atB = g.shell_atom[bp.B], atC = g.shell_atom[kp.A], atD = g.shell_atom[kp.B];
    for (int x = 0; x < 3; ++x) {
        const double a = widen(gA[x]), b = widen(gB[x]), c = widen(gC[x]);
        atomicAdd(g.grad + 3 * atA + x, a);
        atomicAdd(g.grad + 3 * atB + x, b);
        atomicAdd(g.grad + 3 * atC + x, c);
        atomicAdd(g.grad + 3 * atD + x, -(a + b + c));
    }
}

// One-electron part, one thread per ordered function pair (mu, nu) of a geometry:
//   4 D_mn d_mu H_mn - 4 W_mn d_mu S_mn on the atom of mu,
//   and the Hellmann-Feynman term -4 D_mn Z_C d_mu V_mn(C) on each nucleus C
// (d_mu = derivative with respect to the centre of mu; 2-centre translational
// invariance gives the centre of nu, 3-centre invariance the nucleus).
struct AOGrad {
    int shell, lmn[3];
    double cn;
};
struct ShellGrad {
    double R[3];
    int l, nprim, prim0, atom;
};

__device__ __forceinline__ int geom_of(const GeomDev *geo, int ngeom, long long idx) {
    int lo = 0, hi = ngeom - 1;  // last geometry whose block starts at or before idx
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (geo[mid].moff <= idx) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// sum_{tuv} E_x[a_x][b_x][t] E_y[..][u] E_z[..][v] R_{tuv} (R in md_tuv order)
__device__ __forceinline__ double gr_dot_r(const double (*E)[GR_NI][GR_NI][GR_NT], const int *a, const int *b,
                                           const double *R) {
    double s = 0.0;
    for (int t = 0; t <= a[0] + b[0]; ++t) {
        const double ex = E[0][a[0]][b[0]][t];
        for (int u = 0; u <= a[1] + b[1]; ++u) {
            const double ey = ex * E[1][a[1]][b[1]][u];
            for (int v = 0; v <= a[2] + b[2]; ++v) s += ey * E[2][a[2]][b[2]][v] * R[md_tuv(t, u, v)];
        }
    }
    return s;
}

#define GR1_NUCCHUNK 2  // nuclei per thread of k_grad1e (grid y runs over the chunks)

// 1-D overlap factors S[i][j] = int x_A^i x_B^j exp(-p x_P^2) dx (Obara--Saika),
// i <= imax, j <= jmax
__device__ __forceinline__ void gr_s1d(int imax, int jmax, double PA, double PB, double ohp, double p,
                                       double (*S)[5]) {
    S[0][0] = sqrt(3.14159265358979323846 / p);
    for (int i = 0; i <= imax; ++i) {
        if (i > 0) S[i][0] = PA * S[i - 1][0] + (i > 1 ? ohp * (i - 1) * S[i - 2][0] : 0.0);
        for (int j = 1; j <= jmax; ++j)
            S[i][j] = PB * S[i][j - 1] + ohp * ((i > 0 ? i * S[i - 1][j - 1] : 0.0) + (j > 1 ? (j - 1) * S[i][j - 2] : 0.0));
    }
}

// 1-D kinetic factor of x_A^i x_B^j: b(2j+1) S_ij - 2b^2 S_i,j+2 - j(j-1)/2 S_i,j-2
__device__ __forceinline__ double gr_t1d(int i, int j, double b, const double (*S)[5]) {
    double t = b * (2 * j + 1) * S[i][j] - 2.0 * b * b * S[i][j + 2];
    if (j >= 2) t -= 0.5 * j * (j - 1) * S[i][j - 2];
    return t;
}

#ifndef RCHEM_GRAD_NO_KERNELS
// One thread per ordered function pair (mu, nu) of a geometry and chunk of
// GR1_NUCCHUNK nuclei (grid y), so a small system still fills the GPU.  Per
// primitive pair the Gaussian product and the Hermite tables are formed once
// (and, in chunk 0, the 1-D overlap table shared by S, T and every shifted
// component); per nucleus one Boys evaluation and one Hermite Coulomb table
// serve both shifts in all three directions.  The chunk's nuclei's terms are
// summed over the primitive pairs before any atomic.
__global__ void k_grad1e(long long packed, int ngeom, const GeomDev *geo, const AOGrad *ao, const ShellGrad *sh,
                         const double *pexp, const double *pcoef, int natoms_total, const double *Z,
                         const double *Ratoms, const double *boys, const double *D, const double *W, double *grad) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= packed) return;
    const GeomDev gm = geo[geom_of(geo, ngeom, idx)];
    // this thread's nuclei: chunk blockIdx.y; chunk 0 also takes the overlap and kinetic terms
    const int c0 = blockIdx.y * GR1_NUCCHUNK, c1 = min(gm.natoms, c0 + GR1_NUCCHUNK);
    const bool first = blockIdx.y == 0;
    if (!first && c0 >= gm.natoms) return;
    const int loc = (int)(idx - gm.moff), mu = gm.ao0 + loc / gm.n, nu = gm.ao0 + loc % gm.n;
    const double Dmn = D[idx], Wmn = W[idx];
    if (Dmn == 0.0 && Wmn == 0.0) return;
    const AOGrad a = ao[mu], b = ao[nu];
    const ShellGrad sa = sh[a.shell], sb = sh[b.shell];
    double gH[3] = {0, 0, 0}, gS[3] = {0, 0, 0};
    double gN[GR1_NUCCHUNK][3];
    for (int c = 0; c < GR1_NUCCHUNK; ++c) gN[c][0] = gN[c][1] = gN[c][2] = 0.0;
    const int L1 = a.lmn[0] + a.lmn[1] + a.lmn[2] + b.lmn[0] + b.lmn[1] + b.lmn[2] + 1;
    double AB[3], rab2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        AB[d] = sa.R[d] - sb.R[d];
        rab2 += AB[d] * AB[d];
    }
    for (int j = 0; j < sb.nprim; ++j) {
        const double eb = pexp[sb.prim0 + j], cb = pcoef[sb.prim0 + j];
        for (int i = 0; i < sa.nprim; ++i) {
            const double ea = pexp[sa.prim0 + i], cc = pcoef[sa.prim0 + i] * cb * a.cn * b.cn;
            const double p = ea + eb, ohp = 0.5 / p;
            const double Kab = cc * exp(-ea * eb * rab2 / p);
            double P[3], PA[3];
            double S1[3][4][5], E[3][GR_NI][GR_NI][GR_NT];
            for (int d = 0; d < 3; ++d) {
                P[d] = (ea * sa.R[d] + eb * sb.R[d]) / p;
                PA[d] = P[d] - sa.R[d];
                gr_herm<double>(a.lmn[d] + 1, b.lmn[d], PA[d], AB[d], ohp, E[d]);
            }
            if (first) {
            for (int d = 0; d < 3; ++d) gr_s1d(a.lmn[d] + 1, b.lmn[d] + 2, PA[d], P[d] - sb.R[d], ohp, p, S1[d]);
            // overlap and kinetic of the unshifted and shifted components
            double s0[3], t0[3];
            for (int d = 0; d < 3; ++d) {
                s0[d] = S1[d][a.lmn[d]][b.lmn[d]];
                t0[d] = gr_t1d(a.lmn[d], b.lmn[d], eb, S1[d]);
            }
            for (int x = 0; x < 3; ++x) {
                const int y = (x + 1) % 3, z = (x + 2) % 3, ax = a.lmn[x], bx = b.lmn[x];
                const double sy = s0[y] * s0[z], ty = t0[y] * s0[z] + s0[y] * t0[z];
                double ds = 2.0 * ea * S1[x][ax + 1][bx];
                double dt = 2.0 * ea * (gr_t1d(ax + 1, bx, eb, S1[x]) * sy + S1[x][ax + 1][bx] * ty);
                if (ax > 0) {
                    ds -= ax * S1[x][ax - 1][bx];
                    dt -= ax * (gr_t1d(ax - 1, bx, eb, S1[x]) * sy + S1[x][ax - 1][bx] * ty);
                }
                gS[x] += Kab * ds * sy;
                gH[x] += Kab * dt;
            }
            }
            // nuclear attraction: one Boys evaluation and R table per nucleus of the chunk
            const double vpref = -2.0 * 3.14159265358979323846 / p * Kab;
            for (int c = c0; c < c1; ++c) {
                const int cn = gm.atom0 + c;
                const double X = P[0] - Ratoms[3 * cn], Y = P[1] - Ratoms[3 * cn + 1], Zc = P[2] - Ratoms[3 * cn + 2];
                double F[GR_LMAX + 1], R[GR_NR];
                boys_eval_rt<double>(L1, p * (X * X + Y * Y + Zc * Zc), 1.0, boys, F);
                gr_R<double>(L1, p, X, Y, Zc, F, R);
                int s[3];
                double v3[3];
                for (int x = 0; x < 3; ++x) {
                    s[0] = a.lmn[0];
                    s[1] = a.lmn[1];
                    s[2] = a.lmn[2];
                    s[x] += 1;
                    double v = 2.0 * ea * gr_dot_r(E, s, b.lmn, R);
                    if (a.lmn[x] > 0) {
                        s[x] -= 2;
                        v -= a.lmn[x] * gr_dot_r(E, s, b.lmn, R);
                    }
                    v3[x] = v * vpref * Z[cn];
                    gH[x] += v3[x];
                }
                for (int x = 0; x < 3; ++x) gN[c - c0][x] += v3[x];
            }
        }
    }
    for (int c = c0; c < c1; ++c)
        for (int x = 0; x < 3; ++x) atomicAdd(grad + 3 * (gm.atom0 + c) + x, -4.0 * Dmn * gN[c - c0][x]);
    for (int x = 0; x < 3; ++x) atomicAdd(grad + 3 * sa.atom + x, 4.0 * Dmn * gH[x] - 4.0 * Wmn * gS[x]);
    (void)natoms_total;
}
#endif
