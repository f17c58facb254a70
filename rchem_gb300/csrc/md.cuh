// md.cuh -- McMurchie--Davidson (Hermite) integrals for arbitrary Cartesian
// powers, host+device.  Used where the angular momenta are only known at run
// time: the cints-style scalar entry points, the Schwarz diagonal (ab|ab), the
// one-electron S/T/V and multipole matrices.  The ERI class kernels of the
// Fock build use the generated HGP code instead.
//
// Definitions follow the reference's integrals (libpyquante2/cints.c:72-269,
// src/integrals/os86.rs:629-828): unnormalised primitives times the caller's
// norms; V carries the minus sign of an attraction to a unit charge.
#pragma once
#include <math.h>
#include "boys.cuh"

#define MD_MAXE 12  // largest l_a + l_b in one Cartesian direction (kinetic raises l_b by 2)
#define MD_MAXL 8   // largest total L of an ERI or nuclear-attraction integral
#define MD_NR 165   // number of (t,u,v) with t+u+v <= MD_MAXL

RCHEM_HD inline double md_binom(int n, int k) {
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

// Hermite expansion coefficients E_t of x_A^la x_B^lb (no exponential factor),
// t = 0..la+lb, by the recursion in i on x_A^i and the binomial transfer
// x_B = x_A + (A-B).
RCHEM_HD inline void md_E(int la, int lb, double PA, double AB, double ohp, double *E) {
    double Ei[MD_MAXE + 1][MD_MAXE + 1];
    const int n = la + lb;
    for (int i = 0; i <= n; ++i)
        for (int t = 0; t <= n; ++t) Ei[i][t] = 0.0;
    Ei[0][0] = 1.0;
    for (int i = 0; i < n; ++i)
        for (int t = 0; t <= i + 1; ++t) {
            double v = 0.0;
            if (t > 0) v += ohp * Ei[i][t - 1];
            if (t <= i) v += PA * Ei[i][t];
            if (t + 1 <= i) v += (t + 1) * Ei[i][t + 1];
            Ei[i + 1][t] = v;
        }
    for (int t = 0; t <= n; ++t) E[t] = 0.0;
    double abpow = 1.0;
    for (int k = lb; k >= 0; --k) {  // C(lb,k) AB^(lb-k) x_A^(la+k)
        const double c = md_binom(lb, k) * abpow;
        for (int t = 0; t <= la + k; ++t) E[t] += c * Ei[la + k][t];
        abpow *= AB;
    }
}

RCHEM_HD inline int md_tuv(int t, int u, int v) {
    const int n = t + u + v, s = u + v;
    return n * (n + 1) * (n + 2) / 6 + s * (s + 1) / 2 + v;
}

// Hermite Coulomb integrals R_{tuv} (level n = 0) for t+u+v <= L:
// R^n_000 = (-2 a)^n F_n(a |PC|^2), R^n_{t+1,u,v} = t R^{n+1}_{t-1,u,v} + X R^{n+1}_{t,u,v}, ...
// F[] holds F_n (n = 0..L) already multiplied by any prefactor.
RCHEM_HD inline void md_R(int L, double a, double X, double Y, double Z, const double *F, double *out) {
    double buf[2][MD_NR];
    double *cur = buf[0], *nxt = buf[1];
    double m2a = -2.0 * a, pw = 1.0;
    for (int n = 0; n < L; ++n) pw *= m2a;
    cur[0] = pw * F[L];
    for (int n = L - 1; n >= 0; --n) {
        pw /= m2a;
        const int top = L - n;
        for (int N = 0; N <= top; ++N)
            for (int t = N; t >= 0; --t)
                for (int u = N - t; u >= 0; --u) {
                    const int v = N - t - u;
                    double r;
                    if (N == 0) {
                        r = pw * F[n];
                    } else if (t > 0) {
                        r = X * cur[md_tuv(t - 1, u, v)];
                        if (t > 1) r += (t - 1) * cur[md_tuv(t - 2, u, v)];
                    } else if (u > 0) {
                        r = Y * cur[md_tuv(0, u - 1, v)];
                        if (u > 1) r += (u - 1) * cur[md_tuv(0, u - 2, v)];
                    } else {
                        r = Z * cur[md_tuv(0, 0, v - 1)];
                        if (v > 1) r += (v - 1) * cur[md_tuv(0, 0, v - 2)];
                    }
                    nxt[md_tuv(t, u, v)] = r;
                }
        double *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    const int cnt = (L + 1) * (L + 2) * (L + 3) / 6;
    for (int i = 0; i < cnt; ++i) out[i] = cur[i];
}

// Primitive ERI (ab|cd) of unnormalised Cartesian Gaussians; la[] etc. are the
// (l,m,n) powers.  boys = FP64 Boys grid table.
RCHEM_HD inline double md_eri_prim(const double *A, const int *la, double aa, const double *B, const int *lb, double ab,
                                   const double *C, const int *lc, double ac, const double *D, const int *ld, double ad,
                                   const double *boys) {
    const double p = aa + ab, q = ac + ad;
    double P[3], Q[3], Ex[3][MD_MAXE + 1], Ey[3][MD_MAXE + 1];
    double rab2 = 0.0, rcd2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        P[d] = (aa * A[d] + ab * B[d]) / p;
        Q[d] = (ac * C[d] + ad * D[d]) / q;
        rab2 += (A[d] - B[d]) * (A[d] - B[d]);
        rcd2 += (C[d] - D[d]) * (C[d] - D[d]);
        md_E(la[d], lb[d], P[d] - A[d], A[d] - B[d], 0.5 / p, Ex[d]);
        md_E(lc[d], ld[d], Q[d] - C[d], C[d] - D[d], 0.5 / q, Ey[d]);
    }
    const int L = la[0] + la[1] + la[2] + lb[0] + lb[1] + lb[2] + lc[0] + lc[1] + lc[2] + ld[0] + ld[1] + ld[2];
    const double rho = p * q / (p + q);
    const double X = P[0] - Q[0], Y = P[1] - Q[1], Z = P[2] - Q[2];
    const double T = rho * (X * X + Y * Y + Z * Z);
    const double pref = 2.0 * 3.14159265358979323846 * 3.14159265358979323846 * sqrt(3.14159265358979323846) /
                        (p * q * sqrt(p + q)) * exp(-aa * ab * rab2 / p) * exp(-ac * ad * rcd2 / q);
    double F[MD_MAXL + 1], R[MD_NR];
    boys_eval_rt<double>(L, T, pref, boys, F);
    md_R(L, rho, X, Y, Z, F, R);
    const int nx = la[0] + lb[0], ny = la[1] + lb[1], nz = la[2] + lb[2];
    const int mx = lc[0] + ld[0], my = lc[1] + ld[1], mz = lc[2] + ld[2];
    double sum = 0.0;
    for (int t = 0; t <= nx; ++t)
        for (int u = 0; u <= ny; ++u)
            for (int v = 0; v <= nz; ++v) {
                const double eb = Ex[0][t] * Ex[1][u] * Ex[2][v];
                if (eb == 0.0) continue;
                double s = 0.0;
                for (int tt = 0; tt <= mx; ++tt)
                    for (int uu = 0; uu <= my; ++uu)
                        for (int vv = 0; vv <= mz; ++vv) {
                            const double ek = Ey[0][tt] * Ey[1][uu] * Ey[2][vv];
                            const double sg = ((tt + uu + vv) & 1) ? -1.0 : 1.0;
                            s += sg * ek * R[md_tuv(t + tt, u + uu, v + vv)];
                        }
                sum += eb * s;
            }
    return sum;
}

// 1-D overlap factor E_0^{ij} sqrt(pi/p) (no exponential).
RCHEM_HD inline double md_s1d(int i, int j, double PA, double AB, double ohp, double p) {
    if (i < 0 || j < 0) return 0.0;
    double E[MD_MAXE + 1];
    md_E(i, j, PA, AB, ohp, E);
    return E[0] * sqrt(3.14159265358979323846 / p);
}

// Primitive overlap, kinetic and nuclear-attraction (to a unit charge at Cc).
// kind: 0 = S, 1 = T, 2 = V.
RCHEM_HD inline double md_onee_prim(int kind, const double *A, const int *la, double aa, const double *B,
                                    const int *lb, double ab, const double *Cc, const double *boys) {
    const double p = aa + ab, ohp = 0.5 / p;
    double P[3], rab2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        P[d] = (aa * A[d] + ab * B[d]) / p;
        rab2 += (A[d] - B[d]) * (A[d] - B[d]);
    }
    const double Kab = exp(-aa * ab * rab2 / p);
    if (kind == 0) {
        double s = Kab;
        for (int d = 0; d < 3; ++d) s *= md_s1d(la[d], lb[d], P[d] - A[d], A[d] - B[d], ohp, p);
        return s;
    }
    if (kind == 1) {
        double S1[3], T1[3];
        for (int d = 0; d < 3; ++d) {
            const double pa = P[d] - A[d], abd = A[d] - B[d];
            const int j = lb[d];
            S1[d] = md_s1d(la[d], j, pa, abd, ohp, p);
            T1[d] = ab * (2 * j + 1) * S1[d] - 2.0 * ab * ab * md_s1d(la[d], j + 2, pa, abd, ohp, p);
            if (j >= 2) T1[d] -= 0.5 * j * (j - 1) * md_s1d(la[d], j - 2, pa, abd, ohp, p);
        }
        return Kab * (T1[0] * S1[1] * S1[2] + S1[0] * T1[1] * S1[2] + S1[0] * S1[1] * T1[2]);
    }
    double Ex[3][MD_MAXE + 1];
    for (int d = 0; d < 3; ++d) md_E(la[d], lb[d], P[d] - A[d], A[d] - B[d], ohp, Ex[d]);
    const int L = la[0] + la[1] + la[2] + lb[0] + lb[1] + lb[2];
    const double X = P[0] - Cc[0], Y = P[1] - Cc[1], Z = P[2] - Cc[2];
    const double T = p * (X * X + Y * Y + Z * Z);
    double F[MD_MAXL + 1], R[MD_NR];
    boys_eval_rt<double>(L, T, 1.0, boys, F);
    md_R(L, p, X, Y, Z, F, R);
    double sum = 0.0;
    for (int t = 0; t <= la[0] + lb[0]; ++t)
        for (int u = 0; u <= la[1] + lb[1]; ++u)
            for (int v = 0; v <= la[2] + lb[2]; ++v) sum += Ex[0][t] * Ex[1][u] * Ex[2][v] * R[md_tuv(t, u, v)];
    return -2.0 * 3.14159265358979323846 / p * Kab * sum;
}

// Primitive multipole moment <a| (x-Cx)^o0 (y-Cy)^o1 (z-Cz)^o2 |b> (os86.rs:775-828).
RCHEM_HD inline double md_moment_prim(const double *A, const int *la, double aa, const double *B, const int *lb,
                                      double ab, const double *Cc, const int *o) {
    const double p = aa + ab, ohp = 0.5 / p;
    double rab2 = 0.0, val = 1.0;
    for (int d = 0; d < 3; ++d) rab2 += (A[d] - B[d]) * (A[d] - B[d]);
    for (int d = 0; d < 3; ++d) {
        const double Pd = (aa * A[d] + ab * B[d]) / p;
        double s = 0.0, bc = 1.0;
        for (int j = o[d]; j >= 0; --j) {  // (x-C)^o = sum_j C(o,j) (B-C)^(o-j) (x-B)^j
            s += md_binom(o[d], j) * bc * md_s1d(la[d], lb[d] + j, Pd - A[d], A[d] - B[d], ohp, p);
            bc *= (B[d] - Cc[d]);
        }
        val *= s;
    }
    return exp(-aa * ab * rab2 / p) * val;
}
