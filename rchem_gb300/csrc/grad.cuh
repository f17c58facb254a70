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
// and only the 9 centre derivatives leave the thread (translational
// invariance gives the fourth centre).
#pragma once
#include "boys.cuh"
#include "md.cuh"
#include "rchem_types.h"

#define GR_NI 4    // powers 0..3 per centre and direction (l <= 2, shifted by one)
#define GR_NT 7    // Hermite index t <= 6
#define GR_LMAX 9  // largest total L of a shifted quartet
#define GR_NR 220  // (t,u,v) with t+u+v <= 9

struct GradArgs {
    const int2 *quartets;  // (bra pair, ket pair) of every surviving quartet
    int nq;
    int nbf;
    const ShellPair *pairs;
    const PairPrim *prims;
    const int *shell_atom;
    const int *shell_l;
    const double *boys64;
    const double *D;
    double *grad;  // 3 * natoms
};

// E[i][j][t] of x_A^i x_B^j for i <= imax, j <= jmax (no exponential factor)
__device__ __forceinline__ void gr_herm(int imax, int jmax, double PA, double AB, double ohp,
                                        double (*E)[GR_NI][GR_NT]) {
    const double PB = PA + AB;  // P - B = (P - A) + (A - B)
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j <= jmax; ++j)
            for (int t = 0; t < GR_NT; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
    for (int i = 0; i <= imax; ++i) {
        if (i > 0)
            for (int t = 0; t <= i; ++t) {
                double v = PA * E[i - 1][0][t];
                if (t > 0) v += ohp * E[i - 1][0][t - 1];
                if (t + 1 <= i - 1) v += (t + 1) * E[i - 1][0][t + 1];
                E[i][0][t] = v;
            }
        for (int j = 1; j <= jmax; ++j)
            for (int t = 0; t <= i + j; ++t) {
                double v = PB * E[i][j - 1][t];
                if (t > 0) v += ohp * E[i][j - 1][t - 1];
                if (t + 1 <= i + j - 1) v += (t + 1) * E[i][j - 1][t + 1];
                E[i][j][t] = v;
            }
    }
}

__device__ __forceinline__ void gr_R(int L, double a, double X, double Y, double Z, const double *F, double *out) {
    double buf[2][GR_NR];
    double *cur = buf[0], *nxt = buf[1];
    const double m2a = -2.0 * a;
    double pw = 1.0;
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
                    if (N == 0) r = pw * F[n];
                    else if (t > 0) r = X * cur[md_tuv(t - 1, u, v)] + (t > 1 ? (t - 1) * cur[md_tuv(t - 2, u, v)] : 0.0);
                    else if (u > 0) r = Y * cur[md_tuv(0, u - 1, v)] + (u > 1 ? (u - 1) * cur[md_tuv(0, u - 2, v)] : 0.0);
                    else r = Z * cur[md_tuv(0, 0, v - 1)] + (v > 1 ? (v - 1) * cur[md_tuv(0, 0, v - 2)] : 0.0);
                    nxt[md_tuv(t, u, v)] = r;
                }
        double *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    const int cnt = (L + 1) * (L + 2) * (L + 3) / 6;
    for (int i = 0; i < cnt; ++i) out[i] = cur[i];
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

// Z_{tuv} = sum_{t'u'v'} (-1)^{t'+u'+v'} E^{cd}_{t'u'v'} R_{t+t',u+u',v+v'} for every bra
// Hermite index with t+u+v <= bmax (box of side zd): the ket of one component
// contracted with the Coulomb integrals once, reused by every bra component.
__device__ __forceinline__ void gr_zvec(const double (*Ek)[GR_NI][GR_NI][GR_NT], const int *c, const int *d,
                                        const double *R, int zd, int bmax, double *Z) {
    for (int t = 0; t < zd; ++t)
        for (int u = 0; u < zd; ++u)
            for (int v = 0; v < zd; ++v) {
                double z = 0.0;
                if (t + u + v <= bmax)
                    for (int tt = 0; tt <= c[0] + d[0]; ++tt) {
                        const double fx = Ek[0][c[0]][d[0]][tt];
                        for (int uu = 0; uu <= c[1] + d[1]; ++uu) {
                            const double fy = fx * Ek[1][c[1]][d[1]][uu];
                            for (int vv = 0; vv <= c[2] + d[2]; ++vv)
                                z += fy * Ek[2][c[2]][d[2]][vv] * R[md_tuv(t + tt, u + uu, v + vv)];
                        }
                    }
                Z[(t * zd + u) * zd + v] = z;
            }
}

// sum_{tuv} E^{ab}_{tuv} Z_{tuv}
__device__ __forceinline__ double gr_dot(const double (*Eb)[GR_NI][GR_NI][GR_NT], const int *a, const int *b,
                                         const double *Z, int zd) {
    double s = 0.0;
    for (int t = 0; t <= a[0] + b[0]; ++t) {
        const double ex = Eb[0][a[0]][b[0]][t];
        for (int u = 0; u <= a[1] + b[1]; ++u) {
            const double ey = ex * Eb[1][a[1]][b[1]][u];
            const double *Zr = Z + (t * zd + u) * zd;
            for (int v = 0; v <= a[2] + b[2]; ++v) s += ey * Eb[2][a[2]][b[2]][v] * Zr[v];
        }
    }
    return s;
}

#define GR_ZD 6                           // bra Hermite box side: la+lb+2 <= 6
#define GR_ZN (GR_ZD * GR_ZD * GR_ZD)

// One thread per contracted shell quartet (unique, 8-fold): 9 centre derivatives
// of sum Gamma (ab|cd), weighted by the degeneracy factor, added to the gradient.
__global__ void __launch_bounds__(64) k_grad2e(GradArgs g) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= g.nq) return;
    const int2 q = g.quartets[qi];
    const ShellPair bp = g.pairs[q.x], kp = g.pairs[q.y];
    const int la = g.shell_l[bp.A], lb = g.shell_l[bp.B], lc = g.shell_l[kp.A], ld = g.shell_l[kp.B];
    const int na = (la + 1) * (la + 2) / 2, nb = (lb + 1) * (lb + 2) / 2, nc = (lc + 1) * (lc + 2) / 2,
              nd = (ld + 1) * (ld + 2) / 2;
    const int n = bp.mn;  // the quartet's geometry block of the packed D
    const double *Dg = g.D + bp.moff;
    double deg = 8.0;
    if (bp.diag) deg *= 0.5;
    if (kp.diag) deg *= 0.5;
    if (q.x == q.y) deg *= 0.5;
    double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
    const int L1 = la + lb + lc + ld + 1;
    const int zd = la + lb + 2;
    double Eb[3][GR_NI][GR_NI][GR_NT], Ek[3][GR_NI][GR_NI][GR_NT], R[GR_NR], F[GR_LMAX + 1];
    double Z0[GR_ZN], Zp[3][GR_ZN], Zm[3][GR_ZN];
    for (int ia = 0; ia < bp.npp; ++ia) {
        const PairPrim pa = g.prims[bp.prim0 + ia];
        const double aa = pa.pad, ab = pa.p - pa.pad;  // pad holds the exponent on the first shell
        for (int ic = 0; ic < kp.npp; ++ic) {
            const PairPrim pc = g.prims[kp.prim0 + ic];
            const double ac = pc.pad;
            const double pq = pa.p + pc.p, rs = rsqrt(pq), ipq = rs * rs, rho = pa.p * pc.p * ipq;
            const double X = pa.P[0] - pc.P[0], Y = pa.P[1] - pc.P[1], Zc = pa.P[2] - pc.P[2];
            const double T = rho * (X * X + Y * Y + Zc * Zc);
            boys_eval_rt<double>(L1, T, pa.K * pc.K * rs, g.boys64, F);
            gr_R(L1, rho, X, Y, Zc, F, R);
            for (int dd = 0; dd < 3; ++dd) {
                gr_herm(la + 1, lb + 1, pa.PA[dd], bp.AB[dd], pa.ohp, Eb[dd]);
                gr_herm(lc + 1, ld, pc.PA[dd], kp.AB[dd], pc.ohp, Ek[dd]);
                for (int i = 0; i <= lc + 1; ++i)  // ket sign (-1)^t folded in
                    for (int j = 0; j <= ld; ++j)
                        for (int t = 1; t < GR_NT; t += 2) Ek[dd][i][j][t] = -Ek[dd][i][j][t];
            }
            int A[3], B[3], Cc[3], Dd[3], s[3];
            for (int kc = 0; kc < nc; ++kc) {
                gr_comp(lc, kc, Cc);
                const double cnc = gr_cnorm(Cc);
                const int l_ = kp.aoA + kc;
                for (int kd = 0; kd < nd; ++kd) {
                    gr_comp(ld, kd, Dd);
                    const double cncd = cnc * gr_cnorm(Dd);
                    const int s_ = kp.aoB + kd;
                    // ket contracted with R: unshifted (bra may be shifted by one) and C-shifted
                    gr_zvec(Ek, Cc, Dd, R, zd, la + lb + 1, Z0);
                    for (int x = 0; x < 3; ++x) {
                        s[0] = Cc[0]; s[1] = Cc[1]; s[2] = Cc[2];
                        s[x] += 1;
                        gr_zvec(Ek, s, Dd, R, zd, la + lb, Zp[x]);
                        if (Cc[x] > 0) {
                            s[x] -= 2;
                            gr_zvec(Ek, s, Dd, R, zd, la + lb, Zm[x]);
                        }
                    }
                    for (int ka = 0; ka < na; ++ka) {
                        gr_comp(la, ka, A);
                        const double cna = gr_cnorm(A) * cncd;
                        const int mu = bp.aoA + ka;
                        for (int kb = 0; kb < nb; ++kb) {
                            gr_comp(lb, kb, B);
                            const int nu = bp.aoB + kb;
                            const double Gam = deg * cna * gr_cnorm(B) *
                                               (2.0 * Dg[mu * n + nu] * Dg[l_ * n + s_] -
                                                0.5 * (Dg[mu * n + l_] * Dg[nu * n + s_] +
                                                       Dg[mu * n + s_] * Dg[nu * n + l_]));
                            if (Gam == 0.0) continue;
                            for (int x = 0; x < 3; ++x) {
                                // centre A: 2 alpha_a (a+1|..) - a_x (a-1|..)
                                s[0] = A[0]; s[1] = A[1]; s[2] = A[2];
                                s[x] += 1;
                                double v = 2.0 * aa * gr_dot(Eb, s, B, Z0, zd);
                                if (A[x] > 0) {
                                    s[x] -= 2;
                                    v -= A[x] * gr_dot(Eb, s, B, Z0, zd);
                                }
                                gA[x] += Gam * v;
                                // centre B
                                s[0] = B[0]; s[1] = B[1]; s[2] = B[2];
                                s[x] += 1;
                                v = 2.0 * ab * gr_dot(Eb, A, s, Z0, zd);
                                if (B[x] > 0) {
                                    s[x] -= 2;
                                    v -= B[x] * gr_dot(Eb, A, s, Z0, zd);
                                }
                                gB[x] += Gam * v;
                                // centre C
                                v = 2.0 * ac * gr_dot(Eb, A, B, Zp[x], zd);
                                if (Cc[x] > 0) v -= Cc[x] * gr_dot(Eb, A, B, Zm[x], zd);
                                gC[x] += Gam * v;
                            }
                        }
                    }
                }
            }
        }
    }
    const int atA = g.shell_atom[bp.A], atB = g.shell_atom[bp.B], atC = g.shell_atom[kp.A],
              atD = g.shell_atom[kp.B];
    for (int x = 0; x < 3; ++x) {
        atomicAdd(g.grad + 3 * atA + x, gA[x]);
        atomicAdd(g.grad + 3 * atB + x, gB[x]);
        atomicAdd(g.grad + 3 * atC + x, gC[x]);
        atomicAdd(g.grad + 3 * atD + x, -(gA[x] + gB[x] + gC[x]));
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

__global__ void k_grad1e(long long packed, int ngeom, const GeomDev *geo, const AOGrad *ao, const ShellGrad *sh,
                         const double *pexp, const double *pcoef, int natoms_total, const double *Z,
                         const double *Ratoms, const double *boys, const double *D, const double *W, double *grad) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= packed) return;
    const GeomDev gm = geo[geom_of(geo, ngeom, idx)];
    const int loc = (int)(idx - gm.moff), mu = gm.ao0 + loc / gm.n, nu = gm.ao0 + loc % gm.n;
    const double Dmn = D[idx], Wmn = W[idx];
    const AOGrad a = ao[mu], b = ao[nu];
    const ShellGrad sa = sh[a.shell], sb = sh[b.shell];
    double gH[3] = {0, 0, 0}, gS[3] = {0, 0, 0};
    for (int j = 0; j < sb.nprim; ++j) {
        const double eb = pexp[sb.prim0 + j], cb = pcoef[sb.prim0 + j];
        for (int i = 0; i < sa.nprim; ++i) {
            const double ea = pexp[sa.prim0 + i], cc = pcoef[sa.prim0 + i] * cb * a.cn * b.cn;
            for (int x = 0; x < 3; ++x) {
                int up[3] = {a.lmn[0], a.lmn[1], a.lmn[2]}, dn[3] = {a.lmn[0], a.lmn[1], a.lmn[2]};
                up[x] += 1;
                dn[x] -= 1;
                const bool has_dn = a.lmn[x] > 0;
                // overlap and kinetic
                double s = 2.0 * ea * md_onee_prim(0, sa.R, up, ea, sb.R, b.lmn, eb, sa.R, boys);
                double t = 2.0 * ea * md_onee_prim(1, sa.R, up, ea, sb.R, b.lmn, eb, sa.R, boys);
                if (has_dn) {
                    s -= a.lmn[x] * md_onee_prim(0, sa.R, dn, ea, sb.R, b.lmn, eb, sa.R, boys);
                    t -= a.lmn[x] * md_onee_prim(1, sa.R, dn, ea, sb.R, b.lmn, eb, sa.R, boys);
                }
                gS[x] += cc * s;
                gH[x] += cc * t;
                // nuclear attraction, each nucleus of this geometry
                for (int c = gm.atom0; c < gm.atom0 + gm.natoms; ++c) {
                    double v = 2.0 * ea * md_onee_prim(2, sa.R, up, ea, sb.R, b.lmn, eb, Ratoms + 3 * c, boys);
                    if (has_dn) v -= a.lmn[x] * md_onee_prim(2, sa.R, dn, ea, sb.R, b.lmn, eb, Ratoms + 3 * c, boys);
                    v *= cc * Z[c];
                    gH[x] += v;
                    atomicAdd(grad + 3 * c + x, -4.0 * Dmn * v);
                }
            }
        }
    }
    for (int x = 0; x < 3; ++x) atomicAdd(grad + 3 * sa.atom + x, 4.0 * Dmn * gH[x] - 4.0 * Wmn * gS[x]);
    (void)natoms_total;
}
