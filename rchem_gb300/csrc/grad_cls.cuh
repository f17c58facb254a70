// grad_cls.cuh -- the two-electron gradient kernel specialised per integral
// class, in FP64, FP32 (the mixed form's small quartets) or double-float (the
// emulated form): every class of s and p shells, and the smallest classes with a
// d shell ((ds|ss), (ds|ps), (ds|ds), (dp|ss)), whose unrolled code still fits
// the registers; the larger d classes run the run-time-l kernels of grad.cuh.
//
// Same mathematics and work layout as k_grad2e (grad.cuh): McMurchie--Davidson
// Hermite integrals, the shifted-angular-momentum derivative relation, Gamma
// formed once per contracted quartet, G lanes per quartet splitting its
// primitive quartets, shuffle reduction of the 9 centre derivatives.  Here the
// angular momenta are template parameters: every loop bound, Cartesian
// component and Hermite index is a compile-time constant (static_for over
// integer sequences), so the Hermite tables, the Coulomb table R and the
// ket-contracted vectors are plain registers and the arithmetic is straight
// FMA chains instead of run-time index loops over local-memory arrays.
#pragma once
#include <utility>

#include "grad.cuh"

namespace gt {

constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
constexpr int nr(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
constexpr int tuv(int t, int u, int v) {
    const int n = t + u + v, s = u + v;
    return n * (n + 1) * (n + 2) / 6 + s * (s + 1) / 2 + v;
}
// component k of angular momentum l in the reference AO order (src/shell.rs:1-12):
// (l+1-a, a-b, b-1) for a = 1..l+1, b = 1..a
constexpr int comp(int l, int k, int axis) {
    int idx = 0;
    for (int a = 1; a <= l + 1; ++a)
        for (int b = 1; b <= a; ++b, ++idx)
            if (idx == k) return axis == 0 ? l + 1 - a : (axis == 1 ? a - b : b - 1);
    return 0;
}

// N(alpha,l,m,n) / N(alpha,L,0,0) of component k of angular momentum l
// (src/basis.rs:140-149): sqrt((2L-1)!! / ((2l-1)!! (2m-1)!! (2n-1)!!))
__device__ __forceinline__ double cnorm(int l, int k) {
    const double f2[5] = {1.0, 1.0, 3.0, 15.0, 105.0};  // (2j-1)!! for j = 0..4
    return sqrt(f2[l] / (f2[comp(l, k, 0)] * f2[comp(l, k, 1)] * f2[comp(l, k, 2)]));
}

template <typename F, int... I>
__device__ __forceinline__ void sfor_(F &&f, std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
}
// f(integral_constant<int, i>) for i = 0..N-1, unrolled at compile time
template <int N, typename F>
__device__ __forceinline__ void sfor(F &&f) {
    sfor_(f, std::make_integer_sequence<int, N>{});
}

// E[i][j][t] of x_A^i x_B^j (t <= i + j), one Cartesian direction
template <int IM, int JM, typename R>
struct Herm {
    R e[IM + 1][JM + 1][IM + JM + 1];
};

template <int IM, int JM, typename R>
__device__ __forceinline__ void herm(R PA, R AB, R ohp, Herm<IM, JM, R> &E) {
    const R PB = PA + AB;
    E.e[0][0][0] = R(1);
    sfor<IM + 1>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        if constexpr (i > 0) {
            sfor<i + 1>([&](auto t_) {
                constexpr int t = decltype(t_)::value;
                R v = R(0);
                if constexpr (t <= i - 1) v = PA * E.e[i - 1][0][t];
                if constexpr (t > 0) v = rchem_fma(ohp, E.e[i - 1][0][t - 1], v);
                if constexpr (t + 1 <= i - 1) v = rchem_fma(R(t + 1), E.e[i - 1][0][t + 1], v);
                E.e[i][0][t] = v;
            });
        }
        sfor<JM>([&](auto j_) {
            constexpr int j = decltype(j_)::value + 1;
            sfor<i + j + 1>([&](auto t_) {
                constexpr int t = decltype(t_)::value;
                R v = R(0);
                if constexpr (t <= i + j - 1) v = PB * E.e[i][j - 1][t];
                if constexpr (t > 0) v = rchem_fma(ohp, E.e[i][j - 1][t - 1], v);
                if constexpr (t + 1 <= i + j - 1) v = rchem_fma(R(t + 1), E.e[i][j - 1][t + 1], v);
                E.e[i][j][t] = v;
            });
        });
    });
}

// Hermite Coulomb integrals R_{tuv}, t+u+v <= L, from pref * F_n(T) (F[0..L]):
// R^n_000 = (-2 rho)^n F_n, R^n_{t+1,u,v} = t R^{n+1}_{t-1,u,v} + X R^{n+1}_{t,u,v} (and for u, v)
template <int L, typename R>
__device__ __forceinline__ void coulomb(R rho, R X, R Y, R Z, const R *F, R *Rt) {
    R Rn[L + 2][nr(L)];
    R pw[L + 1];
    pw[0] = R(1);
    const R m2r = R(-2) * rho;
    sfor<L>([&](auto n_) {
        constexpr int n = decltype(n_)::value + 1;
        pw[n] = pw[n - 1] * m2r;
    });
    sfor<L + 1>([&](auto m_) {
        constexpr int n = L - decltype(m_)::value;
        constexpr int top = L - n;
        sfor<top + 1>([&](auto t_) {
            sfor<top + 1>([&](auto u_) {
                sfor<top + 1>([&](auto v_) {
                    constexpr int t = decltype(t_)::value, u = decltype(u_)::value, v = decltype(v_)::value;
                    if constexpr (t + u + v <= top) {
                        R r;
                        if constexpr (t + u + v == 0) {
                            r = pw[n] * F[n];
                        } else if constexpr (t > 0) {
                            r = X * Rn[n + 1][tuv(t - 1, u, v)];
                            if constexpr (t > 1) r = rchem_fma(R(t - 1), Rn[n + 1][tuv(t - 2, u, v)], r);
                        } else if constexpr (u > 0) {
                            r = Y * Rn[n + 1][tuv(0, u - 1, v)];
                            if constexpr (u > 1) r = rchem_fma(R(u - 1), Rn[n + 1][tuv(0, u - 2, v)], r);
                        } else {
                            r = Z * Rn[n + 1][tuv(0, 0, v - 1)];
                            if constexpr (v > 1) r = rchem_fma(R(v - 1), Rn[n + 1][tuv(0, 0, v - 2)], r);
                        }
                        Rn[n][tuv(t, u, v)] = r;
                    }
                });
            });
        });
    });
    sfor<nr(L)>([&](auto i_) { Rt[decltype(i_)::value] = Rn[0][decltype(i_)::value]; });
}

// Z_{tuv} = sum_{t'u'v'} Ek_x[c][d][t'] Ek_y[..][u'] Ek_z[..][v'] R_{t+t',u+u',v+v'}, t+u+v <= BM
// (the ket of components (cx,cy,cz),(dx,dy,dz) contracted with R; the sign (-1)^t' is in Ek)
template <int BM, int CX, int CY, int CZ, int DX, int DY, int DZ, int IM, int JM, typename R>
__device__ __forceinline__ void zvec(const Herm<IM, JM, R> *Ek, const R *Rt, R *Zo) {
    sfor<BM + 1>([&](auto t_) {
        sfor<BM + 1>([&](auto u_) {
            sfor<BM + 1>([&](auto v_) {
                constexpr int t = decltype(t_)::value, u = decltype(u_)::value, v = decltype(v_)::value;
                if constexpr (t + u + v <= BM) {
                    R z = R(0);
                    sfor<CX + DX + 1>([&](auto a_) {
                        constexpr int a = decltype(a_)::value;
                        sfor<CY + DY + 1>([&](auto b_) {
                            constexpr int b = decltype(b_)::value;
                            const R fxy = Ek[0].e[CX][DX][a] * Ek[1].e[CY][DY][b];
                            sfor<CZ + DZ + 1>([&](auto c_) {
                                constexpr int c = decltype(c_)::value;
                                z = rchem_fma(fxy * Ek[2].e[CZ][DZ][c], Rt[tuv(t + a, u + b, v + c)], z);
                            });
                        });
                    });
                    Zo[tuv(t, u, v)] = z;
                }
            });
        });
    });
}

// sum_{tuv} Eb_x[ax][bx][t] Eb_y[ay][by][u] Eb_z[az][bz][v] Z_{tuv}
template <int AX, int AY, int AZ, int BX, int BY, int BZ, int IM, int JM, typename R>
__device__ __forceinline__ R dot(const Herm<IM, JM, R> *Eb, const R *Zv) {
    R s = R(0);
    sfor<AX + BX + 1>([&](auto t_) {
        constexpr int t = decltype(t_)::value;
        sfor<AY + BY + 1>([&](auto u_) {
            constexpr int u = decltype(u_)::value;
            const R exy = Eb[0].e[AX][BX][t] * Eb[1].e[AY][BY][u];
            sfor<AZ + BZ + 1>([&](auto v_) {
                constexpr int v = decltype(v_)::value;
                s = rchem_fma(exy * Eb[2].e[AZ][BZ][v], Zv[tuv(t, u, v)], s);
            });
        });
    });
    return s;
}

}  // namespace gt

template <int LA, int LB, int LC, int LD, typename R>
__global__ void __launch_bounds__(64) k_grad2e_cls(GradArgs g) {
    using namespace gt;
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int L1 = LA + LB + LC + LD + 1;
    constexpr int BM = LA + LB + 1;  // bra Hermite range including the shift
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
    const int n = bp.mn;
    const double *Dg = g.D + bp.moff;
    double deg = 8.0;
    if (bp.diag) deg *= 0.5;
    if (kp.diag) deg *= 0.5;
    if (seg.bra == seg.ket0 + off) deg *= 0.5;
    // Gamma with the degeneracy and the component norms (1 for s and p shells),
    // formed in FP64 and then rounded to the kernel's arithmetic
    constexpr bool kNorms = LA > 1 || LB > 1 || LC > 1 || LD > 1;
    R Gam[NC * ND * NA * NB];
    sfor<NC>([&](auto kc_) {
        sfor<ND>([&](auto kd_) {
            constexpr int kc = decltype(kc_)::value, kd = decltype(kd_)::value;
            const int l_ = kp.aoA + kc, s_ = kp.aoB + kd;
            const double Dls = Dg[l_ * n + s_];
            sfor<NA>([&](auto ka_) {
                sfor<NB>([&](auto kb_) {
                    constexpr int ka = decltype(ka_)::value, kb = decltype(kb_)::value;
                    const int mu = bp.aoA + ka, nu = bp.aoB + kb;
                    double w = deg;
                    if constexpr (kNorms)
                        w *= cnorm(LA, ka) * cnorm(LB, kb) * cnorm(LC, kc) * cnorm(LD, kd);
                    Gam[((kc * ND + kd) * NA + ka) * NB + kb] = gt_narrow(
                        w * (2.0 * Dg[mu * n + nu] * Dls -
                             0.5 * (Dg[mu * n + l_] * Dg[nu * n + s_] + Dg[mu * n + s_] * Dg[nu * n + l_])),
                        (R *)nullptr);
                });
            });
        });
    });
    R AB[3], CD[3];
    Tabs<R>::ab(bp, AB);
    Tabs<R>::ab(kp, CD);
    const R *btab = GradPrim<R>::boys(g);
    R gA[3] = {R(0), R(0), R(0)}, gB[3] = {R(0), R(0), R(0)}, gC[3] = {R(0), R(0), R(0)};
    const int nk = kp.npp, ntot = active ? bp.npp * nk : 0;  // idle lanes only join the reduction
    for (int tq = r; tq < ntot; tq += G) {
        const int ia = tq / nk, ic = tq - ia * nk;
        R p, ohp, Pc[3], PA[3], Kab, aa, q, ohq, Qc[3], QC[3], Kcd, ac;
        GradPrim<R>::get(g, bp.prim0 + ia, p, ohp, Pc, PA, Kab, aa);
        GradPrim<R>::get(g, kp.prim0 + ic, q, ohq, Qc, QC, Kcd, ac);
        const R ab = p - aa;
        R rs, ipq, rho, qi, pi;
        // (pp|ps) and (pp|pp) compute the factors: with the table's loads in
        // flight they spill several KB more per thread
        pq_factors<R, !(LA == 1 && LB == 1 && LC == 1)>(g, bp.prim0 + ia, kp.prim0 + ic, p, q, rs, ipq, rho, qi, pi);
        const R X = Pc[0] - Qc[0], Y = Pc[1] - Qc[1], Zc = Pc[2] - Qc[2];
        const R T = rho * (X * X + Y * Y + Zc * Zc);
        R F[L1 + 1], Rt[nr(L1)];
        // FP64: one instruction stream for every T (not (pp|ps), (pp|pp): register-bound)
        if constexpr (std::is_same<R, double>::value && L1 <= BOYS_FAR_M - 1 && !(LA == 1 && LB == 1 && LC == 1))
            boys_eval_u<L1, true>(T, Kab * Kcd * rs, btab, g.boysfar, F);
        else
            boys_eval<L1, R>(T, Kab * Kcd * rs, btab, F);
        coulomb<L1, R>(rho, X, Y, Zc, F, Rt);
        Herm<LA + 1, LB + 1, R> Eb[3];
        Herm<LC + 1, LD, R> Ek[3];
        sfor<3>([&](auto d_) {
            constexpr int d = decltype(d_)::value;
            herm<LA + 1, LB + 1, R>(PA[d], AB[d], ohp, Eb[d]);
            herm<LC + 1, LD, R>(QC[d], CD[d], ohq, Ek[d]);
            sfor<LC + 2>([&](auto i_) {  // ket sign (-1)^t folded in
                sfor<LD + 1>([&](auto j_) {
                    constexpr int i = decltype(i_)::value, j = decltype(j_)::value;
                    sfor<(i + j + 1) / 2>([&](auto h_) {
                        constexpr int t = 2 * decltype(h_)::value + 1;
                        Ek[d].e[i][j][t] = -Ek[d].e[i][j][t];
                    });
                });
            });
        });
        const R a2 = aa + aa, b2 = ab + ab, c2 = ac + ac;
        sfor<NC>([&](auto kc_) {
            sfor<ND>([&](auto kd_) {
                constexpr int kc = decltype(kc_)::value, kd = decltype(kd_)::value;
                constexpr int cx = comp(LC, kc, 0), cy = comp(LC, kc, 1), cz = comp(LC, kc, 2);
                constexpr int dx = comp(LD, kd, 0), dy = comp(LD, kd, 1), dz = comp(LD, kd, 2);
                // ket contracted with R: unshifted (the bra may be shifted by one), C shifted by +-1
                R Z0[nr(BM)], Zp[3][nr(BM - 1)], Zm[3][nr(BM - 1)];
                zvec<BM, cx, cy, cz, dx, dy, dz>(Ek, Rt, Z0);
                zvec<BM - 1, cx + 1, cy, cz, dx, dy, dz>(Ek, Rt, Zp[0]);
                zvec<BM - 1, cx, cy + 1, cz, dx, dy, dz>(Ek, Rt, Zp[1]);
                zvec<BM - 1, cx, cy, cz + 1, dx, dy, dz>(Ek, Rt, Zp[2]);
                if constexpr (cx > 0) zvec<BM - 1, cx - 1, cy, cz, dx, dy, dz>(Ek, Rt, Zm[0]);
                if constexpr (cy > 0) zvec<BM - 1, cx, cy - 1, cz, dx, dy, dz>(Ek, Rt, Zm[1]);
                if constexpr (cz > 0) zvec<BM - 1, cx, cy, cz - 1, dx, dy, dz>(Ek, Rt, Zm[2]);
                sfor<NA>([&](auto ka_) {
                    sfor<NB>([&](auto kb_) {
                        constexpr int ka = decltype(ka_)::value, kb = decltype(kb_)::value;
                        constexpr int ax = comp(LA, ka, 0), ay = comp(LA, ka, 1), az = comp(LA, ka, 2);
                        constexpr int bx = comp(LB, kb, 0), by = comp(LB, kb, 1), bz = comp(LB, kb, 2);
                        const R Gm = Gam[((kc * ND + kd) * NA + ka) * NB + kb];
                        // centre A: 2 alpha_a (a+1|..) - a_x (a-1|..)
                        R vx = a2 * dot<ax + 1, ay, az, bx, by, bz>(Eb, Z0);
                        R vy = a2 * dot<ax, ay + 1, az, bx, by, bz>(Eb, Z0);
                        R vz = a2 * dot<ax, ay, az + 1, bx, by, bz>(Eb, Z0);
                        if constexpr (ax > 0) vx = vx - R(ax) * dot<ax - 1, ay, az, bx, by, bz>(Eb, Z0);
                        if constexpr (ay > 0) vy = vy - R(ay) * dot<ax, ay - 1, az, bx, by, bz>(Eb, Z0);
                        if constexpr (az > 0) vz = vz - R(az) * dot<ax, ay, az - 1, bx, by, bz>(Eb, Z0);
                        gA[0] = rchem_fma(Gm, vx, gA[0]);
                        gA[1] = rchem_fma(Gm, vy, gA[1]);
                        gA[2] = rchem_fma(Gm, vz, gA[2]);
                        // centre B
                        vx = b2 * dot<ax, ay, az, bx + 1, by, bz>(Eb, Z0);
                        vy = b2 * dot<ax, ay, az, bx, by + 1, bz>(Eb, Z0);
                        vz = b2 * dot<ax, ay, az, bx, by, bz + 1>(Eb, Z0);
                        if constexpr (bx > 0) vx = vx - R(bx) * dot<ax, ay, az, bx - 1, by, bz>(Eb, Z0);
                        if constexpr (by > 0) vy = vy - R(by) * dot<ax, ay, az, bx, by - 1, bz>(Eb, Z0);
                        if constexpr (bz > 0) vz = vz - R(bz) * dot<ax, ay, az, bx, by, bz - 1>(Eb, Z0);
                        gB[0] = rchem_fma(Gm, vx, gB[0]);
                        gB[1] = rchem_fma(Gm, vy, gB[1]);
                        gB[2] = rchem_fma(Gm, vz, gB[2]);
                        // centre C
                        vx = c2 * dot<ax, ay, az, bx, by, bz>(Eb, Zp[0]);
                        vy = c2 * dot<ax, ay, az, bx, by, bz>(Eb, Zp[1]);
                        vz = c2 * dot<ax, ay, az, bx, by, bz>(Eb, Zp[2]);
                        if constexpr (cx > 0) vx = vx - R(cx) * dot<ax, ay, az, bx, by, bz>(Eb, Zm[0]);
                        if constexpr (cy > 0) vy = vy - R(cy) * dot<ax, ay, az, bx, by, bz>(Eb, Zm[1]);
                        if constexpr (cz > 0) vz = vz - R(cz) * dot<ax, ay, az, bx, by, bz>(Eb, Zm[2]);
                        gC[0] = rchem_fma(Gm, vx, gC[0]);
                        gC[1] = rchem_fma(Gm, vy, gC[1]);
                        gC[2] = rchem_fma(Gm, vz, gC[2]);
                    });
                });
            });
        });
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
