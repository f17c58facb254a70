// onee_cls.cuh -- overlap, kinetic-energy and nuclear-attraction matrices
// (src/basis.rs:214-338 over src/integrals/os86.rs:629-773) with one thread per
// shell pair and the angular momenta as template parameters.
//
// Per primitive pair the Gaussian product, the 1-D Obara--Saika overlap tables
// (x, y, z; the kinetic term needs the ket index raised by two) and the Hermite
// expansion coefficients E^{ij}_t are formed once and serve every Cartesian
// component pair of the shell pair.  For V the nuclei are summed in Hermite
// space first: Phi_tuv = sum_C Z_C R_tuv(P - C) (one Boys evaluation and one
// Coulomb table per nucleus), then each component pair contracts
// E^x_t E^y_u E^z_v Phi_tuv.  A component-per-thread kernel repeats the Boys
// function and the Coulomb table for every component pair (9x for a (p|p)
// pair, 36x for (d|d)).
//
// Values as the reference defines them: contracted over the shell's primitive
// coefficients (times N(alpha, l, 0, 0)) and scaled by each component's
// N(alpha,l,m,n)/N(alpha,L,0,0) ratio; V = sum_C Z_C <a|-1/|r - C||b> over the
// geometry's atoms; only the lower triangle is evaluated (row shell = bra) and
// mirrored (src/basis.rs:237-248).
#pragma once
#include "eri_kernel.cuh"
#include "grad_cls.cuh"

// One shell pair of one geometry: shell indices, the first AO of each shell
// within the geometry's block (ra >= rb), the block (moff, n) and its atoms.
struct OneePair {
    int sa, sb, ra, rb, moff, n, atom0, natoms;
};

// matrix kinds of the class kernels
#define RCHEM_ONEE_S 0
#define RCHEM_ONEE_T 1
#define RCHEM_ONEE_V 2
#define RCHEM_ONEE_H 5  // T + V in one pass (the core Hamiltonian)

namespace oe {
using gt::comp;
using gt::ncart;
using gt::nr;
using gt::sfor;
using gt::tuv;

constexpr double fact2c(int n) {
    double r = 1.0;
    for (int k = n; k > 1; k -= 2) r *= k;
    return r;
}
// square of the component normalisation ratio N(alpha,l,m,n)/N(alpha,L,0,0)
constexpr double cn2(int l, int k) {
    return fact2c(2 * l - 1) /
           (fact2c(2 * comp(l, k, 0) - 1) * fact2c(2 * comp(l, k, 1) - 1) * fact2c(2 * comp(l, k, 2) - 1));
}

// 1-D overlap s[i][j] of x_A^i x_B^j over the Gaussian product, without its
// sqrt(pi/p) factor (Obara--Saika): s(i+1,j) = PA s(i,j) + (i s(i-1,j) + j s(i,j-1)) / 2p,
// s(i,j+1) = PB s(i,j) + (i s(i-1,j) + j s(i,j-1)) / 2p
template <int IM, int JM>
__device__ __forceinline__ void ovl1d(double PA, double PB, double ohp, double (&s)[IM + 1][JM + 1]) {
    s[0][0] = 1.0;
    sfor<IM>([&](auto i_) {
        constexpr int i = decltype(i_)::value;
        double v = PA * s[i][0];
        if constexpr (i > 0) v = fma(ohp * i, s[i - 1][0], v);
        s[i + 1][0] = v;
    });
    sfor<JM>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        sfor<IM + 1>([&](auto i_) {
            constexpr int i = decltype(i_)::value;
            double v = PB * s[i][j];
            if constexpr (i > 0) v = fma(ohp * i, s[i - 1][j], v);
            if constexpr (j > 0) v = fma(ohp * j, s[i][j - 1], v);
            s[i][j + 1] = v;
        });
    });
}

// 1-D kinetic factor: b (2j+1) s(i,j) - 2 b^2 s(i,j+2) - j(j-1)/2 s(i,j-2)
template <int I, int J, int IM, int JM>
__device__ __forceinline__ double kin1d(const double (&s)[IM + 1][JM + 1], double eb) {
    double t = eb * (2 * J + 1) * s[I][J] - 2.0 * eb * eb * s[I][J + 2];
    if constexpr (J >= 2) t -= 0.5 * J * (J - 1) * s[I][J - 2];
    return t;
}
}  // namespace oe

template <int LA, int LB, int KIND>
__global__ void __launch_bounds__(128)
    k_onee_cls(int npairs, const OneePair *__restrict__ pairs, const ShellGrad *__restrict__ sh,
               const double *__restrict__ pexp, const double *__restrict__ pcoef, const double *__restrict__ Zn,
               const double *__restrict__ Ratoms, const double *__restrict__ boys, double *__restrict__ out) {
    using namespace oe;
    constexpr int NA = ncart(LA), NB = ncart(LB), L = LA + LB;
    constexpr bool DO_S = KIND == RCHEM_ONEE_S;
    constexpr bool DO_T = KIND == RCHEM_ONEE_T || KIND == RCHEM_ONEE_H;
    constexpr bool DO_V = KIND == RCHEM_ONEE_V || KIND == RCHEM_ONEE_H;
    constexpr int JS = DO_T ? LB + 2 : LB;  // ket powers of the overlap tables
    constexpr double PI = 3.14159265358979323846;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= npairs) return;
    const OneePair pr = pairs[idx];
    const ShellGrad A = sh[pr.sa], B = sh[pr.sb];
    double AB[3], rab2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        AB[d] = A.R[d] - B.R[d];
        rab2 = fma(AB[d], AB[d], rab2);
    }
    double acc[NA][NB];
    sfor<NA>([&](auto a_) { sfor<NB>([&](auto b_) { acc[decltype(a_)::value][decltype(b_)::value] = 0.0; }); });

    for (int jb = 0; jb < B.nprim; ++jb) {
        const double eb = pexp[B.prim0 + jb], cb = pcoef[B.prim0 + jb];
        for (int ia = 0; ia < A.nprim; ++ia) {
            const double ea = pexp[A.prim0 + ia];
            const double p = ea + eb, rp = 1.0 / p, ohp = 0.5 * rp;
            const double cc = pcoef[A.prim0 + ia] * cb * exp(-ea * eb * rp * rab2);
            double PA[3], PB[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                PA[d] = -eb * rp * AB[d];  // P - A = b (B - A) / p
                PB[d] = ea * rp * AB[d];   // P - B = a (A - B) / p
            }
            if constexpr (DO_S || DO_T) {
                double s[3][LA + 1][JS + 1];
#pragma unroll
                for (int d = 0; d < 3; ++d) ovl1d<LA, JS>(PA[d], PB[d], ohp, s[d]);
                const double f = cc * (PI * rp) * sqrt(PI * rp);  // (pi/p)^{3/2}
                sfor<NA>([&](auto a_) {
                    sfor<NB>([&](auto b_) {
                        constexpr int a = decltype(a_)::value, b = decltype(b_)::value;
                        constexpr int ax = comp(LA, a, 0), ay = comp(LA, a, 1), az = comp(LA, a, 2);
                        constexpr int bx = comp(LB, b, 0), by = comp(LB, b, 1), bz = comp(LB, b, 2);
                        const double sx = s[0][ax][bx], sy = s[1][ay][by], sz = s[2][az][bz];
                        if constexpr (DO_S) acc[a][b] = fma(f, sx * sy * sz, acc[a][b]);
                        if constexpr (DO_T) {
                            const double tx = kin1d<ax, bx, LA, JS>(s[0], eb);
                            const double ty = kin1d<ay, by, LA, JS>(s[1], eb);
                            const double tz = kin1d<az, bz, LA, JS>(s[2], eb);
                            acc[a][b] = fma(f, tx * sy * sz + sx * ty * sz + sx * sy * tz, acc[a][b]);
                        }
                    });
                });
            }
            if constexpr (DO_V) {
                const double P0 = A.R[0] + PA[0], P1 = A.R[1] + PA[1], P2 = A.R[2] + PA[2];
                double Phi[nr(L)];
#pragma unroll
                for (int k = 0; k < nr(L); ++k) Phi[k] = 0.0;
                for (int at = pr.atom0; at < pr.atom0 + pr.natoms; ++at) {
                    const double X = P0 - Ratoms[3 * at], Y = P1 - Ratoms[3 * at + 1], Z = P2 - Ratoms[3 * at + 2];
                    double F[L + 1], Rt[nr(L)];
                    boys_eval<L, double>(p * (X * X + Y * Y + Z * Z), Zn[at], boys, F);
                    gt::coulomb<L, double>(p, X, Y, Z, F, Rt);
#pragma unroll
                    for (int k = 0; k < nr(L); ++k) Phi[k] += Rt[k];
                }
                gt::Herm<LA, LB, double> E[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) gt::herm<LA, LB, double>(PA[d], AB[d], ohp, E[d]);
                const double f = -2.0 * PI * rp * cc;
                sfor<NA>([&](auto a_) {
                    sfor<NB>([&](auto b_) {
                        constexpr int a = decltype(a_)::value, b = decltype(b_)::value;
                        constexpr int ax = comp(LA, a, 0), ay = comp(LA, a, 1), az = comp(LA, a, 2);
                        constexpr int bx = comp(LB, b, 0), by = comp(LB, b, 1), bz = comp(LB, b, 2);
                        double sum = 0.0;
                        sfor<ax + bx + 1>([&](auto t_) {
                            sfor<ay + by + 1>([&](auto u_) {
                                constexpr int t = decltype(t_)::value, u = decltype(u_)::value;
                                const double exy = E[0].e[ax][bx][t] * E[1].e[ay][by][u];
                                sfor<az + bz + 1>([&](auto v_) {
                                    constexpr int v = decltype(v_)::value;
                                    sum = fma(exy * E[2].e[az][bz][v], Phi[tuv(t, u, v)], sum);
                                });
                            });
                        });
                        acc[a][b] = fma(f, sum, acc[a][b]);
                    });
                });
            }
        }
    }
    const bool diag = pr.sa == pr.sb;
    double *o = out + pr.moff;
    sfor<NA>([&](auto a_) {
        sfor<NB>([&](auto b_) {
            constexpr int a = decltype(a_)::value, b = decltype(b_)::value;
            if (!diag || b <= a) {
                const int r = pr.ra + a, c = pr.rb + b;
                const double v = acc[a][b] * (sqrt(cn2(LA, a)) * sqrt(cn2(LB, b)));
                o[(size_t)r * pr.n + c] = v;
                o[(size_t)c * pr.n + r] = v;
            }
        });
    });
}
