// host_eri_check.cpp -- test harness (not part of the library).
//
// Compiles the generated HGP class code (csrc/_gen/eri_class_*.inc) and the
// Boys evaluator (csrc/boys.cuh) for the host with g++, so the CPU test suite
// can check the code generator against the oracle without a GPU.  It repeats
// the primitive loop of eri_kernel.cuh for one contracted shell quartet.
#define __host__
#define __device__
#define __forceinline__ inline
#include <cmath>
#include <cstring>
#include <vector>

#include "boys.cuh"

template <int LA, int LB, int LC, int LD> struct EriClass;
#include "eri_all.inc"

// the warp-cooperative programs (csrc/_gen/eri_prog_*.inc), read on the host
struct uint4 {
    unsigned x, y, z, w;
};
struct uint2 {
    unsigned x, y;
};
template <int LA, int LB, int LC, int LD> struct EriProg;
#include "eri_prog_all.inc"

static std::vector<double> g_b64;
static std::vector<float> g_b32;

static void init_tables() {
    if (!g_b64.empty()) return;
    g_b64.resize(boys_table_size(BOYS_NT64, BOYS_NGRID64));
    g_b32.resize(boys_table_size(BOYS_NT32, BOYS_NGRID32));
    boys_fill_tables(g_b64.data(), g_b32.data());
}

struct Sh {
    double R[3];
    int n;
    const double *e, *c;  // c already multiplied by N(alpha, l, 0, 0)
};

template <typename R> const R *tab();
template <> const double *tab<double>() { return g_b64.data(); }
template <> const float *tab<float>() { return g_b32.data(); }

template <int LA, int LB, int LC, int LD, typename R>
static void block(const Sh &A, const Sh &B, const Sh &C, const Sh &D, double *res) {
    using K = EriClass<LA, LB, LC, LD>;
    R acc[K::NE * K::NF];
    for (int i = 0; i < K::NE * K::NF; ++i) acc[i] = 0;
    const double cp = std::sqrt(2.0) * std::pow(M_PI, 1.25);
    for (int i = 0; i < A.n; ++i)
        for (int j = 0; j < B.n; ++j) {
            double p = A.e[i] + B.e[j], P[3], r2 = 0;
            for (int d = 0; d < 3; ++d) {
                P[d] = (A.e[i] * A.R[d] + B.e[j] * B.R[d]) / p;
                r2 += (A.R[d] - B.R[d]) * (A.R[d] - B.R[d]);
            }
            double Kab = A.c[i] * B.c[j] * std::exp(-A.e[i] * B.e[j] / p * r2) * cp / p;
            for (int k = 0; k < C.n; ++k)
                for (int l = 0; l < D.n; ++l) {
                    double q = C.e[k] + D.e[l], Q[3], s2 = 0;
                    for (int d = 0; d < 3; ++d) {
                        Q[d] = (C.e[k] * C.R[d] + D.e[l] * D.R[d]) / q;
                        s2 += (C.R[d] - D.R[d]) * (C.R[d] - D.R[d]);
                    }
                    double Kcd = C.c[k] * D.c[l] * std::exp(-C.e[k] * D.e[l] / q * s2) * cp / q;
                    R rp = (R)p, rq = (R)q;
                    R rs = rchem_rsqrt(rp + rq), ipq = rs * rs;
                    R PQ[3] = {(R)P[0] - (R)Q[0], (R)P[1] - (R)Q[1], (R)P[2] - (R)Q[2]};
                    R qi = rq * ipq, pi = rp * ipq;
                    R T = rp * qi * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]);
                    R F[K::L + 1];
                    boys_eval<K::L, R>(T, (R)Kab * (R)Kcd * rs, tab<R>(), F);
                    K::template vrr<R>(acc, F, (R)(P[0] - A.R[0]), (R)(P[1] - A.R[1]), (R)(P[2] - A.R[2]),
                                       -qi * PQ[0], -qi * PQ[1], -qi * PQ[2], (R)(Q[0] - C.R[0]),
                                       (R)(Q[1] - C.R[1]), (R)(Q[2] - C.R[2]), pi * PQ[0], pi * PQ[1], pi * PQ[2],
                                       (R)(0.5 / p), (R)(0.5 / q), R(0.5) * ipq, qi, pi);
                }
        }
    R out[K::NA * K::NB * K::NC * K::ND];
    K::template hrr<R>(acc, out, (R)(A.R[0] - B.R[0]), (R)(A.R[1] - B.R[1]), (R)(A.R[2] - B.R[2]),
                       (R)(C.R[0] - D.R[0]), (R)(C.R[1] - D.R[1]), (R)(C.R[2] - D.R[2]));
    for (int i = 0; i < K::NA * K::NB * K::NC * K::ND; ++i) res[i] = (double)out[i];
}

// The same contracted block, evaluated by running the class's warp-cooperative
// program one term after another (level order is a valid sequential order).
template <int LA, int LB, int LC, int LD>
static void block_prog(const Sh &A, const Sh &B, const Sh &C, const Sh &D, double *res) {
    using K = EriClass<LA, LB, LC, LD>;
    using P = EriProg<LA, LB, LC, LD>;
    // one warp's shared array: accumulators S[0, NT), Boys values at S[NT + m]
    std::vector<double> S(P::SCR, 0.0);
    const double cp = std::sqrt(2.0) * std::pow(M_PI, 1.25);
    for (int i = 0; i < A.n; ++i)
        for (int j = 0; j < B.n; ++j) {
            double p = A.e[i] + B.e[j], Pc[3], r2 = 0;
            for (int d = 0; d < 3; ++d) {
                Pc[d] = (A.e[i] * A.R[d] + B.e[j] * B.R[d]) / p;
                r2 += (A.R[d] - B.R[d]) * (A.R[d] - B.R[d]);
            }
            double Kab = A.c[i] * B.c[j] * std::exp(-A.e[i] * B.e[j] / p * r2) * cp / p;
            for (int k = 0; k < C.n; ++k)
                for (int l = 0; l < D.n; ++l) {
                    double q = C.e[k] + D.e[l], Qc[3], s2 = 0;
                    for (int d = 0; d < 3; ++d) {
                        Qc[d] = (C.e[k] * C.R[d] + D.e[l] * D.R[d]) / q;
                        s2 += (C.R[d] - D.R[d]) * (C.R[d] - D.R[d]);
                    }
                    double Kcd = C.c[k] * D.c[l] * std::exp(-C.e[k] * D.e[l] / q * s2) * cp / q;
                    const double rs = 1.0 / std::sqrt(p + q), ipq = rs * rs;
                    const double PQ[3] = {Pc[0] - Qc[0], Pc[1] - Qc[1], Pc[2] - Qc[2]};
                    const double qi = q * ipq, pi = p * ipq;
                    const double T = p * qi * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]);
                    double F[K::L + 1];
                    boys_eval<K::L, double>(T, Kab * Kcd * rs, g_b64.data(), F);
                    for (int m = 0; m <= K::L; ++m) S[P::NT + m] = F[m];
                    const double PA[3] = {Pc[0] - A.R[0], Pc[1] - A.R[1], Pc[2] - A.R[2]};
                    const double QC[3] = {Qc[0] - C.R[0], Qc[1] - C.R[1], Qc[2] - C.R[2]};
                    const double WP[3] = {-qi * PQ[0], -qi * PQ[1], -qi * PQ[2]};
                    const double WQ[3] = {pi * PQ[0], pi * PQ[1], pi * PQ[2]};
                    const double ohp = 0.5 / p, ohq = 0.5 / q, ohpq = 0.5 * ipq;
                    // each level's terms last to first: the GPU's lanes take them in
                    // any order, so no term may read what another of its level writes
                    for (int lv = 0; lv < P::NVL; ++lv)
                    for (int t = P::vrrlv()[lv + 1] - 1; t >= P::vrrlv()[lv]; --t) {
                        const uint4 op = P::vrr()[t];
                        const int dir = op.w & 3, ket = (op.w >> 2) & 1, n1 = (op.w >> 3) & 7, n2 = (op.w >> 6) & 7;
                        const int tg = (int)(op.w >> 9), dest = (int)(op.x & 0xffff);
                        const double X = ket ? QC[dir] : PA[dir], Y = ket ? WQ[dir] : WP[dir];
                        double v = Y * S[op.y & 0xffff] + X * S[op.x >> 16];
                        if (n1) v += n1 * (ket ? ohq : ohp) * (S[op.y >> 16] - (ket ? pi : qi) * S[op.z & 0xffff]);
                        if (n2) v += n2 * ohpq * S[op.z >> 16];
                        if (dest != 0xffff) S[dest] = v;
                        if (tg) S[tg - 1] += v;
                    }
                }
        }
    const double AB[3] = {A.R[0] - B.R[0], A.R[1] - B.R[1], A.R[2] - B.R[2]};
    const double CD[3] = {C.R[0] - D.R[0], C.R[1] - D.R[1], C.R[2] - D.R[2]};
    for (int lv = 0; lv < P::NHL; ++lv)
    for (int t = P::hrrlv()[lv + 1] - 1; t >= P::hrrlv()[lv]; --t) {
        const uint2 op = P::hrr()[t];
        const int dir = (op.y >> 16) & 255, side = op.y >> 24;
        S[op.x & 0xffff] = S[op.x >> 16] + (side ? CD[dir] : AB[dir]) * S[op.y & 0xffff];
    }
    for (int k = 0; k < P::NOUT; ++k) res[k] = P::onorm()[k] * S[P::out()[k]];
}

template <int LA, int LB, int LC, int LD>
static void blk(int f32, const Sh &A, const Sh &B, const Sh &C, const Sh &D, double *res) {
    if (f32) block<LA, LB, LC, LD, float>(A, B, C, D, res);
    else block<LA, LB, LC, LD, double>(A, B, C, D, res);
}

extern "C" int host_eri_block(int la, int lb, int lc, int ld, int f32, const double *R, const int *n,
                              const double *e, const double *c, double *res) {
    init_tables();
    Sh s[4];
    int off = 0;
    for (int k = 0; k < 4; ++k) {
        for (int d = 0; d < 3; ++d) s[k].R[d] = R[3 * k + d];
        s[k].n = n[k];
        s[k].e = e + off;
        s[k].c = c + off;
        off += n[k];
    }
    const int key = la * 1000 + lb * 100 + lc * 10 + ld;
#define CASE(a, b, c_, d)                                                   \
    case a * 1000 + b * 100 + c_ * 10 + d:                                  \
        blk<a, b, c_, d>(f32, s[0], s[1], s[2], s[3], res);                 \
        return 0;
    switch (key) {
        CASE(0, 0, 0, 0) CASE(1, 0, 0, 0) CASE(1, 0, 1, 0) CASE(1, 1, 0, 0) CASE(1, 1, 1, 0) CASE(1, 1, 1, 1)
        CASE(2, 0, 0, 0) CASE(2, 0, 1, 0) CASE(2, 0, 1, 1) CASE(2, 0, 2, 0) CASE(2, 1, 0, 0) CASE(2, 1, 1, 0)
        CASE(2, 1, 1, 1) CASE(2, 1, 2, 0) CASE(2, 1, 2, 1) CASE(2, 2, 0, 0) CASE(2, 2, 1, 0) CASE(2, 2, 1, 1)
        CASE(2, 2, 2, 0) CASE(2, 2, 2, 1) CASE(2, 2, 2, 2)
    }
    return 1;
}

extern "C" int host_eri_block_prog(int la, int lb, int lc, int ld, const double *R, const int *n, const double *e,
                                   const double *c, double *res) {
    init_tables();
    Sh s[4];
    int off = 0;
    for (int k = 0; k < 4; ++k) {
        for (int d = 0; d < 3; ++d) s[k].R[d] = R[3 * k + d];
        s[k].n = n[k];
        s[k].e = e + off;
        s[k].c = c + off;
        off += n[k];
    }
    const int key = la * 1000 + lb * 100 + lc * 10 + ld;
#define PCASE(a, b, c_, d)                                                  \
    case a * 1000 + b * 100 + c_ * 10 + d:                                  \
        block_prog<a, b, c_, d>(s[0], s[1], s[2], s[3], res);              \
        return 0;
    switch (key) {
        PCASE(1, 1, 1, 1) PCASE(2, 0, 1, 1) PCASE(2, 0, 2, 0) PCASE(2, 1, 1, 0) PCASE(2, 1, 1, 1) PCASE(2, 1, 2, 0)
        PCASE(2, 1, 2, 1) PCASE(2, 2, 0, 0) PCASE(2, 2, 1, 0) PCASE(2, 2, 1, 1) PCASE(2, 2, 2, 0) PCASE(2, 2, 2, 1)
        PCASE(2, 2, 2, 2)
    }
    return 1;
}

extern "C" double host_boys(int m, double x, int f32) {
    init_tables();
    if (f32) {
        float F[BOYS_MMAX + 1];
        boys_eval_rt<float>(m, (float)x, 1.0f, g_b32.data(), F);
        return F[m];
    }
    double F[BOYS_MMAX + 1];
    boys_eval_rt<double>(m, x, 1.0, g_b64.data(), F);
    return F[m];
}
