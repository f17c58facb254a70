// rchem_types.h -- device data layout shared by the host planner and the kernels.
//
// A basis lives on the GPU as shells (pure l, reference AO order), shell pairs
// and primitive pairs.  Everything the inner ERI loop reads per primitive
// quartet is precomputed per primitive pair (product centre, P-A, 1/(2p), the
// contraction/normalisation/Gaussian-product prefactor), so the loop itself
// does no divisions and no exponentials.
#pragma once

#ifdef __CUDACC__
#define RCHEM_HD __host__ __device__
#else
#define RCHEM_HD
#endif

#ifndef __CUDACC__
struct float2;  // host-only compiles see the device argument block by pointer only
struct double2;
struct float4;
#endif

#define RCHEM_LMAX 2          // s, p, d shells (Cartesian)
#define RCHEM_MAX_NCART 6

// One primitive pair (alpha_a on shell A, alpha_b on shell B), 80 bytes.
struct PairPrim {
    double p;      // alpha_a + alpha_b
    double ohp;    // 1/(2p)
    double P[3];   // (alpha_a A + alpha_b B)/p
    double PA[3];  // P - A
    double K;      // c_a c_b N_a N_b exp(-alpha_a alpha_b |AB|^2 / p) * sqrt(2) pi^(5/4) / p
    double pad;
};

// The same in single precision, for the FP32 part of the mixed form, 48 bytes.
struct PairPrim32 {
    float p, ohp, P[3], PA[3], K, pad[3];
};

// One shell pair (A,B) with l_A >= l_B, 80 bytes.
struct ShellPair {
    int A, B;        // shell indices
    int aoA, aoB;    // first basis function of A and of B
    int prim0, npp;  // primitive pairs [prim0, prim0 + npp)
    int group, diag; // pair group; 1 if A == B
    double AB[3];    // A - B
    double Q;        // Schwarz bound sqrt(max |(ab|ab)|) over the pair's functions
    float AB32[3];   // A - B in single precision (the high words of the double-float form)
    int la_lb;       // 10*l_A + l_B
    int moff, mn;    // the pair's geometry: offset of its n x n block in the packed matrices, n
    float ABlo[3];   // low words: AB32 + ABlo = A - B to ~48 bits
    int pad2;
};

// The same as PairPrim, each value an unevaluated float pair (hi, lo), for the
// emulated-FP64 (double-float) form; 80 bytes.
struct PairPrimDF {
    float p[2], ohp[2], P[3][2], PA[3][2], K[2], pad[2];
};

// One geometry of a (possibly batched) basis: its block of the packed
// matrices, its first basis function and its atoms.
struct GeomDev {
    int moff, n, ao0, atom0, natoms, pad;
};

// A run of quartets sharing one bra pair: (bra | ket0 .. ket0+count-1), kets
// taken consecutively from one pair group.
struct EriSeg {
    int bra, ket0, count, pad;
};

// One warp of work: up to 32/G consecutive quartets of a chain of segments of
// one (bra group, ket group) combination, so every lane runs the same
// primitive-loop trip counts.  G = 2^lg lanes share one quartet (they split its
// primitive quartets and reduce the contraction accumulators with warp
// shuffles).  Lane l takes quartet off + l/G counted from the start of
// segment seg.  nq_lg = nq | (lg << 8).
struct EriTask {
    int seg, off, nq_lg, cost;
};

// Arguments of every ERI class kernel.
struct EriArgs {
    const EriTask *tasks;
    const EriSeg *segs;
    int ntasks;
    int nbf;
    const ShellPair *pairs;
    const PairPrim *prims;
    const PairPrim32 *prims32;
    const double *boys64;  // Boys Taylor tables (boys.cuh layout)
    const double *boysfar; // and the FP64 power-law table beyond them (boys_eval_u)
    const float *boys32;
    const double *D;       // density, nbf x nbf row-major
    const float *D32;      // the same in single precision (mixed form)
    const PairPrimDF *primsdf;  // double-float forms (emulated FP64)
    const float2 *boysdf;
    const float2 *Ddf;
    double *J;             // unsymmetrised accumulators (J-hat, K-hat)
    double *K;
    double *eri;           // ERI-tensor epilogue output: dense nbf^4, or packed (eri_packed)
    int eri_packed;        // 1: one value per unique integral at the 8-fold index (rchem_eri_pack8)
    int wc;                // J/K epilogue of a large class: the warp-cooperative kernel with 32, 16 or 8
                           // lanes per quartet, 0 = one lane group per quartet
    int f32_boys64;        // FP32 quartets' Boys function: 0 FP32, 1 FP64 (values and recursion),
                           // 2 FP32 table / asymptotic values with the recursion in FP64
    // per (bra, ket) primitive-pair exponent: 1/sqrt(p+q), pq/(p+q), q/(p+q),
    // p/(p+q) from a table (FP64 and double-float kernels); npq = 0: computed
    int npq;               // distinct primitive-pair exponents p (table side)
    const int *prim_eid;   // per primitive pair: index of its p among them
    const double2 *pq64;   // entry (i, j) at 2 (i npq + j): {rs, rho}, {q/(p+q), p/(p+q)}
    const float4 *pqdf;    // the same as (hi, lo) float pairs
};

// Shell as the planner sees it.
struct ShellInfo {
    int atom, l, nprim, prim0, ao;
    double R[3];
};
