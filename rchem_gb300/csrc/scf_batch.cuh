// scf_batch.cuh -- kernels of the native RHF driver (rchem_rhf): every
// geometry of a handle at once, all matrices in the packed layout (geometry g's
// n_g x n_g block at GeomDev::moff), one thread block per geometry.
//
// The loop follows the reference's SCF (src/bin/rchem.rs:40-127): symmetric
// orthogonalisation X = U diag(lambda^-1/2) U^T, core-Hamiltonian guess,
// D = C_occ C_occ^T without the factor 2, F = H + 2J - K, E = sum (H + F) o D;
// with Pulay DIIS on the orthogonalised commutator X^T (FDS - SDF) X added.
// Diagonalisations use the Jacobi solver of eigh.cuh, so n_g <= 64.
#pragma once
#include "eigh.cuh"
#include "rchem_types.h"

#define RCHEM_SCF_THREADS 256
#define RCHEM_DIIS_MAX 8

// The loop's state on the device, so that one captured iteration serves every
// iteration: the DIIS ring position and length, the iteration count and the
// stop decision (taken on the device by k_scf_check).
struct ScfState {
    int it;         // iterations completed
    int nstored;    // Fock/error pairs held in the DIIS ring
    int newest;     // ring slot of this iteration's pair
    int converged;  // 1 once every geometry met the thresholds
    int stop;       // 1 once converged or at the iteration cap
    int pad[3];
};

// C = alpha op(A) op(B) + beta C for every geometry (op = transpose if tA/tB);
// A, B, C packed.  n <= 64: operands are read through L1, no tiling needed.
// With st, C is the DIIS ring slot st->newest of a ring of stride `slot`.
__global__ void __launch_bounds__(RCHEM_SCF_THREADS)
    k_scf_gemm(const GeomDev *geo, const double *A, int tA, const double *B, int tB, double *C, double alpha,
               double beta, const ScfState *st = nullptr, long long slot = 0) {
    const GeomDev g = geo[blockIdx.x];
    const int n = g.n;
    const double *a = A + g.moff, *b = B + g.moff;
    double *c = C + g.moff + (st ? (long long)st->newest * slot : 0);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        double s = 0.0;
        for (int k = 0; k < n; ++k) s = fma(tA ? a[k * n + i] : a[i * n + k], tB ? b[j * n + k] : b[k * n + j], s);
        c[e] = beta == 0.0 ? alpha * s : fma(beta, c[e], alpha * s);
    }
}

// F = H + 2 J - K
__global__ void k_scf_fock(long long packed, const double *H, const double *J, const double *K, double *F) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < packed) F[i] = H[i] + 2.0 * J[i] - K[i];
}

// block sum of one value per thread (all threads of the block must call it)
__device__ __forceinline__ double scf_block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    return s;
}

// e[g] = sum (H + F) o D over geometry g's block; dmax[g] = max |D - Dold|
__global__ void __launch_bounds__(RCHEM_SCF_THREADS)
    k_scf_energy(const GeomDev *geo, const double *H, const double *F, const double *D, const double *Dold,
                 double *e, double *dmax) {
    __shared__ double red[RCHEM_SCF_THREADS / 32];
    const GeomDev g = geo[blockIdx.x];
    double s = 0.0, m = 0.0;
    for (int i = threadIdx.x; i < g.n * g.n; i += blockDim.x) {
        const long long k = g.moff + i;
        s = fma(H[k] + F[k], D[k], s);
        if (Dold) m = fmax(m, fabs(D[k] - Dold[k]));
    }
    const double tot = scf_block_sum(s, red);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mm = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) mm = fmax(mm, red[k]);
        e[blockIdx.x] = tot;
        dmax[blockIdx.x] = mm;
    }
}

// C = T - T^T (the commutator FDS - SDF from T = FDS, F, D, S symmetric)
__global__ void k_scf_antisym(const GeomDev *geo, const double *T, double *C) {
    const GeomDev g = geo[blockIdx.x];
    const int n = g.n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        C[g.moff + e] = T[g.moff + e] - T[g.moff + j * n + i];
    }
}

// This iteration's DIIS ring slot (one thread).
__global__ void k_scf_diis_slot(ScfState *st, int diis) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->newest = st->it % diis;
        st->nstored = min(st->nstored + 1, diis);
    }
}

// F into the DIIS ring slot st->newest (stride `packed`)
__global__ void k_scf_store_slot(const GeomDev *geo, const double *F, double *Fh, long long packed,
                                 const ScfState *st) {
    const GeomDev g = geo[blockIdx.x];
    double *dst = Fh + (long long)st->newest * packed + g.moff;
    for (int e = threadIdx.x; e < g.n * g.n; e += blockDim.x) dst[e] = F[g.moff + e];
}

// B = A over every geometry's block
__global__ void k_scf_copy(const GeomDev *geo, const double *A, double *B) {
    const GeomDev g = geo[blockIdx.x];
    for (int e = threadIdx.x; e < g.n * g.n; e += blockDim.x) B[g.moff + e] = A[g.moff + e];
}

// DIIS: B_ij = <e_i, e_j> over the m = st->nstored stored error matrices
// (slots of the ring buffers, stride `packed`), then the (m+1) x (m+1) Pulay
// system solved by Gaussian elimination with partial pivoting (one thread); a
// singular system keeps the newest Fock matrix.  coef[g][0..m) receives the
// coefficients in slot order.  Nothing to do before two pairs are stored.
__global__ void __launch_bounds__(RCHEM_SCF_THREADS)
    k_scf_diis(const GeomDev *geo, const double *E, long long packed, const ScfState *st, double *coef) {
    __shared__ double red[RCHEM_SCF_THREADS / 32];
    __shared__ double Bm[RCHEM_DIIS_MAX + 1][RCHEM_DIIS_MAX + 2];
    const int m = st->nstored;
    if (m < 2) return;  // block-uniform
    const GeomDev g = geo[blockIdx.x];
    const int nn = g.n * g.n;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = 0.0;
            for (int k = threadIdx.x; k < nn; k += blockDim.x)
                s = fma(E[i * packed + g.moff + k], E[j * packed + g.moff + k], s);
            const double t = scf_block_sum(s, red);
            if (threadIdx.x == 0) Bm[i][j] = Bm[j][i] = t;
        }
    if (threadIdx.x != 0) return;
    // augmented system [B -1; -1 0] c = [0; -1], right-hand side in column m+1
    for (int i = 0; i < m; ++i) {
        Bm[i][m] = -1.0;
        Bm[m][i] = -1.0;
        Bm[i][m + 1] = 0.0;
    }
    Bm[m][m] = 0.0;
    Bm[m][m + 1] = -1.0;
    const int dim = m + 1;
    bool ok = true;
    for (int c = 0; c < dim && ok; ++c) {
        int piv = c;
        for (int r = c + 1; r < dim; ++r)
            if (fabs(Bm[r][c]) > fabs(Bm[piv][c])) piv = r;
        if (!(fabs(Bm[piv][c]) > 1e-300)) {
            ok = false;
            break;
        }
        if (piv != c)
            for (int k = 0; k <= dim; ++k) {
                const double t = Bm[c][k];
                Bm[c][k] = Bm[piv][k];
                Bm[piv][k] = t;
            }
        for (int r = 0; r < dim; ++r) {
            if (r == c) continue;
            const double f = Bm[r][c] / Bm[c][c];
            for (int k = c; k <= dim; ++k) Bm[r][k] -= f * Bm[c][k];
        }
    }
    double *cg = coef + (size_t)blockIdx.x * RCHEM_DIIS_MAX;
    for (int i = 0; i < m; ++i) {
        const double v = ok ? Bm[i][dim] / Bm[i][i] : 0.0;
        cg[i] = isfinite(v) ? v : 0.0;
        if (!ok || !isfinite(v)) ok = false;
    }
    if (!ok)  // keep the newest Fock matrix
        for (int i = 0; i < m; ++i) cg[i] = 0.0;
    (void)ok;
}

// Fx = sum_i coef[g][i] F_i (ring buffer slots), or F_newest when every
// coefficient is zero (a singular DIIS system) or fewer than two pairs are stored
__global__ void __launch_bounds__(RCHEM_SCF_THREADS)
    k_scf_extrapolate(const GeomDev *geo, const double *Fh, long long packed, const ScfState *st, const double *coef,
                      double *Fx) {
    const GeomDev g = geo[blockIdx.x];
    const int m = st->nstored, newest = st->newest;
    const double *cg = coef + (size_t)blockIdx.x * RCHEM_DIIS_MAX;
    bool any = false;
    if (m >= 2)
        for (int i = 0; i < m; ++i) any |= cg[i] != 0.0;
    for (int k = threadIdx.x; k < g.n * g.n; k += blockDim.x) {
        const long long o = g.moff + k;
        double s = 0.0;
        if (any)
            for (int i = 0; i < m; ++i) s = fma(cg[i], Fh[i * packed + o], s);
        else
            s = Fh[newest * packed + o];
        Fx[o] = s;
    }
}

// eigenvalues (w, at the same packed offsets as the matrices' first rows:
// w[moff + i]) and eigenvectors of every geometry's block
__global__ void __launch_bounds__(RCHEM_EIGH_THREADS)
    k_scf_eigh(const GeomDev *geo, const double *A, double *w, double *V) {
    extern __shared__ double sm[];
    __shared__ int s_done;
    const GeomDev g = geo[blockIdx.x];
    eigh_jacobi_block(g.n, A + g.moff, w + g.moff, V + g.moff, sm, &s_done, nullptr);
}

// X = U diag(lambda^-1/2) U^T from the eigenpairs of S
__global__ void k_scf_invsqrt(const GeomDev *geo, const double *w, const double *U, double *X) {
    const GeomDev g = geo[blockIdx.x];
    const int n = g.n;
    const double *u = U + g.moff;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        double s = 0.0;
        for (int k = 0; k < n; ++k) s = fma(u[i * n + k] * rsqrt(w[g.moff + k]), u[j * n + k], s);
        X[g.moff + e] = s;
    }
}

// D = C_occ C_occ^T and W = sum_i eps_i C_i C_i^T over the nocc[g] lowest orbitals
__global__ void k_scf_density(const GeomDev *geo, const int *nocc, const double *C, const double *eps, double *D,
                              double *W) {
    const GeomDev g = geo[blockIdx.x];
    const int n = g.n, no = nocc[blockIdx.x];
    const double *c = C + g.moff;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        double d = 0.0, wv = 0.0;
        for (int k = 0; k < no; ++k) {
            const double cc = c[i * n + k] * c[j * n + k];
            d += cc;
            if (W) wv = fma(eps[g.moff + k], cc, wv);
        }
        D[g.moff + e] = d;
        if (W) W[g.moff + e] = wv;
    }
}

// End of an iteration (one block): this iteration's energies e against the
// previous ones and the density change dm against the thresholds, as the
// host-side loop tests them (no test on the first iteration); eprev = e; the
// iteration count; the stop decision (converged, or the iteration cap).  In a
// graph with a WHILE node, the loop continues while the node's condition is
// non-zero: the decision goes there too (use_handle), so the loop always ends
// by max_iter.
__global__ void __launch_bounds__(RCHEM_SCF_THREADS)
    k_scf_check(ScfState *st, int ng, const double *e, double *eprev, const double *dm, double thresh_e,
                double thresh_d, int max_iter, cudaGraphConditionalHandle h, int use_handle) {
    __shared__ double red[RCHEM_SCF_THREADS / 32];
    int ok = 1;
    double m = 0.0;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        ok &= fabs(e[g] - eprev[g]) < thresh_e ? 1 : 0;
        m = fmax(m, dm[g]);
    }
    ok = __syncthreads_and(ok);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    for (int g = threadIdx.x; g < ng; g += blockDim.x) eprev[g] = e[g];
    if (threadIdx.x == 0) {
        double mm = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) mm = fmax(mm, red[k]);
        const int it = st->it + 1;
        const int conv = (it > 1 && ok && mm < thresh_d) ? 1 : 0;
        st->it = it;
        st->converged = conv;
        st->stop = (conv || it >= max_iter) ? 1 : 0;
        if (use_handle) cudaGraphSetConditional(h, st->stop ? 0u : 1u);
    }
}
