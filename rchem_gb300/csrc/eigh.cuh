// eigh.cuh -- batched symmetric eigensolver for the small Fock matrices of
// the batched SCF: one thread block per matrix, two-sided cyclic Jacobi in
// FP64 with the matrix and the eigenvectors resident in shared memory.
//
// Each sweep visits every off-diagonal pair (p, q) once, in the round-robin
// ("circle method") order: in round r of m-1 rounds the m/2 disjoint pairs
// rotate at the same time (rows of A, then columns of A and V, one
// __syncthreads between phases).  Rotation as in Rutishauser's Jacobi
// (theta = (a_qq - a_pp) / (2 a_pq), t = sgn(theta) / (|theta| + sqrt(1 + theta^2)),
// c = 1/sqrt(1 + t^2), s = t c), which zeroes a_pq and keeps |phi| <= pi/4.
// Sweeps stop when the off-diagonal Frobenius norm is below 1e-15 of the
// whole matrix's (a fixed maximum of RCHEM_EIGH_MAXSWEEP sweeps bounds the
// loop).  Eigenvalues come out ascending with their eigenvectors as columns,
// as LAPACK's dsyevd returns them.
#pragma once
#include <cuda_runtime.h>

#define RCHEM_EIGH_MAXN 64
#define RCHEM_EIGH_MAXSWEEP 40
#define RCHEM_EIGH_THREADS 256

// One matrix per thread block: A (n x n, row-major, lower triangle read) ->
// w[n] ascending, V[n x n] eigenvectors as columns.  Shared layout: A[n][ld],
// V[n][ld] (ld = n | 1, odd, so column walks do not repeat banks), then the
// m/2 rotations (c, s, p, q) and the reduction slots.
__device__ __forceinline__ void eigh_jacobi_block(int n, const double *__restrict__ Ain, double *__restrict__ w_out,
                                                  double *__restrict__ V_out, double *sm, int *s_done_ptr,
                                                  int *sweeps_out) {
    const int ld = n | 1;
    const int m = n + (n & 1);  // players of the round-robin (one dummy when n is odd)
    const int np = m / 2;
    double *A = sm;
    double *V = A + n * ld;
    double *rc = V + n * ld;      // c[np]
    double *rs = rc + np;         // s[np]
    double *red = rs + np;        // reduction scratch [RCHEM_EIGH_THREADS / 32 * 2]
    int *rp = (int *)(red + 2 * (RCHEM_EIGH_THREADS / 32));  // p[np], q[np]
    int *rq = rp + np;
    int &s_done = *s_done_ptr;
    const int tid = threadIdx.x, nth = blockDim.x;

    // load the lower triangle, mirror it; V = I
    for (int e = tid; e < n * n; e += nth) {
        const int i = e / n, j = e - i * n;
        const double v = i >= j ? Ain[(size_t)i * n + j] : Ain[(size_t)j * n + i];
        A[i * ld + j] = v;
        V[i * ld + j] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();

    int sweep = 0;
    for (; sweep < RCHEM_EIGH_MAXSWEEP; ++sweep) {
        // convergence test: off-diagonal vs total Frobenius norm
        double off = 0.0, tot = 0.0;
        for (int e = tid; e < n * n; e += nth) {
            const int i = e / n, j = e - i * n;
            const double a = A[i * ld + j];
            tot += a * a;
            if (i != j) off += a * a;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        if ((tid & 31) == 0) {
            red[2 * (tid >> 5)] = off;
            red[2 * (tid >> 5) + 1] = tot;
        }
        __syncthreads();
        if (tid == 0) {
            double so = 0.0, st = 0.0;
            for (int k = 0; k < nth / 32; ++k) {
                so += red[2 * k];
                st += red[2 * k + 1];
            }
            s_done = !(so > 1e-30 * st);  // also stops on an all-zero matrix
        }
        __syncthreads();
        if (s_done) break;

        for (int r = 0; r < m - 1; ++r) {
            // rotations of this round
            for (int k = tid; k < np; k += nth) {
                const int a = k == 0 ? 0 : (k - 1 + r) % (m - 1) + 1;
                const int b = (m - 1 - k - 1 + r) % (m - 1) + 1;
                int p = min(a, b), q = max(a, b);
                double c = 1.0, s = 0.0;
                if (q < n) {
                    const double apq = A[p * ld + q];
                    if (apq != 0.0) {
                        const double theta = (A[q * ld + q] - A[p * ld + p]) / (2.0 * apq);
                        double t = 1.0 / (fabs(theta) + hypot(1.0, theta));
                        if (theta < 0.0) t = -t;
                        c = rsqrt(1.0 + t * t);
                        s = t * c;
                    }
                } else {
                    p = q = -1;  // the dummy player's partner sits out
                }
                rc[k] = c;
                rs[k] = s;
                rp[k] = p;
                rq[k] = q;
            }
            __syncthreads();
            // rows: A <- P^T A
            for (int e = tid; e < np * n; e += nth) {
                const int k = e / n, j = e - k * n;
                const int p = rp[k], q = rq[k];
                if (p < 0) continue;
                const double c = rc[k], s = rs[k];
                const double ap = A[p * ld + j], aq = A[q * ld + j];
                A[p * ld + j] = c * ap - s * aq;
                A[q * ld + j] = s * ap + c * aq;
            }
            __syncthreads();
            // columns: A <- A P, V <- V P
            for (int e = tid; e < np * n; e += nth) {
                const int k = e / n, i = e - k * n;
                const int p = rp[k], q = rq[k];
                if (p < 0) continue;
                const double c = rc[k], s = rs[k];
                const double ap = A[i * ld + p], aq = A[i * ld + q];
                // the rotation annihilates a_pq: store the exact zero, not its rounding
                A[i * ld + p] = i == q ? 0.0 : c * ap - s * aq;
                A[i * ld + q] = i == p ? 0.0 : s * ap + c * aq;
                const double vp = V[i * ld + p], vq = V[i * ld + q];
                V[i * ld + p] = c * vp - s * vq;
                V[i * ld + q] = s * vp + c * vq;
            }
            __syncthreads();
        }
    }
    // ascending order: each eigenvalue's rank among the diagonal
    for (int i = tid; i < n; i += nth) {
        const double wi = A[i * ld + i];
        int rank = 0;
        for (int j = 0; j < n; ++j) {
            const double wj = A[j * ld + j];
            rank += (wj < wi) || (wj == wi && j < i);
        }
        w_out[rank] = wi;
        for (int row = 0; row < n; ++row) V_out[(size_t)row * n + rank] = V[row * ld + i];
    }
    if (sweeps_out && tid == 0) *sweeps_out = sweep;
}

__global__ void __launch_bounds__(RCHEM_EIGH_THREADS) k_eigh_jacobi(int n, const double *__restrict__ Ain,
                                                                     double *__restrict__ w_out,
                                                                     double *__restrict__ V_out, int *sweeps_out) {
    extern __shared__ double sm[];
    __shared__ int s_done;
    const size_t base = (size_t)blockIdx.x * n * n;
    eigh_jacobi_block(n, Ain + base, w_out + (size_t)blockIdx.x * n, V_out + base, sm, &s_done,
                      sweeps_out ? sweeps_out + blockIdx.x : nullptr);
}

inline size_t eigh_smem_bytes(int n) {
    const int ld = n | 1, m = n + (n & 1), np = m / 2;
    return (size_t)(2 * n * ld + 2 * np + 2 * (RCHEM_EIGH_THREADS / 32)) * sizeof(double) + 2 * np * sizeof(int);
}
