/*
 * rchem_gpu.h -- C ABI of librchem_gpu.so, the GB300 (sm_103a) implementation
 * of rchem's restricted Hartree-Fock hot path: contracted-Gaussian ERIs, the
 * Boys function, the one-electron integrals and the direct-SCF Fock build.
 *
 * Plain C types only.  Matrices are row-major FP64, n x n, in the reference's
 * AO order (atoms in order, shells in basis-file order, each angular momentum
 * of a shell in order, Cartesian components in src/shell.rs:1-12 order),
 * coordinates in bohr.  Every array argument lives where the accompanying
 * `where` / opts->where says (RCHEM_HOST or RCHEM_DEVICE).  Calls are
 * asynchronous on the basis handle's stream and synchronise before returning.
 *
 * Errors: every entry returns an int status (RCHEM_OK = 0); rchem_last_error()
 * gives the message of the calling thread's last failure.  Nothing exits the
 * process or prints.  (The reference panics through unwrap()/assert!, e.g.
 * src/basis.rs:89-105,163,191.)
 *
 * Threading: a handle is used by one host thread at a time.
 */
#ifndef RCHEM_GPU_H
#define RCHEM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    RCHEM_OK = 0,
    RCHEM_ERR_INVALID = 1,     /* bad argument (null pointer, size, non-finite value) */
    RCHEM_ERR_UNSUPPORTED = 2, /* l > 2 on a shell, too many primitives, ... */
    RCHEM_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    RCHEM_ERR_NOMEM = 4        /* device or host allocation failed */
};

enum { RCHEM_HOST = 0, RCHEM_DEVICE = 1 };

#define RCHEM_MAX_L 2      /* Cartesian s, p, d shells */
#define RCHEM_MAX_NPRIM 16 /* primitives per shell */

typedef struct rchem_basis_s *rchem_basis;

/* Message of the calling thread's last error ("" if none). */
const char *rchem_last_error(void);
/* ABI version, currently 1. */
int rchem_abi_version(void);

/*
 * Basis::new (src/basis.rs:181-211).  The reference fetches the basis through
 * embedded Python (src/basis.rs:87-106); here the caller passes the shells,
 * already expanded to pure angular momenta in AO order: a combined sp shell is
 * its s shell followed by its p shell with the same exponents.
 *   atomnos[natoms], coords[3*natoms] (bohr)
 *   shell_atom[nshells], shell_l[nshells] (0..2), shell_nprim[nshells]
 *   exps[], coefs[]: the shells' primitives back to back (raw basis-file
 *   contraction coefficients; the primitive normalisation of basis.rs:140-149
 *   is applied here, the contraction is not renormalised, as in the reference).
 * All arrays are host arrays.  The handle owns its own CUDA stream.
 */
int rchem_basis_create(rchem_basis *out, int natoms, const int *atomnos, const double *coords, int nshells,
                       const int *shell_atom, const int *shell_l, const int *shell_nprim, const double *exps,
                       const double *coefs);
/*
 * Many geometries in one handle (no counterpart in the reference, which builds
 * one molecule at a time): every Fock build, S/T/V and gradient call then
 * covers all of them in one set of kernel launches.  Geometry g owns the next
 * geom_natoms[g] atoms of atomnos/coords; shell_atom indexes the concatenated
 * atoms and the shells must come in geometry order.  Matrices are packed:
 * geometry g's n_g x n_g block (row-major) starts at element geom_offset[g]
 * (rchem_basis_layout); blocks never couple.
 */
int rchem_batch_create(rchem_basis *out, int ngeom, const int *geom_natoms, int natoms, const int *atomnos,
                       const double *coords, int nshells, const int *shell_atom, const int *shell_l,
                       const int *shell_nprim, const double *exps, const double *coefs);
/* Number of geometries, total packed matrix elements, and per geometry (arrays
 * of ngeom, may be NULL) its basis size and block offset. */
int rchem_basis_layout(rchem_basis b, int *ngeom, long long *packed, int *geom_nbf, long long *geom_offset);
int rchem_basis_destroy(rchem_basis b);
/* Number of contracted Cartesian functions (the reference's cgtos.len());
 * summed over the geometries of a batched handle. */
int rchem_basis_nbf(rchem_basis b);
/* Use the caller's CUDA stream (a cudaStream_t) instead of the handle's own. */
int rchem_basis_set_stream(rchem_basis b, void *stream);

/* S, T and V matrices: basis::S / T / V, src/basis.rs:234,273,316.
 * V = sum_C Z_C V_C over the handle's atoms. */
int rchem_S(rchem_basis b, double *out, int where);
int rchem_T(rchem_basis b, double *out, int where);
int rchem_V(rchem_basis b, double *out, int where);
/* Multipole-moment matrix <mu|(x-Cx)^ox (y-Cy)^oy (z-Cz)^oz|nu>, the integral of
 * src/integrals/os86.rs:775-828, normalised like S.  center: 3 host doubles. */
int rchem_moment(rchem_basis b, const double *center, int ox, int oy, int oz, double *out, int where);

/* Arithmetic flags of rchem_jk_opts.emulated (combinable). */
#define RCHEM_JK_EMULATED 1    /* the FP64 quartets in double-float arithmetic on the FP32 pipe */
#define RCHEM_JK_FP32_BOYS64 2 /* the FP32 quartets (below fp32_tau) evaluate the Boys function and its
                                  downward recursion in FP64, from their FP32 argument and prefactor */
#define RCHEM_JK_FP32_REC64 4  /* the FP32 quartets evaluate the Boys function's table (or asymptotic)
                                  values in FP32 and its recursion in FP64; with RCHEM_JK_FP32_BOYS64:
                                  RCHEM_ERR_INVALID */

/* Fock-build options.  Zero-initialised options mean: FP64 everywhere,
 * Schwarz threshold 1e-12, host arrays. */
typedef struct {
    double schwarz_tau; /* drop quartets with Q_ab Q_cd < tau (0 => 1e-12; <0 => no screening) */
    double fp32_tau;    /* quartets with Q_ab Q_cd < fp32_tau in FP32, FP64 accumulation (0 => FP64 only) */
    int where;          /* RCHEM_HOST or RCHEM_DEVICE for D, J, K */
    int emulated;       /* flags; 0: native FP64 above fp32_tau, FP32 Boys function below.
                           RCHEM_JK_EMULATED: the FP64 quartets in double-float arithmetic
                           (~48-bit significand): every class with l_a+l_b+l_c+l_d <= 4, and
                           the larger classes whose list runs the warp-cooperative kernel
                           (rchem_autotune's choice); the others stay FP64.
                           RCHEM_JK_FP32_BOYS64, RCHEM_JK_FP32_REC64: see above.  Other bits:
                           RCHEM_ERR_INVALID */
} rchem_jk_opts;

/* Work done by the last Fock build of a handle. */
typedef struct {
    long long quartets_fp64, quartets_fp32; /* contracted shell quartets computed */
    long long prim_quartets_fp64, prim_quartets_fp32;
    long long eris_fp64, eris_fp32;         /* contracted Cartesian integrals computed (unique, 8-fold) */
    double flops_fp64, flops_fp32;          /* algorithmic FLOPs (generated op counts) */
    long long warp_tasks;                   /* warps launched */
    int kernels;                            /* class kernels launched */
    int reserved;
    double gpu_ms;                          /* device time of the last rchem_jk_direct (CUDA events on its
                                               stream, from the copy of D in to the copies of J and K out) */
} rchem_jk_stats;

/*
 * JK_direct (src/basis.rs:383-428): J_mn = sum_ls (mn|ls) D_ls,
 * K_mn = sum_ls (ml|ns) D_ls, for a symmetric density D.  J and K are
 * overwritten (the reference zero-fills them first, basis.rs:389-390).
 * Each unique quartet is computed once (8-fold symmetry), Schwarz-screened.
 */
int rchem_jk_direct(rchem_basis b, const double *D, double *J, double *K, const rchem_jk_opts *opts);
int rchem_jk_stats_get(rchem_basis b, rchem_jk_stats *out);
/*
 * One share of a Fock build, for splitting a single large system over
 * nparts processes (one GPU each; no counterpart in the reference, whose
 * JK_direct, src/basis.rs:383-428, is one serial loop nest): the bra shell
 * pairs are split into nparts shares of about equal cost (longest-processing-
 * time assignment of each pair's surviving quartets, deterministic, so every
 * process computes the same split), and this call computes J and K from the
 * quartets whose bra pair is in share `part` only -- symmetrised like a whole
 * build, so the element-wise sum of the nparts results is rchem_jk_direct's J
 * and K (one sum all-reduce of 2 n^2 doubles).  0 <= part < nparts; nparts = 1
 * is the whole build.  Same options, arrays and errors as rchem_jk_direct;
 * the handle replans (and re-captures its graph) when the share changes.
 */
int rchem_jk_direct_part(rchem_basis b, const double *D, double *J, double *K, const rchem_jk_opts *opts, int part,
                         int nparts);
/* Per integral class (21 classes, arrays of 21*4 / 21*2 entries, any may be
 * NULL) of the current work plan: the class (l_a,l_b,l_c,l_d), and for {FP64,
 * FP32} the shell quartets, primitive quartets and algorithmic FLOPs. */
int rchem_jk_class_stats(rchem_basis b, int *class_l, long long *quartets, long long *prim_quartets, double *flops);
/* Device time of every class list of the Fock build planned for these
 * options, each list launched alone on the handle's stream (one warm-up launch,
 * then one launch between CUDA events), J/K epilogue, the density of the last
 * Fock build (zeros before the first): ms[2*21] in the order of
 * rchem_jk_class_stats, 0 for an empty list.  No counterpart in the
 * reference; with rchem_jk_class_stats' FLOPs it gives each kernel's rate.
 * J-hat/K-hat scratch is overwritten; the next rchem_jk_direct clears it. */
int rchem_jk_list_times(rchem_basis b, const rchem_jk_opts *opts, float *ms);

/*
 * The Fock build of rchem_jk_direct without any device allocation (this entry
 * point has no counterpart in the reference, which runs on the CPU).  It is
 * for callers that cannot allocate GPU memory where they need the build:
 * programs whose device memory is owned by an external pooled allocator that
 * forbids cudaMalloc after start-up, or long-running services whose
 * steady-state loop must never allocate.
 *  - D, J and K are device arrays (opts->where must be RCHEM_DEVICE); opts is
 *    required.  Results equal rchem_jk_direct's up to summation order.
 *    opts->emulated is not honoured: quartets above fp32_tau always run in
 *    native FP64 here.
 *  - The scratch (J-hat, K-hat, the FP32 copy of D) is a static device array
 *    inside the library sized for at most 640 basis functions (about 8 MiB,
 *    held by every GPU that loads the library until the process exits);
 *    larger bases get RCHEM_ERR_UNSUPPORTED.
 *  - The basis must already be planned for the same thresholds: call
 *    rchem_jk_direct once with the same options first (planning may allocate).
 *  - The handle's device must be the current device (RCHEM_ERR_INVALID
 *    otherwise).  The first call on a device looks up the array's device
 *    address; make that first call before any stream capture.
 *  - Like rchem_jk_direct, the call is synchronous: it returns once J and K
 *    are written.
 *  - Every call on a device shares the one array: calls whose GPU work
 *    overlaps (different threads, streams or handles at the same time) race.
 *    Each call clears the accumulators it uses.
 */
int rchem_jk_direct_noalloc(rchem_basis b, const double *D, double *J, double *K, const rchem_jk_opts *opts);

/*
 * Nuclear gradient dE/dR (hartree/bohr, grad[3*natoms]) of the RHF energy the
 * reference computes, E = sum (H + F) o D + E_nuc (src/bin/rchem.rs:106-108,
 * plus the nuclear repulsion it does not print), at a converged density
 * D = C_occ C_occ^T and energy-weighted density W = sum_i eps_i C_i C_i^T
 * (both without the factor 2, as in src/bin/rchem.rs:101-104).  Adjoint
 * kernels: derivative ERIs contracted on the fly with the density products,
 * derivative S/T/V contracted with W and D, Hellmann-Feynman term included.
 * No counterpart in the reference, which has no gradients.  opts: schwarz_tau,
 * where (for D, W and grad), fp32_tau (quartets with Q_ab Q_cd below it in
 * FP32, the rest FP64) and emulated (the FP64 quartets of the s/p classes up to
 * (pp|ps) in double-float arithmetic on the FP32 pipe; (pp|pp) and the classes
 * with a d shell stay FP64).
 */
int rchem_gradient(rchem_basis b, const double *D, const double *W, double *grad, const rchem_jk_opts *opts);

/*
 * Batched symmetric eigensolver for the batched SCF (no counterpart in the
 * reference, whose SCF diagonalises one matrix at a time through
 * ndarray-linalg's eigh, src/bin/rchem.rs:44,75): A[batch][n][n] (the lower
 * triangle is read) -> w[batch][n] ascending and V[batch][n][n] with the
 * eigenvectors as columns (row-major: V[b][i][k] is component i of vector k),
 * the layout LAPACK dsyevd returns.  One thread block per matrix, cyclic
 * Jacobi in FP64 in shared memory.  n <= 64 (RCHEM_ERR_UNSUPPORTED above).
 * Device arrays only; queued on `stream` (a cudaStream_t; NULL = the legacy
 * default stream) without synchronising.
 */
int rchem_eigh_batched(int n, int batch, const double *A, double *w, double *V, void *stream);

/*
 * Restricted Hartree-Fock for every geometry of a handle at once, entirely on
 * the GPU (no counterpart in the reference's C layer: it is the SCF loop of
 * src/bin/rchem.rs:40-127 -- symmetric orthogonalisation, core-Hamiltonian
 * guess, D = C_occ C_occ^T without the factor 2, F = H + 2J - K,
 * E = sum (H + F) o D -- with Pulay DIIS on X^T (FDS - SDF) X added).  All
 * geometries iterate together until every energy changes by less than
 * thresh_e and the density by less than thresh_d.  Diagonalisations use the
 * batched Jacobi solver: every geometry must have n <= 64 basis functions
 * (RCHEM_ERR_UNSUPPORTED otherwise; the Python driver rchem_gb300.scf covers
 * larger single geometries).
 *   opts      thresholds, iteration cap, DIIS length (0..8) and the Fock-build
 *             options (jk.schwarz_tau, jk.fp32_tau, jk.emulated; jk.where
 *             says where D_out / W_out live); NULL = defaults
 *             (1e-10, 1e-7, 128, 8, FP64, host)
 *   nocc      doubly occupied orbitals per geometry (NULL: half the electrons)
 *   e_elec, e_nuc   host arrays[ngeom] (may be NULL): E_elec as the reference
 *             prints it and the nuclear repulsion
 *   D_out, W_out    packed density and energy-weighted density (may be NULL),
 *             the inputs of rchem_gradient
 */
typedef struct {
    double thresh_e;   /* |Delta E| per geometry between iterations */
    double thresh_d;   /* max |Delta D| */
    int max_iter;
    int diis;          /* DIIS history length, 0 = plain Roothaan iterations */
    rchem_jk_opts jk;
} rchem_scf_opts;
int rchem_rhf(rchem_basis b, const rchem_scf_opts *opts, const int *nocc, double *e_elec, double *e_nuc,
              double *D_out, double *W_out, int *iterations, int *converged);

/*
 * Autotune the Fock build's tile shapes for this basis and these thresholds
 * (no counterpart in the reference): for every integral class list (21
 * classes x {FP64, FP32}) time the list alone under each candidate number of
 * lanes per shell quartet, and for the classes with l_a+l_b+l_c+l_d >= 4 also
 * the warp-cooperative kernel (32, 16 or 8 lanes per quartet, so 1, 2 or 4
 * quartets per warp, intermediates in shared memory), and keep the fastest;
 * then, since the lists run concurrently in a build, settle each list of those
 * classes (longest first) on the shape that gives the fastest whole build.
 * chosen (may be NULL) receives 2*21 ints: the minimum primitive quartets per
 * lane picked for each list (2^30 = never split), or 0, -16, -8 for the
 * warp-cooperative kernel with 32, 16, 8 lanes per quartet.  Later
 * rchem_jk_direct calls use the choices.
 */
int rchem_autotune(rchem_basis b, const rchem_jk_opts *opts, int *chosen);

/*
 * Set one class list's tile shape by hand (no counterpart in the reference;
 * overrides rchem_autotune for that list): class index cls 0..20 in the order
 * of the generated class table (s,p,d pairs with l_a >= l_b), prec 0 = FP64 /
 * emulated list, 1 = FP32 list; ppl = minimum primitive quartets per lane, or
 * 0, -16, -8 for the warp-cooperative kernel with 32, 16, 8 lanes per quartet
 * (classes with l_a+l_b+l_c+l_d >= 4 only, else RCHEM_ERR_UNSUPPORTED; other
 * negative values RCHEM_ERR_INVALID).  The next Fock build replans.
 */
int rchem_set_tile_shape(rchem_basis b, int cls, int prec, int ppl);

/*
 * The factors of a primitive quartet that depend only on its two exponent sums
 * p and q (1/sqrt(p+q), pq/(p+q), q/(p+q), p/(p+q)) come from a table built at
 * rchem_basis_create over the basis's distinct p (up to 1024 of them), or, with
 * on = 0, are computed in every primitive quartet (no counterpart in the
 * reference; the same integrals to rounding).  Default on; on = 1 for a basis
 * without a table gives RCHEM_ERR_UNSUPPORTED.  The FP64 and emulated-FP64
 * kernels of the Fock build and the gradient read it; the FP32 ones compute.
 */
int rchem_set_exponent_table(rchem_basis b, int on);

/* build_I (src/basis.rs:430-460): the dense n^4 ERI tensor I[m][n][l][s]. */
int rchem_build_I(rchem_basis b, double *I, int where);
/* JK_inmem (src/basis.rs:462-484): J and K from a dense tensor. */
int rchem_jk_inmem(int n, const double *I, const double *D, double *J, double *K, int where);

/* The ERI tensor in the 8-fold packed layout of libpyquante2 (cints.c:375-387,
 * ijkl2intindex): I[ijkl2intindex(i,j,k,l)] = (ij|kl), npair (npair + 1) / 2
 * doubles with npair = n (n + 1) / 2 -- an eighth of build_I's n^4, so (H2O)32
 * in 6-31G* (n = 608, 137 GB) fits in one GB300's memory.  Same integrals as
 * rchem_build_I; RCHEM_ERR_UNSUPPORTED when the device has no room for it. */
int rchem_build_I_packed(rchem_basis b, double *I, int where);
/* J and K (JK_inmem's definitions) from the packed tensor. */
int rchem_jk_packed(int n, const double *I, const double *D, double *J, double *K, int where);

#ifdef __cplusplus
}
#endif
#endif /* RCHEM_GPU_H */
