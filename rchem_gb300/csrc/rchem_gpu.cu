// rchem_gpu.cu -- C ABI (include/rchem_gpu.h, include/rchem_cints.h), the
// host-side planner and the non-class kernels of librchem_gpu.so.
//
// Planner: shells -> shell pairs (l_A >= l_B) -> primitive pairs with all
// per-pair quantities precomputed -> Schwarz bounds Q_ab on the GPU (the class
// kernels' diagonal epilogue) -> pair groups (l_A, l_B, primitive-pair count),
// each sorted by Q descending -> per-class warp task lists.  Because a group
// is sorted by Q, the kets surviving Q_ab Q_cd >= tau for a bra are a prefix
// of every ket group, found by binary search: no quartet list is ever built.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>
#include <tuple>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rchem_cints.h"
#include "../../include/rchem_gpu.h"
#include "_gen/eri_classes.h"
#include "_gen/eri_dispatch.h"
#include "boys.cuh"
#include "eigh.cuh"
#include "eri_kernel.cuh"
#include "grad.cuh"
#include "scf_batch.cuh"
#include "md.cuh"
#include "onee_cls.cuh"
#include "rchem_types.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

static int set_err(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return set_err(e_ == cudaErrorMemoryAllocation ? RCHEM_ERR_NOMEM : RCHEM_ERR_CUDA, "%s: %s", \
                           #call, cudaGetErrorString(e_));                                             \
    } while (0)

#define CKR(expr)                      \
    do {                               \
        int r_ = (expr);               \
        if (r_ != RCHEM_OK) return r_; \
    } while (0)

// frees a temporary device allocation on every return path
struct CudaFreeGuard {
    void *p;
    explicit CudaFreeGuard(void *q) : p(q) {}
    ~CudaFreeGuard() {
        if (p) cudaFree(p);
    }
    CudaFreeGuard(const CudaFreeGuard &) = delete;
    CudaFreeGuard &operator=(const CudaFreeGuard &) = delete;
};
// ... and a list of them
// NVTX range over one entry point (header-only NVTX v3: a no-op unless a
// profiler is attached), so a timeline shows each Fock build, gradient, SCF
// iteration and one-electron matrix.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

struct CudaFreeList {
    std::vector<void *> p;
    ~CudaFreeList() {
        for (void *q : p)
            if (q) cudaFree(q);
    }
};

extern "C" const char *rchem_last_error(void) { return g_err; }
extern "C" int rchem_abi_version(void) { return 1; }

// ---------------------------------------------------------------------------
// Boys tables (one copy per device)
// ---------------------------------------------------------------------------
struct DevTables {
    double *boys64 = nullptr;
    double *boysfar = nullptr;  // power-law table of the branch-free FP64 evaluation
    float *boys32 = nullptr;
    float2 *boysdf = nullptr;  // the FP64 table split into (hi, lo) float pairs
};
static DevTables g_tabs[64];
static std::mutex g_tab_mu;

static int get_tables(const DevTables **out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_err(RCHEM_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lk(g_tab_mu);
    DevTables &t = g_tabs[dev];
    if (!t.boys64) {
        std::vector<double> b64(boys_table_size(BOYS_NT64, BOYS_NGRID64));
        std::vector<float> b32(boys_table_size(BOYS_NT32, BOYS_NGRID32));
        boys_fill_tables(b64.data(), b32.data());
        std::vector<double> bfar(BOYS_FAR_SIZE);
        boys_fill_far(bfar.data());
        std::vector<float2> bdf(b64.size());
        for (size_t i = 0; i < b64.size(); ++i) {
            const float hi = (float)b64[i];
            bdf[i] = make_float2(hi, (float)(b64[i] - (double)hi));
        }
        for (int k = 0; k < RCHEM_NCLASS; ++k) CK(rchem_eri_prepare[k]());  // before any stream capture
        DevTables n;
        CK(cudaMalloc(&n.boys64, b64.size() * sizeof(double)));
        CudaFreeGuard g64(n.boys64);
        CK(cudaMalloc(&n.boys32, b32.size() * sizeof(float)));
        CudaFreeGuard g32(n.boys32);
        CK(cudaMalloc(&n.boysdf, bdf.size() * sizeof(float2)));
        CudaFreeGuard gdf(n.boysdf);
        CK(cudaMalloc(&n.boysfar, bfar.size() * sizeof(double)));
        CudaFreeGuard gfar(n.boysfar);
        CK(cudaMemcpy(n.boys64, b64.data(), b64.size() * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(n.boys32, b32.data(), b32.size() * sizeof(float), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(n.boysdf, bdf.data(), bdf.size() * sizeof(float2), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(n.boysfar, bfar.data(), bfar.size() * sizeof(double), cudaMemcpyHostToDevice));
        g64.p = g32.p = gdf.p = gfar.p = nullptr;  // kept for the life of the process
        t = n;
    }
    *out = &t;
    return RCHEM_OK;
}

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
static int ncart(int l) { return (l + 1) * (l + 2) / 2; }

static double fact2(int n) {
    double r = 1.0;
    for (int i = n; i > 1; i -= 2) r *= i;
    return r;
}

// PGTO::normalization, src/basis.rs:140-149
static double pgto_norm(double alpha, int l, int m, int n) {
    const int L = l + m + n;
    const double num = std::pow(2.0, 2.0 * L + 1.5) * std::pow(alpha, L + 1.5);
    const double den = fact2(2 * l - 1) * fact2(2 * m - 1) * fact2(2 * n - 1) * std::pow(M_PI, 1.5);
    return std::sqrt(num / den);
}

// Cartesian component k of a shell with angular momentum l, src/shell.rs:1-12
RCHEM_HD inline void cart_comp(int l, int k, int *lmn) {
    int idx = 0;
    for (int a = 1; a <= l + 1; ++a)
        for (int b = 1; b <= a; ++b, ++idx)
            if (idx == k) {
                lmn[0] = l + 1 - a;
                lmn[1] = a - b;
                lmn[2] = b - 1;
                return;
            }
    lmn[0] = lmn[1] = lmn[2] = 0;
}

static int pair_cls(int la, int lb) {
    static const int t[3][3] = {{0, -1, -1}, {1, 2, -1}, {3, 4, 5}};
    return t[la][lb];
}
static int quartet_kernel(int cb, int ck) { return cb * (cb + 1) / 2 + ck; }
// gradient work lists: (s/p class, precision) pairs, then (every class with a d shell, precision)
// gradient lists: 2k + prec for the s/p class k; 2 NCLASS + prec for the smaller
// classes with a d shell (per-lane kernel), 2 NCLASS + 2 + prec for the larger ones
// (warp-cooperative kernel)
#define GRAD_NLIST (2 * RCHEM_NCLASS + 4)
// the specialised s/p gradient kernels, one translation unit per arithmetic (grad_sp_*.cu)
bool rchem_grad_sp_f64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st);
bool rchem_grad_sp_f32(int k, const GradArgs &g, unsigned blocks, cudaStream_t st);
bool rchem_grad_sp_df64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st);
bool rchem_grad_sd_f64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st);
bool rchem_grad_pppp_f64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st);
bool rchem_grad_sd_f32(int k, const GradArgs &g, unsigned blocks, cudaStream_t st);
bool rchem_grad_wc_f32(const GradArgs &g, unsigned blocks, cudaStream_t st);
void rchem_grad_rt_f32(const GradArgs &g, unsigned blocks, cudaStream_t st);

// ---------------------------------------------------------------------------
// generic kernels (scalar cints entry points, one-electron matrices)
// ---------------------------------------------------------------------------
__global__ void k_eri_prim_batch(int count, const rchem_prim *pr, const double *boys, double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const rchem_prim *q = pr + 4 * (size_t)i;
    double R[4][3];
    int l[4][3];
    for (int k = 0; k < 4; ++k) {
        R[k][0] = q[k].x; R[k][1] = q[k].y; R[k][2] = q[k].z;
        l[k][0] = q[k].l; l[k][1] = q[k].m; l[k][2] = q[k].n;
    }
    out[i] = q[0].norm * q[1].norm * q[2].norm * q[3].norm *
             md_eri_prim(R[0], l[0], q[0].alpha, R[1], l[1], q[1].alpha, R[2], l[2], q[2].alpha, R[3], l[3],
                         q[3].alpha, boys);
}

__global__ void k_onee_prim_batch(int kind, int count, const rchem_prim *pr, const double *C, const double *boys,
                                  double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const rchem_prim *q = pr + 2 * (size_t)i;
    const double A[3] = {q[0].x, q[0].y, q[0].z}, B[3] = {q[1].x, q[1].y, q[1].z};
    const int la[3] = {q[0].l, q[0].m, q[0].n}, lb[3] = {q[1].l, q[1].m, q[1].n};
    const double zero[3] = {0, 0, 0};
    const double *Cc = (kind == 2) ? C + 3 * (size_t)i : zero;
    double v = md_onee_prim(kind, A, la, q[0].alpha, B, lb, q[1].alpha, Cc, boys);
    if (kind == 2) v *= q[0].norm * q[1].norm;
    out[i] = v;
}

__global__ void k_boys_batch(int count, const int *m, const double *x, const double *b64, const float *b32,
                             const double *bfar, int prec, double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int mm = m[i];
    if (mm < 0 || mm > (prec == 65 ? BOYS_FAR_M - 1 : BOYS_MMAX)) {  // device input unchecked on the host
        out[i] = nan("");
        return;
    }
    if (prec == 65) {  // the ERI kernels' branch-free evaluation, through the L = 8 recursion
        double F[BOYS_FAR_M];
        boys_eval_u<BOYS_FAR_M - 1, false>(x[i], 1.0, b64, bfar, F);
        out[i] = F[mm];
    } else if (prec == 32) {
        float F[BOYS_MMAX + 1];
        boys_eval_rt<float>(mm, (float)x[i], 1.0f, b32, F);
        out[i] = F[mm];
    } else {
        double F[BOYS_MMAX + 1];
        boys_eval_rt<double>(mm, x[i], 1.0, b64, F);
        out[i] = F[mm];
    }
}

// one basis function for the one-electron kernels
struct AODev {
    int shell, lmn[3];
    double cn;  // N(alpha,l,m,n)/N(alpha,L,0,0)
};
struct ShellDev {
    double R[3];
    int l, nprim, prim0, atom;
};

// kind: 0 S, 1 T, 2 V (sum over the geometry's atoms, Z-weighted), 3 moment.
// One thread per element of the packed per-geometry blocks.
__global__ void k_onee_matrix(int kind, long long packed, int ngeom, const GeomDev *geo, const AODev *ao,
                              const ShellDev *sh, const double *pexp, const double *pcoef, const double *Z,
                              const double *Ratoms, const double *boys, const double *center, int ox, int oy, int oz,
                              double *out) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= packed) return;
    const GeomDev gm = geo[geom_of(geo, ngeom, idx)];
    const int loc = (int)(idx - gm.moff), r = loc / gm.n, c = loc % gm.n;
    if (c > r) return;  // lower triangle + mirror, src/basis.rs:237-248
    const AODev a = ao[gm.ao0 + r], b = ao[gm.ao0 + c];
    const ShellDev sa = sh[a.shell], sb = sh[b.shell];
    const int ord[3] = {ox, oy, oz};
    double v = 0.0;
    for (int j = 0; j < sb.nprim; ++j) {
        const double ebj = pexp[sb.prim0 + j], cbj = pcoef[sb.prim0 + j];
        for (int i = 0; i < sa.nprim; ++i) {
            const double eai = pexp[sa.prim0 + i], cc = pcoef[sa.prim0 + i] * cbj;
            double x;
            if (kind == 2) {
                x = 0.0;
                for (int at = gm.atom0; at < gm.atom0 + gm.natoms; ++at)
                    x += Z[at] * md_onee_prim(2, sa.R, a.lmn, eai, sb.R, b.lmn, ebj, Ratoms + 3 * at, boys);
            } else if (kind == 3) {
                x = md_moment_prim(sa.R, a.lmn, eai, sb.R, b.lmn, ebj, center, ord);
            } else {
                x = md_onee_prim(kind, sa.R, a.lmn, eai, sb.R, b.lmn, ebj, sa.R, boys);
            }
            v += cc * x;
        }
    }
    v *= a.cn * b.cn;
    out[gm.moff + (size_t)r * gm.n + c] = v;
    out[gm.moff + (size_t)c * gm.n + r] = v;
}

// J = Jhat + Jhat^T, K = Khat + Khat^T, block by block
__global__ void k_symmetrize(long long packed, int ngeom, const GeomDev *geo, const double *Jh, const double *Kh,
                             double *J, double *K) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= packed) return;
    const GeomDev gm = geo[geom_of(geo, ngeom, idx)];
    const int loc = (int)(idx - gm.moff), r = loc / gm.n, c = loc % gm.n;
    const size_t ji = gm.moff + (size_t)c * gm.n + r;
    J[idx] = Jh[idx] + Jh[ji];
    K[idx] = Kh[idx] + Kh[ji];
}

__global__ void k_to_df64(long long n, const double *x, float2 *y) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) {
        const float hi = (float)x[i];
        y[i] = make_float2(hi, (float)(x[i] - (double)hi));
    }
}

__global__ void k_to_f32(long long n, const double *x, float *y) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}

// JK_inmem, src/basis.rs:462-484
__global__ void k_jk_inmem(int n, const double *I, const double *D, double *J, double *K) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)n * n) return;
    const int mu = (int)(idx / n), nu = (int)(idx % n);
    if (nu > mu) return;
    const size_t N1 = n, N2 = N1 * n, N3 = N2 * n;
    double j = 0.0, k = 0.0;
    for (int la = 0; la < n; ++la)
        for (int sg = 0; sg < n; ++sg) {
            const double d = D[(size_t)la * n + sg];
            j += I[mu * N3 + nu * N2 + la * N1 + sg] * d;
            k += I[mu * N3 + la * N2 + nu * N1 + sg] * d;
        }
    J[(size_t)mu * n + nu] = J[(size_t)nu * n + mu] = j;
    K[(size_t)mu * n + nu] = K[(size_t)nu * n + mu] = k;
}

// ---------------------------------------------------------------------------
// basis handle
// ---------------------------------------------------------------------------
struct PairGroup {
    int cls, la, lb, npp, begin, end, geom;
};

struct rchem_basis_s {
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int natoms = 0, nbf = 0, nshells = 0;
    // geometries (one for rchem_basis_create): packed n_g x n_g matrix blocks
    int ngeom = 1;
    long long packed = 0;
    std::vector<GeomDev> geoms;
    std::vector<int> atom_geom;
    std::vector<int> geom_group_begin, geom_group_end;
    GeomDev *d_geom = nullptr;
    std::vector<int> Z;
    std::vector<double> R;
    std::vector<ShellInfo> shells;
    std::vector<double> pexp, pcoef;  // per primitive, coefficient x N(alpha,l,0,0)
    std::vector<AODev> aos;
    // pairs (sorted: by group, then Q descending)
    std::vector<ShellPair> pairs;
    std::vector<PairGroup> groups;
    int nprims = 0;
    // device
    ShellPair *d_pairs = nullptr;
    PairPrim *d_prims = nullptr;
    PairPrim32 *d_prims32 = nullptr;
    PairPrimDF *d_primsdf = nullptr;
    // factors of (p, q) by primitive-pair exponent number (EriArgs::pq64)
    int npq = 0;          // 0: no table (more than kPqMax exponents)
    bool pq_on = true;    // rchem_set_exponent_table
    int *d_prim_eid = nullptr;
    double2 *d_pq64 = nullptr;
    float4 *d_pqdf = nullptr;
    float2 *d_Ddf = nullptr;
    AODev *d_ao = nullptr;
    ShellDev *d_sh = nullptr;
    double *d_pexp = nullptr, *d_pcoef = nullptr, *d_Z = nullptr, *d_R = nullptr;
    const DevTables *tabs = nullptr;
    // plan
    bool planned = false;
    double plan_tau = -1.0, plan_tau32 = -1.0;
    int plan_part = 0, plan_nparts = 1;  // share of the bra pairs the plan covers
    EriTask *d_tasks = nullptr;
    EriSeg *d_segs = nullptr;
    size_t tasks_cap = 0, segs_cap = 0;
    long long task_off[RCHEM_NCLASS][2], task_cnt[RCHEM_NCLASS][2];
    double list_flops[RCHEM_NCLASS][2];
    long long class_quartets[RCHEM_NCLASS][2], class_prims[RCHEM_NCLASS][2];
    // tile shape per class list: lanes share a quartet while each keeps at
    // least this many primitive quartets (rchem_autotune chooses them)
    int ppl[RCHEM_NCLASS][2];
    int wc[RCHEM_NCLASS][2];  // large classes: warp-cooperative J/K kernel, lanes per quartet (0: not; the autotuner)
    // concurrent class kernels: fork/join over auxiliary streams
    static const int NAUX = 16;
    cudaStream_t aux[NAUX] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[NAUX] = {};
    // the device part of a Fock build, captured once per work plan
    int plan_version = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_version = -1;
    int graph_emul = -1;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;  // device time of a Fock build
    rchem_jk_stats plan_stats;
    rchem_jk_stats last_stats;
    // Fock-build work buffers
    double *d_D = nullptr, *d_Jh = nullptr, *d_Kh = nullptr, *d_Jo = nullptr, *d_Ko = nullptr;
    float *d_D32 = nullptr;
    // gradient: shell atoms / angular momenta, surviving quartets, W, result
    int *d_shell_atom = nullptr, *d_shell_l = nullptr;
    EriTask *d_gtasks = nullptr;  // the gradient's warp tasks (grouped by class) and segments
    EriSeg *d_gsegs = nullptr;
    long long gq_n = 0;
    long long gtask_off[GRAD_NLIST] = {}, gtask_cnt[GRAD_NLIST] = {};
    double gtask_cost[GRAD_NLIST] = {};
    double gq_tau32 = -1.0;
    double gq_tau = -1.0;
    double *d_W = nullptr, *d_grad = nullptr;
    // one-electron matrices: shell pairs of every geometry (lower triangle),
    // grouped by class la*3+lb at [opair_begin[c], opair_begin[c+1])
    OneePair *d_opairs = nullptr;
    int opair_begin[10] = {};
    bool opairs_built = false;
};

static void free_basis(rchem_basis b) {
    if (!b) return;
    void *ptrs[] = {b->d_pairs, b->d_prims, b->d_prims32, b->d_primsdf, b->d_Ddf, b->d_ao, b->d_sh, b->d_pexp, b->d_pcoef, b->d_Z,
                    b->d_R, b->d_tasks, b->d_segs, b->d_D, b->d_Jh, b->d_Kh, b->d_Jo, b->d_Ko, b->d_D32,
                    b->d_shell_atom, b->d_shell_l, b->d_gtasks, b->d_gsegs, b->d_W, b->d_grad, b->d_geom,
                    b->d_opairs, b->d_prim_eid, b->d_pq64, b->d_pqdf};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int i = 0; i < rchem_basis_s::NAUX; ++i) {
        if (b->aux[i]) cudaStreamDestroy(b->aux[i]);
        if (b->ev_join[i]) cudaEventDestroy(b->ev_join[i]);
    }
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_t0) cudaEventDestroy(b->ev_t0);
    if (b->ev_t1) cudaEventDestroy(b->ev_t1);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

template <typename T>
static int upload(T **dst, const std::vector<T> &src, cudaStream_t s) {
    if (src.empty()) return RCHEM_OK;
    CK(cudaMalloc(dst, src.size() * sizeof(T)));
    CK(cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return RCHEM_OK;
}

static const double kPrimCut = 1e-22;  // drop primitive pairs with exp(-ab/p |AB|^2) below this
// ... and those whose prefactor bounds every primitive integral they enter below
// 1e-14: |K_ab| max|K_cd| < kPrimRel (an integral of such a pair with any ket is
// below about kPrimRel times its angular factors, two orders under the 1e-12
// Schwarz screen of whole quartets; against the oracle's unscreened primitives
// the full (H2O)8 J and K are unchanged at 6.6e-13 from 1e-16, with 4.7 % fewer
// primitive quartets in the (H2O)32 build)
static const double kPrimRel = 1e-14;

// distinct exponents of the table the kernels read (0: they compute the factors)
static int pq_active(rchem_basis b) { return b->pq_on ? b->npq : 0; }

static EriArgs base_args(rchem_basis b) {
    EriArgs a;
    memset(&a, 0, sizeof(a));
    a.nbf = b->nbf;
    a.pairs = b->d_pairs;
    a.prims = b->d_prims;
    a.prims32 = b->d_prims32;
    a.boys64 = b->tabs->boys64;
    a.boysfar = b->tabs->boysfar;
    a.boys32 = b->tabs->boys32;
    a.boysdf = b->tabs->boysdf;
    a.primsdf = b->d_primsdf;
    a.Ddf = b->d_Ddf;
    a.npq = pq_active(b);
    a.prim_eid = b->d_prim_eid;
    a.pq64 = b->d_pq64;
    a.pqdf = b->d_pqdf;
    return a;
}

// Schwarz bounds for every pair (class kernels, diagonal epilogue)
// Pack the run of segments sv[s0..] (total quartets) into warp tasks of
// 32 >> lg quartets each, G = 2^lg lanes per quartet.
static void pack_tasks(const std::vector<EriSeg> &sv, int s0, long long total, int lg, long long cost,
                       std::vector<EriTask> &out) {
    const int perwarp = 32 >> lg;
    int sg = s0, off = 0;
    long long left = total;
    while (left > 0) {
        const int nl = (int)std::min<long long>(perwarp, left);
        out.push_back(EriTask{sg, off, nl | (lg << 8), (int)std::min<long long>(cost, 1 << 30)});
        int adv = nl;
        while (adv > 0) {
            const int rem = sv[sg].count - off;
            if (adv < rem) {
                off += adv;
                adv = 0;
            } else {
                adv -= rem;
                ++sg;
                off = 0;
            }
        }
        left -= nl;
    }
}

static int compute_schwarz(rchem_basis b, std::vector<double> &Q) {
    const int np = (int)b->pairs.size();
    std::vector<EriSeg> segs(np);
    for (int i = 0; i < np; ++i) segs[i] = EriSeg{i, i, 1, 0};  // (ab|ab), one quartet per segment
    // per diagonal class, every geometry's pairs in one launch; G lanes per
    // quartet so that each lane has at least 4 primitive quartets
    std::vector<EriTask> per_class[RCHEM_NCLASS];
    for (const PairGroup &g : b->groups) {
        const long long nprimq = (long long)g.npp * g.npp;
        int lg = 0;
        while (lg < 5 && nprimq >= 4LL << (lg + 1)) ++lg;
        if (rchem_class_wc_only[quartet_kernel(g.cls, g.cls)]) lg = 5;  // warp-cooperative: one quartet per warp
        pack_tasks(segs, g.begin, g.end - g.begin, lg, 0, per_class[quartet_kernel(g.cls, g.cls)]);
    }
    std::vector<EriTask> tasks;
    std::vector<int> tkern;
    for (int k = 0; k < RCHEM_NCLASS; ++k) {
        tasks.insert(tasks.end(), per_class[k].begin(), per_class[k].end());
        tkern.insert(tkern.end(), per_class[k].size(), k);
    }
    EriTask *d_t = nullptr;
    EriSeg *d_s = nullptr;
    double *d_Q = nullptr;
    CKR(upload(&d_t, tasks, b->stream));
    CudaFreeGuard g_t(d_t);
    CKR(upload(&d_s, segs, b->stream));
    CudaFreeGuard g_s(d_s);
    CK(cudaMalloc(&d_Q, (size_t)np * sizeof(double)));
    CudaFreeGuard g_Q(d_Q);
    EriArgs a = base_args(b);
    a.J = d_Q;
    a.segs = d_s;
    size_t pos = 0;
    while (pos < tasks.size()) {
        size_t e = pos;
        while (e < tasks.size() && tkern[e] == tkern[pos]) ++e;
        a.tasks = d_t + pos;
        a.ntasks = (int)(e - pos);
        rchem_eri_launchers[tkern[pos]](a, 0, EPI_DIAG, b->stream);
        pos = e;
    }
    CK(cudaGetLastError());
    Q.assign(np, 0.0);
    CK(cudaMemcpyAsync(Q.data(), d_Q, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return RCHEM_OK;
}

// The primitive pairs' distinct exponents p (numbered by first appearance)
// and, for every ordered couple (p, q) of them, 1/sqrt(p+q), pq/(p+q),
// q/(p+q), p/(p+q) in FP64 and as double-float pairs.  A basis has few
// distinct exponents (the exponent sums of its shells), so the table is small
// and cache-resident; past kPqMax exponents the kernels compute the factors.
static const int kPqMax = 1024;  // at most 64 MB of tables
static int build_pq_table(rchem_basis b, const std::vector<PairPrim> &prims) {
    std::unordered_map<unsigned long long, int> num;
    std::vector<double> pv;
    std::vector<int> eid(prims.size());
    for (size_t i = 0; i < prims.size(); ++i) {
        unsigned long long bits;
        memcpy(&bits, &prims[i].p, sizeof(bits));
        auto it = num.find(bits);
        if (it == num.end()) {
            it = num.emplace(bits, (int)pv.size()).first;
            pv.push_back(prims[i].p);
        }
        eid[i] = it->second;
    }
    const int n = (int)pv.size();
    if (n == 0 || n > kPqMax) {
        b->npq = 0;
        return RCHEM_OK;
    }
    std::vector<double2> t64((size_t)2 * n * n);
    std::vector<float4> tdf((size_t)2 * n * n);
    auto split = [](double v, float &hi, float &lo) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    };
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double p = pv[i], q = pv[j], s = p + q;
            const double v[4] = {1.0 / std::sqrt(s), p * q / s, q / s, p / s};
            const size_t e = (size_t)2 * (i * n + j);
            t64[e] = make_double2(v[0], v[1]);
            t64[e + 1] = make_double2(v[2], v[3]);
            float h[8];
            for (int k = 0; k < 4; ++k) split(v[k], h[2 * k], h[2 * k + 1]);
            tdf[e] = make_float4(h[0], h[1], h[2], h[3]);
            tdf[e + 1] = make_float4(h[4], h[5], h[6], h[7]);
        }
    CKR(upload(&b->d_prim_eid, eid, b->stream));
    CKR(upload(&b->d_pq64, t64, b->stream));
    CKR(upload(&b->d_pqdf, tdf, b->stream));
    b->npq = n;
    return RCHEM_OK;
}

static int build_pairs(rchem_basis b) {
    struct Cand {
        ShellPair sp;
        std::vector<PairPrim> pp;
        int cls;
    };
    std::vector<Cand> cands;
    const double c_pref = std::sqrt(2.0) * std::pow(M_PI, 1.25);
    for (int A = 0; A < b->nshells; ++A)
        for (int B = 0; B < b->nshells; ++B) {
            const ShellInfo &sa = b->shells[A], &sb = b->shells[B];
            if (!(sa.l > sb.l || (sa.l == sb.l && A >= B))) continue;
            const int gA = b->atom_geom[sa.atom];
            if (b->atom_geom[sb.atom] != gA) continue;  // pairs never span two geometries
            Cand c;
            double AB[3], r2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                AB[d] = sa.R[d] - sb.R[d];
                r2 += AB[d] * AB[d];
            }
            for (int i = 0; i < sa.nprim; ++i)
                for (int j = 0; j < sb.nprim; ++j) {
                    const double aa = b->pexp[sa.prim0 + i], ab = b->pexp[sb.prim0 + j];
                    const double p = aa + ab, E = std::exp(-aa * ab / p * r2);
                    if (E < kPrimCut) continue;
                    PairPrim q;
                    q.p = p;
                    q.ohp = 0.5 / p;
                    for (int d = 0; d < 3; ++d) {
                        q.P[d] = (aa * sa.R[d] + ab * sb.R[d]) / p;
                        q.PA[d] = q.P[d] - sa.R[d];
                    }
                    q.K = b->pcoef[sa.prim0 + i] * b->pcoef[sb.prim0 + j] * E * c_pref / p;
                    q.pad = aa;  // exponent on shell A (the gradient kernels need it)
                    c.pp.push_back(q);
                }
            if (c.pp.empty()) continue;
            ShellPair &s = c.sp;
            memset(&s, 0, sizeof(s));
            s.A = A;
            s.B = B;
            s.aoA = sa.ao - b->geoms[gA].ao0;  // basis-function index within the geometry
            s.aoB = sb.ao - b->geoms[gA].ao0;
            s.moff = b->geoms[gA].moff;
            s.mn = b->geoms[gA].n;
            s.npp = (int)c.pp.size();
            s.diag = (A == B) ? 1 : 0;
            for (int d = 0; d < 3; ++d) {
                s.AB[d] = AB[d];
                s.AB32[d] = (float)AB[d];
                s.ABlo[d] = (float)(AB[d] - (double)s.AB32[d]);
            }
            s.la_lb = 10 * sa.l + sb.l;
            c.cls = pair_cls(sa.l, sb.l);
            cands.push_back(std::move(c));
        }
    // relative primitive cut against the largest pair prefactor
    double kmax = 0.0;
    for (const Cand &c : cands)
        for (const PairPrim &q : c.pp) kmax = std::max(kmax, std::fabs(q.K));
    {
        std::vector<Cand> kept;
        kept.reserve(cands.size());
        for (Cand &c : cands) {
            std::vector<PairPrim> pp;
            for (const PairPrim &q : c.pp)
                if (std::fabs(q.K) * kmax >= kPrimRel) pp.push_back(q);
            if (pp.empty()) continue;
            c.pp = std::move(pp);
            c.sp.npp = (int)c.pp.size();
            kept.push_back(std::move(c));
        }
        cands = std::move(kept);
    }
    // groups keyed by (geometry, class, npp), geometries in order
    std::map<std::tuple<int, int, int>, std::vector<int>> gm;
    for (int i = 0; i < (int)cands.size(); ++i)
        gm[std::make_tuple(b->atom_geom[b->shells[cands[i].sp.A].atom], cands[i].cls, cands[i].sp.npp)].push_back(i);
    b->pairs.clear();
    b->groups.clear();
    std::vector<PairPrim> prims;
    b->geom_group_begin.assign(b->ngeom, 0);
    b->geom_group_end.assign(b->ngeom, 0);
    for (auto &kv : gm) {
        PairGroup g;
        g.geom = std::get<0>(kv.first);
        g.cls = std::get<1>(kv.first);
        g.npp = std::get<2>(kv.first);
        if (b->geom_group_end[g.geom] == 0) b->geom_group_begin[g.geom] = (int)b->groups.size();
        b->geom_group_end[g.geom] = (int)b->groups.size() + 1;
        const ShellPair &s0 = cands[kv.second[0]].sp;
        g.la = s0.la_lb / 10;
        g.lb = s0.la_lb % 10;
        g.begin = (int)b->pairs.size();
        for (int ci : kv.second) {
            Cand &c = cands[ci];
            c.sp.prim0 = (int)prims.size();
            c.sp.group = (int)b->groups.size();
            prims.insert(prims.end(), c.pp.begin(), c.pp.end());
            b->pairs.push_back(c.sp);
        }
        g.end = (int)b->pairs.size();
        b->groups.push_back(g);
    }
    b->nprims = (int)prims.size();
    std::vector<PairPrim32> p32(prims.size());
    for (size_t i = 0; i < prims.size(); ++i) {
        const PairPrim &q = prims[i];
        PairPrim32 &r = p32[i];
        r.p = (float)q.p;
        r.ohp = (float)q.ohp;
        for (int d = 0; d < 3; ++d) {
            r.P[d] = (float)q.P[d];
            r.PA[d] = (float)q.PA[d];
        }
        r.K = (float)q.K;
        r.pad[0] = (float)q.pad;  // exponent on the first shell (the gradient's weight)
        r.pad[1] = r.pad[2] = 0.f;
    }
    std::vector<PairPrimDF> pdf(prims.size());
    auto split = [](double v, float *hl) {
        hl[0] = (float)v;
        hl[1] = (float)(v - (double)hl[0]);
    };
    for (size_t i = 0; i < prims.size(); ++i) {
        const PairPrim &q = prims[i];
        PairPrimDF &r = pdf[i];
        split(q.p, r.p);
        split(q.ohp, r.ohp);
        for (int d = 0; d < 3; ++d) {
            split(q.P[d], r.P[d]);
            split(q.PA[d], r.PA[d]);
        }
        split(q.K, r.K);
        split(q.pad, r.pad);  // exponent on the first shell
    }
    CKR(upload(&b->d_prims, prims, b->stream));
    CKR(upload(&b->d_prims32, p32, b->stream));
    CKR(upload(&b->d_primsdf, pdf, b->stream));
    CKR(build_pq_table(b, prims));
    CKR(upload(&b->d_pairs, b->pairs, b->stream));
    // Schwarz bounds, then sort each group by Q descending
    std::vector<double> Q;
    CKR(compute_schwarz(b, Q));
    for (size_t i = 0; i < b->pairs.size(); ++i) b->pairs[i].Q = Q[i];
    for (const PairGroup &g : b->groups)
        std::stable_sort(b->pairs.begin() + g.begin, b->pairs.begin() + g.end,
                         [](const ShellPair &x, const ShellPair &y) { return x.Q > y.Q; });
    CK(cudaMemcpyAsync(b->d_pairs, b->pairs.data(), b->pairs.size() * sizeof(ShellPair), cudaMemcpyHostToDevice,
                       b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return RCHEM_OK;
}

// number of kets in [g.begin, g.end) with Q >= thr (Q sorted descending)
static int count_ge(const std::vector<ShellPair> &p, const PairGroup &g, double thr) {
    auto it = std::partition_point(p.begin() + g.begin, p.begin() + g.end,
                                   [thr](const ShellPair &s) { return s.Q >= thr; });
    return (int)(it - (p.begin() + g.begin));
}

// default tile shape: lanes share a quartet only while each keeps at least
// this many primitive quartets
static const int kMinPrimPerLane = 16;

// Algorithmic FLOPs of one primitive quartet of class kernel k: the generated
// count (the operations the FP64 kernel evaluates, its (p, q) factors read
// from the exponent table), plus p+q, 1/sqrt(p+q) (counted as 4), 1/(p+q),
// q/(p+q), p/(p+q) and pq/(p+q) where the kernel computes them (the FP32
// lists, and every list of a basis without the table)
static double prim_flops(rchem_basis b, int k, int prec) {
    return rchem_class_flops[k][0] + ((prec == 0 && pq_active(b) > 0) ? 0.0 : 9.0);
}

// Split the bra shell pairs of a build into nparts shares of about equal cost:
// each bra pair's cost is the algorithmic FLOPs of its surviving quartets
// (both precisions), and the pairs go heaviest first to the least-loaded share
// (ties: the lower share; equal costs in pair order).  Deterministic, so every
// process computes the same split for the same basis and thresholds.
static void split_bras(rchem_basis b, double tau, int nparts, std::vector<int> &owner) {
    const std::vector<ShellPair> &P = b->pairs;
    std::vector<double> cost(P.size(), 0.0);
    for (int gbi = 0; gbi < (int)b->groups.size(); ++gbi) {
        const PairGroup &gb = b->groups[gbi];
        for (int gki = b->geom_group_begin[gb.geom]; gki < b->geom_group_end[gb.geom]; ++gki) {
            const PairGroup &gk = b->groups[gki];
            if (gk.cls > gb.cls || (gk.cls == gb.cls && gki > gbi)) continue;
            const int k = quartet_kernel(gb.cls, gk.cls);
            const double per = rchem_class_flops[k][0] * (double)gb.npp * gk.npp + rchem_class_flops[k][1];
            for (int ib = gb.begin; ib < gb.end; ++ib) {
                const double Qb = P[ib].Q;
                if (!(Qb > 0.0)) continue;
                int nk = (tau > 0.0) ? count_ge(P, gk, tau / Qb) : (gk.end - gk.begin);
                if (gki == gbi) nk = std::min(nk, ib - gb.begin + 1);
                cost[ib] += per * nk;
            }
        }
    }
    std::vector<int> order(P.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    std::vector<double> load(nparts, 0.0);
    owner.assign(P.size(), 0);
    for (int i : order) {
        int best = 0;
        for (int r = 1; r < nparts; ++r)
            if (load[r] < load[best]) best = r;
        owner[i] = best;
        load[best] += cost[i];
    }
}

// The work plan of a Fock build: every surviving unique quartet (or, with
// nparts > 1, those whose bra pair belongs to share `part` of split_bras).
static int plan_tasks(rchem_basis b, double tau, double tau32, int part = 0, int nparts = 1) {
    if (b->planned && tau == b->plan_tau && tau32 == b->plan_tau32 && part == b->plan_part &&
        nparts == b->plan_nparts)
        return RCHEM_OK;
    std::vector<EriSeg> segs[RCHEM_NCLASS][2];
    std::vector<EriTask> lists[RCHEM_NCLASS][2];
    rchem_jk_stats st;
    memset(&st, 0, sizeof(st));
    memset(b->list_flops, 0, sizeof(b->list_flops));
    memset(b->class_quartets, 0, sizeof(b->class_quartets));
    memset(b->class_prims, 0, sizeof(b->class_prims));
    const std::vector<ShellPair> &P = b->pairs;
    std::vector<int> owner;
    if (nparts > 1) split_bras(b, tau, nparts, owner);
    for (int gbi = 0; gbi < (int)b->groups.size(); ++gbi) {
        const PairGroup &gb = b->groups[gbi];
        for (int gki = b->geom_group_begin[gb.geom]; gki < b->geom_group_end[gb.geom]; ++gki) {
            const PairGroup &gk = b->groups[gki];
            if (gk.cls > gb.cls || (gk.cls == gb.cls && gki > gbi)) continue;
            const int k = quartet_kernel(gb.cls, gk.cls);
            const int ncomp = ncart(gb.la) * ncart(gb.lb) * ncart(gk.la) * ncart(gk.lb);
            const long long nprimq = (long long)gb.npp * gk.npp;
            for (int prec = 0; prec < 2; ++prec) {
                std::vector<EriSeg> &sv = segs[k][prec];
                const int s0 = (int)sv.size();
                long long total = 0;
                for (int ib = gb.begin; ib < gb.end; ++ib) {
                    const double Qb = P[ib].Q;
                    if (!(Qb > 0.0)) continue;
                    if (nparts > 1 && owner[ib] != part) continue;
                    int nk = (tau > 0.0) ? count_ge(P, gk, tau / Qb) : (gk.end - gk.begin);
                    if (gki == gbi) nk = std::min(nk, ib - gb.begin + 1);
                    const int m = (tau32 > 0.0) ? std::min(nk, count_ge(P, gk, tau32 / Qb)) : nk;
                    const int lo = prec ? m : 0, hi = prec ? nk : m;
                    if (hi <= lo) continue;
                    sv.push_back(EriSeg{ib, gk.begin + lo, hi - lo, 0});
                    total += hi - lo;
                }
                if (total == 0) continue;
                // G = 2^lg lanes per quartet: at least kMinPrimPerLane primitive
                // quartets per lane, at most 32 lanes
                int lg = 0;
                const long long ppl = b->ppl[k][prec];
                while (lg < 5 && nprimq >= ppl << (lg + 1)) ++lg;
                if (b->wc[k][prec] || rchem_class_wc_only[k]) lg = 5;  // warp-cooperative: one quartet per warp
                pack_tasks(sv, s0, total, lg, (nprimq + (1 << lg) - 1) >> lg, lists[k][prec]);
                const double fl = prim_flops(b, k, prec) * nprimq * total + rchem_class_flops[k][1] * total;
                b->list_flops[k][prec] += fl;
                b->class_quartets[k][prec] += total;
                b->class_prims[k][prec] += total * nprimq;
                if (prec) {
                    st.quartets_fp32 += total;
                    st.prim_quartets_fp32 += total * nprimq;
                    st.eris_fp32 += total * ncomp;
                    st.flops_fp32 += fl;
                } else {
                    st.quartets_fp64 += total;
                    st.prim_quartets_fp64 += total * nprimq;
                    st.eris_fp64 += total * ncomp;
                    st.flops_fp64 += fl;
                }
            }
        }
    }
    // flatten (segment indices become global), heaviest tasks first in each list
    size_t ntask = 0, nseg = 0;
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < 2; ++p) {
            ntask += lists[k][p].size();
            nseg += segs[k][p].size();
        }
    std::vector<EriTask> flat;
    std::vector<EriSeg> fseg;
    flat.reserve(ntask);
    fseg.reserve(nseg);
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < 2; ++p) {
            const int sbase = (int)fseg.size();
            fseg.insert(fseg.end(), segs[k][p].begin(), segs[k][p].end());
            std::vector<EriTask> &L = lists[k][p];
            for (EriTask &t : L) t.seg += sbase;
            std::stable_sort(L.begin(), L.end(), [](const EriTask &x, const EriTask &y) { return x.cost > y.cost; });
            b->task_off[k][p] = (long long)flat.size();
            b->task_cnt[k][p] = (long long)L.size();
            flat.insert(flat.end(), L.begin(), L.end());
            if (!L.empty()) st.kernels += 1;
        }
    st.warp_tasks = (long long)flat.size();
    if (flat.size() > b->tasks_cap || b->d_tasks == nullptr) {
        if (b->d_tasks) cudaFree(b->d_tasks);
        b->d_tasks = nullptr;
        CK(cudaMalloc(&b->d_tasks, std::max<size_t>(flat.size(), 1) * sizeof(EriTask)));
        b->tasks_cap = flat.size();
    }
    if (fseg.size() > b->segs_cap || b->d_segs == nullptr) {
        if (b->d_segs) cudaFree(b->d_segs);
        b->d_segs = nullptr;
        CK(cudaMalloc(&b->d_segs, std::max<size_t>(fseg.size(), 1) * sizeof(EriSeg)));
        b->segs_cap = fseg.size();
    }
    if (!flat.empty())
        CK(cudaMemcpyAsync(b->d_tasks, flat.data(), flat.size() * sizeof(EriTask), cudaMemcpyHostToDevice,
                           b->stream));
    if (!fseg.empty())
        CK(cudaMemcpyAsync(b->d_segs, fseg.data(), fseg.size() * sizeof(EriSeg), cudaMemcpyHostToDevice,
                           b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->plan_stats = st;
    b->planned = true;
    b->plan_version += 1;
    b->plan_tau = tau;
    b->plan_tau32 = tau32;
    b->plan_part = part;
    b->plan_nparts = nparts;
    return RCHEM_OK;
}

// Launch every non-empty class list of an epilogue over the auxiliary streams
// so the class kernels run concurrently: longest-processing-time-first onto
// the least-loaded stream (cost = algorithmic FLOPs; FP32 ones weighted by the
// FP32/FP64 throughput gap); the handle's stream waits for all of them.
static int launch_lists(rchem_basis b, EriArgs a, int epi, bool with32, bool emul = false) {
    struct L {
        int k, p;
        double cost;
    };
    std::vector<L> ls;
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < (with32 ? 2 : 1); ++p)
            if (b->task_cnt[k][p] > 0) ls.push_back(L{k, p, b->list_flops[k][p] / (p ? 16.0 : 1.0)});
    // largest lists first, each onto the least-loaded stream (launching the
    // lists with the longest single warps first measured slower)
    std::stable_sort(ls.begin(), ls.end(), [](const L &x, const L &y) { return x.cost > y.cost; });
    a.segs = b->d_segs;
    const int nuse = std::min<int>((int)ls.size(), rchem_basis_s::NAUX);
    CK(cudaEventRecord(b->ev_fork, b->stream));
    for (int i = 0; i < nuse; ++i) CK(cudaStreamWaitEvent(b->aux[i], b->ev_fork, 0));
    double load[rchem_basis_s::NAUX] = {0};
    for (size_t i = 0; i < ls.size(); ++i) {
        int best = 0;
        for (int j = 1; j < nuse; ++j)
            if (load[j] < load[best]) best = j;
        load[best] += ls[i].cost;
        a.tasks = b->d_tasks + b->task_off[ls[i].k][ls[i].p];
        a.ntasks = (int)b->task_cnt[ls[i].k][ls[i].p];
        a.wc = b->wc[ls[i].k][ls[i].p];
        rchem_eri_launchers[ls[i].k](a, ls[i].p == 1 ? 1 : (emul ? 2 : 0), epi, b->aux[best]);
    }
    CK(cudaGetLastError());
    for (int i = 0; i < nuse; ++i) {
        CK(cudaEventRecord(b->ev_join[i], b->aux[i]));
        CK(cudaStreamWaitEvent(b->stream, b->ev_join[i], 0));
    }
    return RCHEM_OK;
}

// Shared by rchem_basis_create (one geometry) and rchem_batch_create: geometry
// g owns atoms [atom0_g, atom0_g + geom_natoms[g]) and the shells on them,
// which must come in geometry order.
static int create_impl(rchem_basis *out, int ngeom, const int *geom_natoms, int natoms, const int *atomnos,
                       const double *coords, int nshells, const int *shell_atom, const int *shell_l,
                       const int *shell_nprim, const double *exps, const double *coefs) {
    if (!out) return set_err(RCHEM_ERR_INVALID, "out is null");
    *out = nullptr;
    if (natoms <= 0 || nshells <= 0 || ngeom <= 0)
        return set_err(RCHEM_ERR_INVALID, "natoms=%d nshells=%d ngeom=%d", natoms, nshells, ngeom);
    if (!atomnos || !coords || !shell_atom || !shell_l || !shell_nprim || !exps || !coefs || !geom_natoms)
        return set_err(RCHEM_ERR_INVALID, "null array argument");
    for (int i = 0; i < 3 * natoms; ++i)
        if (!std::isfinite(coords[i])) return set_err(RCHEM_ERR_INVALID, "coordinate %d is not finite", i);
    {
        long long tot = 0;
        for (int g = 0; g < ngeom; ++g) {
            if (geom_natoms[g] <= 0) return set_err(RCHEM_ERR_INVALID, "geometry %d has %d atoms", g, geom_natoms[g]);
            tot += geom_natoms[g];
        }
        if (tot != natoms) return set_err(RCHEM_ERR_INVALID, "geometry atom counts sum to %lld, not %d", tot, natoms);
    }
    // Every shell is checked here, on the host, before any CUDA call or
    // allocation (the same checks, in the same order, as the set-up loop below).
    {
        std::vector<int> atom_geom(natoms, 0);
        for (int g = 0, a0 = 0; g < ngeom; a0 += geom_natoms[g], ++g)
            for (int k = 0; k < geom_natoms[g]; ++k) atom_geom[a0 + k] = g;
        long long pos = 0;
        int gprev = 0;
        for (int s = 0; s < nshells; ++s) {
            const int l = shell_l[s], np = shell_nprim[s], at = shell_atom[s];
            if (at >= 0 && at < natoms) {
                if (atom_geom[at] < gprev)
                    return set_err(RCHEM_ERR_INVALID, "shell %d: shells must come in geometry order", s);
                gprev = atom_geom[at];
            }
            if (l < 0 || l > RCHEM_MAX_L)
                return set_err(RCHEM_ERR_UNSUPPORTED, "shell %d has l=%d (supported: 0..%d)", s, l, RCHEM_MAX_L);
            if (np < 1 || np > RCHEM_MAX_NPRIM)
                return set_err(RCHEM_ERR_UNSUPPORTED, "shell %d has %d primitives (supported: 1..%d)", s, np,
                               RCHEM_MAX_NPRIM);
            if (at < 0 || at >= natoms) return set_err(RCHEM_ERR_INVALID, "shell %d on atom %d of %d", s, at, natoms);
            for (int k = 0; k < np; ++k) {
                const double e = exps[pos + k], c = coefs[pos + k];
                if (!(e > 0.0) || !std::isfinite(e) || !std::isfinite(c))
                    return set_err(RCHEM_ERR_INVALID, "shell %d primitive %d: exponent %g coefficient %g", s, k, e,
                                   c);
            }
            pos += np;
        }
    }
    int dev = 0;
    CK(cudaGetDevice(&dev));
    rchem_basis b = new rchem_basis_s();
    b->dev = dev;
    for (int k = 0; k < RCHEM_NCLASS; ++k) {
        // until rchem_autotune chooses: the warp-cooperative kernel for (dd|dp) and
        // up, one lane group per quartet below
        const int L = rchem_class_l[k][0] + rchem_class_l[k][1] + rchem_class_l[k][2] + rchem_class_l[k][3];
        b->ppl[k][0] = b->ppl[k][1] = kMinPrimPerLane;
        b->wc[k][0] = b->wc[k][1] = (rchem_class_wc[k] && L >= 7) ? 32 : 0;
    }
    b->natoms = natoms;
    b->Z.assign(atomnos, atomnos + natoms);
    b->R.assign(coords, coords + 3 * natoms);
    b->nshells = nshells;
    b->ngeom = ngeom;
    b->geoms.assign(ngeom, GeomDev{0, 0, 0, 0, 0, 0});
    b->atom_geom.assign(natoms, 0);
    for (int g = 0, a0 = 0; g < ngeom; ++g) {
        b->geoms[g].atom0 = a0;
        b->geoms[g].natoms = geom_natoms[g];
        for (int k = 0; k < geom_natoms[g]; ++k) b->atom_geom[a0 + k] = g;
        a0 += geom_natoms[g];
    }
    int pos = 0, ao = 0, gprev = 0;
    for (int s = 0; s < nshells; ++s) {
        const int l = shell_l[s], np = shell_nprim[s], at = shell_atom[s];
        if (at >= 0 && at < natoms) {
            const int g = b->atom_geom[at];
            if (g < gprev) {
                free_basis(b);
                return set_err(RCHEM_ERR_INVALID, "shell %d: shells must come in geometry order", s);
            }
            for (int gg = gprev + (s == 0 ? 0 : 1); gg <= g; ++gg) b->geoms[gg].ao0 = ao;
            if (s == 0)
                for (int gg = 0; gg <= g; ++gg) b->geoms[gg].ao0 = 0;
            gprev = g;
        }
        if (l < 0 || l > RCHEM_MAX_L) {
            free_basis(b);
            return set_err(RCHEM_ERR_UNSUPPORTED, "shell %d has l=%d (supported: 0..%d)", s, l, RCHEM_MAX_L);
        }
        if (np < 1 || np > RCHEM_MAX_NPRIM) {
            free_basis(b);
            return set_err(RCHEM_ERR_UNSUPPORTED, "shell %d has %d primitives (supported: 1..%d)", s, np,
                           RCHEM_MAX_NPRIM);
        }
        if (at < 0 || at >= natoms) {
            free_basis(b);
            return set_err(RCHEM_ERR_INVALID, "shell %d on atom %d of %d", s, at, natoms);
        }
        ShellInfo si;
        si.atom = at;
        si.l = l;
        si.nprim = np;
        si.prim0 = (int)b->pexp.size();
        si.ao = ao;
        for (int d = 0; d < 3; ++d) si.R[d] = coords[3 * at + d];
        for (int k = 0; k < np; ++k) {
            const double e = exps[pos + k], c = coefs[pos + k];
            if (!(e > 0.0) || !std::isfinite(e) || !std::isfinite(c)) {
                free_basis(b);
                return set_err(RCHEM_ERR_INVALID, "shell %d primitive %d: exponent %g coefficient %g", s, k, e, c);
            }
            b->pexp.push_back(e);
            b->pcoef.push_back(c * pgto_norm(e, l, 0, 0));
        }
        pos += np;
        for (int k = 0; k < ncart(l); ++k) {
            AODev a;
            a.shell = s;
            cart_comp(l, k, a.lmn);
            a.cn = std::sqrt(fact2(2 * l - 1) / (fact2(2 * a.lmn[0] - 1) * fact2(2 * a.lmn[1] - 1) *
                                                  fact2(2 * a.lmn[2] - 1)));
            b->aos.push_back(a);
        }
        ao += ncart(l);
        b->shells.push_back(si);
    }
    b->nbf = ao;
    for (int gg = gprev + 1; gg < ngeom; ++gg) b->geoms[gg].ao0 = ao;
    {
        long long moff = 0;
        for (int g = 0; g < ngeom; ++g) {
            const int end = (g + 1 < ngeom) ? b->geoms[g + 1].ao0 : ao;
            b->geoms[g].n = end - b->geoms[g].ao0;
            if (b->geoms[g].n <= 0) {
                free_basis(b);
                return set_err(RCHEM_ERR_INVALID, "geometry %d has no basis functions", g);
            }
            b->geoms[g].moff = (int)moff;
            moff += (long long)b->geoms[g].n * b->geoms[g].n;
            if (moff >= (1LL << 31)) {
                free_basis(b);
                return set_err(RCHEM_ERR_UNSUPPORTED, "packed matrices exceed 2^31 elements");
            }
        }
        b->packed = moff;
    }
    int rc;
    if ((rc = get_tables(&b->tabs)) != RCHEM_OK) {
        free_basis(b);
        return rc;
    }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        free_basis(b);
        return set_err(RCHEM_ERR_CUDA, "cudaStreamCreate failed");
    }
    b->own_stream = true;
    for (int i = 0; i < rchem_basis_s::NAUX; ++i) {
        if (cudaStreamCreateWithFlags(&b->aux[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->ev_join[i], cudaEventDisableTiming) != cudaSuccess) {
            free_basis(b);
            return set_err(RCHEM_ERR_CUDA, "auxiliary stream creation failed");
        }
    }
    if (cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->ev_t0) != cudaSuccess || cudaEventCreate(&b->ev_t1) != cudaSuccess) {
        free_basis(b);
        return set_err(RCHEM_ERR_CUDA, "event creation failed");
    }
    std::vector<ShellDev> shd(nshells);
    for (int s = 0; s < nshells; ++s) {
        for (int d = 0; d < 3; ++d) shd[s].R[d] = b->shells[s].R[d];
        shd[s].l = b->shells[s].l;
        shd[s].nprim = b->shells[s].nprim;
        shd[s].prim0 = b->shells[s].prim0;
        shd[s].atom = b->shells[s].atom;
    }
    std::vector<double> Zd(b->Z.begin(), b->Z.end());
    std::vector<int> sh_atom(nshells), sh_l(nshells);
    for (int s2 = 0; s2 < nshells; ++s2) {
        sh_atom[s2] = b->shells[s2].atom;
        sh_l[s2] = b->shells[s2].l;
    }
    if ((rc = upload(&b->d_shell_atom, sh_atom, b->stream)) != RCHEM_OK ||
        (rc = upload(&b->d_shell_l, sh_l, b->stream)) != RCHEM_OK) {
        free_basis(b);
        return rc;
    }
    const size_t nn = (size_t)b->packed;
    if ((rc = upload(&b->d_geom, b->geoms, b->stream)) != RCHEM_OK) {
        free_basis(b);
        return rc;
    }
    if ((rc = upload(&b->d_sh, shd, b->stream)) != RCHEM_OK || (rc = upload(&b->d_ao, b->aos, b->stream)) != RCHEM_OK ||
        (rc = upload(&b->d_pexp, b->pexp, b->stream)) != RCHEM_OK ||
        (rc = upload(&b->d_pcoef, b->pcoef, b->stream)) != RCHEM_OK ||
        (rc = upload(&b->d_Z, Zd, b->stream)) != RCHEM_OK || (rc = upload(&b->d_R, b->R, b->stream)) != RCHEM_OK) {
        free_basis(b);
        return rc;
    }
    if (cudaMalloc(&b->d_D, nn * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&b->d_Jh, nn * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&b->d_Kh, nn * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&b->d_Jo, nn * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&b->d_Ko, nn * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&b->d_D32, nn * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&b->d_Ddf, nn * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&b->d_W, nn * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&b->d_grad, 3 * (size_t)natoms * sizeof(double)) != cudaSuccess) {
        free_basis(b);
        return set_err(RCHEM_ERR_NOMEM, "work buffers for nbf=%d", ao);
    }
    if (cudaMemsetAsync(b->d_D, 0, nn * sizeof(double), b->stream) != cudaSuccess) {
        free_basis(b);
        return set_err(RCHEM_ERR_CUDA, "clearing the density buffer");
    }
    if ((rc = build_pairs(b)) != RCHEM_OK) {
        free_basis(b);
        return rc;
    }
    memset(&b->last_stats, 0, sizeof(b->last_stats));
    *out = b;
    return RCHEM_OK;
}

extern "C" int rchem_basis_create(rchem_basis *out, int natoms, const int *atomnos, const double *coords,
                                  int nshells, const int *shell_atom, const int *shell_l, const int *shell_nprim,
                                  const double *exps, const double *coefs) {
    NvtxRange nv("rchem_basis_create");
    return create_impl(out, 1, &natoms, natoms, atomnos, coords, nshells, shell_atom, shell_l, shell_nprim, exps,
                       coefs);
}

extern "C" int rchem_batch_create(rchem_basis *out, int ngeom, const int *geom_natoms, int natoms, const int *atomnos,
                                  const double *coords, int nshells, const int *shell_atom, const int *shell_l,
                                  const int *shell_nprim, const double *exps, const double *coefs) {
    NvtxRange nv("rchem_batch_create");
    return create_impl(out, ngeom, geom_natoms, natoms, atomnos, coords, nshells, shell_atom, shell_l, shell_nprim,
                       exps, coefs);
}

extern "C" int rchem_basis_layout(rchem_basis b, int *ngeom, long long *packed, int *geom_nbf, long long *geom_offset) {
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    if (ngeom) *ngeom = b->ngeom;
    if (packed) *packed = b->packed;
    for (int g = 0; g < b->ngeom; ++g) {
        if (geom_nbf) geom_nbf[g] = b->geoms[g].n;
        if (geom_offset) geom_offset[g] = b->geoms[g].moff;
    }
    return RCHEM_OK;
}

extern "C" int rchem_basis_destroy(rchem_basis b) {
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_basis(b);
    return RCHEM_OK;
}

extern "C" int rchem_basis_nbf(rchem_basis b) { return b ? b->nbf : -1; }

extern "C" int rchem_basis_set_stream(rchem_basis b, void *stream) {
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    CK(cudaStreamSynchronize(b->stream));
    if (b->own_stream) cudaStreamDestroy(b->stream);
    b->own_stream = false;
    b->stream = (cudaStream_t)stream;
    return RCHEM_OK;  // a captured graph stays valid: it is launched onto whatever stream is current
}

// ---------------------------------------------------------------------------
// output staging: device results -> caller's buffer
// ---------------------------------------------------------------------------
static int finish_out(rchem_basis b, const double *d_src, double *dst, size_t n, int where) {
    if (where == RCHEM_DEVICE) {
        if (d_src != dst) CK(cudaMemcpyAsync(dst, d_src, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    } else {
        CK(cudaMemcpyAsync(dst, d_src, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    }
    CK(cudaStreamSynchronize(b->stream));
    return RCHEM_OK;
}

bool rchem_onee_cls_launch(int kind, const int *begin, const OneePair *pairs, const ShellGrad *sh,
                           const double *pexp, const double *pcoef, const double *Z, const double *R,
                           const double *boys, double *out, cudaStream_t st);

// The shell pairs of the one-electron class kernels, built on first use: per
// geometry every (row shell, column shell) with the row shell's first AO at or
// after the column shell's, grouped by (l_row, l_col) and, within a class, by
// primitive-pair count and atom count (lanes of a warp loop alike).
static int build_onee_pairs(rchem_basis b) {
    if (b->opairs_built) return RCHEM_OK;
    std::vector<std::vector<int>> by_geom(b->ngeom);
    for (int s = 0; s < b->nshells; ++s) by_geom[b->atom_geom[b->shells[s].atom]].push_back(s);
    std::vector<std::pair<long long, OneePair>> keyed;
    for (int g = 0; g < b->ngeom; ++g) {
        const GeomDev &gm = b->geoms[g];
        for (int s1 : by_geom[g])
            for (int s2 : by_geom[g]) {
                const ShellInfo &A = b->shells[s1], &B = b->shells[s2];
                if (A.ao < B.ao) continue;
                OneePair o;
                o.sa = s1;
                o.sb = s2;
                o.ra = A.ao - gm.ao0;
                o.rb = B.ao - gm.ao0;
                o.moff = gm.moff;
                o.n = gm.n;
                o.atom0 = gm.atom0;
                o.natoms = gm.natoms;
                const long long cls = A.l * 3 + B.l;
                const long long cost = (long long)A.nprim * B.nprim * (1 + gm.natoms);
                keyed.push_back({(cls << 40) - cost, o});
            }
    }
    std::stable_sort(keyed.begin(), keyed.end(),
                     [](const std::pair<long long, OneePair> &x, const std::pair<long long, OneePair> &y) {
                         return x.first < y.first;
                     });
    std::vector<OneePair> v(keyed.size());
    int cnt[9] = {};
    for (size_t i = 0; i < keyed.size(); ++i) {
        v[i] = keyed[i].second;
        ++cnt[b->shells[v[i].sa].l * 3 + b->shells[v[i].sb].l];
    }
    b->opair_begin[0] = 0;
    for (int c = 0; c < 9; ++c) b->opair_begin[c + 1] = b->opair_begin[c] + cnt[c];
    CKR(upload(&b->d_opairs, v, b->stream));
    b->opairs_built = true;
    return RCHEM_OK;
}

// kind: 0 S, 1 T, 2 V, 5 T + V (shell-pair class kernels), 3 moment (element kernel)
static int onee(rchem_basis b, int kind, const double *center, int ox, int oy, int oz, double *out, int where) {
    NvtxRange nv(kind == 0 ? "rchem_S" : kind == 1 ? "rchem_T" : kind == 2 ? "rchem_V" : kind == 3 ? "rchem_moment" : "rchem_H");
    if (!b || !out) return set_err(RCHEM_ERR_INVALID, "null argument");
    if (where != RCHEM_HOST && where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", where);
    double *dst = (where == RCHEM_DEVICE) ? out : b->d_Jo;
    if (kind != 3) {
        CKR(build_onee_pairs(b));
        if (!rchem_onee_cls_launch(kind, b->opair_begin, b->d_opairs, reinterpret_cast<const ShellGrad *>(b->d_sh),
                                   b->d_pexp, b->d_pcoef, b->d_Z, b->d_R, b->tabs->boys64, dst, b->stream))
            return set_err(RCHEM_ERR_INVALID, "one-electron kind %d", kind);
        CK(cudaGetLastError());
        return finish_out(b, dst, out, (size_t)b->packed, where);
    }
    double *d_c = nullptr;
    if (kind == 3) CK(cudaMalloc(&d_c, 3 * sizeof(double)));
    CudaFreeGuard g_c(d_c);
    if (kind == 3) CK(cudaMemcpyAsync(d_c, center, 3 * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    const long long n2 = b->packed;
    const int th = 128;
    k_onee_matrix<<<(unsigned)((n2 + th - 1) / th), th, 0, b->stream>>>(kind, n2, b->ngeom, b->d_geom, b->d_ao, b->d_sh,
                                                                         b->d_pexp, b->d_pcoef, b->d_Z, b->d_R,
                                                                         b->tabs->boys64, d_c, ox, oy, oz, dst);
    CK(cudaGetLastError());
    return finish_out(b, dst, out, (size_t)n2, where);
}

extern "C" int rchem_S(rchem_basis b, double *out, int where) { return onee(b, 0, nullptr, 0, 0, 0, out, where); }
extern "C" int rchem_T(rchem_basis b, double *out, int where) { return onee(b, 1, nullptr, 0, 0, 0, out, where); }
extern "C" int rchem_V(rchem_basis b, double *out, int where) { return onee(b, 2, nullptr, 0, 0, 0, out, where); }
extern "C" int rchem_moment(rchem_basis b, const double *center, int ox, int oy, int oz, double *out, int where) {
    if (!center) return set_err(RCHEM_ERR_INVALID, "null center");
    if (ox < 0 || oy < 0 || oz < 0 || ox + oy + oz > 4) return set_err(RCHEM_ERR_UNSUPPORTED, "moment order");
    return onee(b, 3, center, ox, oy, oz, out, where);
}

// ---------------------------------------------------------------------------
// Fock build
// ---------------------------------------------------------------------------
// The device part of a Fock build on the handle's internal buffers:
// d_D -> (d_D32) -> class kernels -> J-hat, K-hat -> d_Jo, d_Ko.
// The FP32 quartets' Boys function from the arithmetic flags: 0 = FP32, 1 = FP64
// (RCHEM_JK_FP32_BOYS64), 2 = FP32 values with the recursion in FP64
// (RCHEM_JK_FP32_REC64); -1 = an invalid combination of flags.
static int f32_boys_mode(int flags) {
    if (flags & ~(RCHEM_JK_EMULATED | RCHEM_JK_FP32_BOYS64 | RCHEM_JK_FP32_REC64)) return -1;
    if ((flags & RCHEM_JK_FP32_BOYS64) && (flags & RCHEM_JK_FP32_REC64)) return -1;
    return (flags & RCHEM_JK_FP32_BOYS64) ? 1 : ((flags & RCHEM_JK_FP32_REC64) ? 2 : 0);
}

static int record_build(rchem_basis b, bool any32, bool emul, int boys64 = 0) {
    const size_t nn = (size_t)b->packed;
    const int th = 256;
    if (any32) {
        k_to_f32<<<(unsigned)((nn + th - 1) / th), th, 0, b->stream>>>((long long)nn, b->d_D, b->d_D32);
        CK(cudaGetLastError());
    }
    if (emul) {
        k_to_df64<<<(unsigned)((nn + th - 1) / th), th, 0, b->stream>>>((long long)nn, b->d_D, b->d_Ddf);
        CK(cudaGetLastError());
    }
    CK(cudaMemsetAsync(b->d_Jh, 0, nn * sizeof(double), b->stream));
    CK(cudaMemsetAsync(b->d_Kh, 0, nn * sizeof(double), b->stream));
    EriArgs a = base_args(b);
    a.D = b->d_D;
    a.D32 = b->d_D32;
    a.J = b->d_Jh;
    a.K = b->d_Kh;
    a.f32_boys64 = boys64;
    CKR(launch_lists(b, a, EPI_JK, any32, emul));
    k_symmetrize<<<(unsigned)((nn + th - 1) / th), th, 0, b->stream>>>((long long)nn, b->ngeom, b->d_geom, b->d_Jh,
                                                                        b->d_Kh, b->d_Jo, b->d_Ko);
    CK(cudaGetLastError());
    return RCHEM_OK;
}

// The captured Fock build of the current plan and arithmetic flags, captured
// again when either has changed since the last capture.
static int ensure_graph(rchem_basis b, bool any32, int flags) {
    if (b->graph_version == b->plan_version && b->graph_emul == flags && b->graph) return RCHEM_OK;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_version = -1;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = record_build(b, any32, (flags & RCHEM_JK_EMULATED) != 0, f32_boys_mode(flags));
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != RCHEM_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return set_err(RCHEM_ERR_CUDA, "capturing the Fock build: %s", cudaGetErrorString(e));
    const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return set_err(RCHEM_ERR_CUDA, "instantiating the Fock build: %s", cudaGetErrorString(ei));
    b->graph_version = b->plan_version;
    b->graph_emul = flags;
    return RCHEM_OK;
}

static bool stream_capturable(rchem_basis b) { return b->stream != nullptr && b->stream != cudaStreamLegacy; }

static int jk_direct_impl(rchem_basis b, const double *D, double *J, double *K, const rchem_jk_opts *opts, int part,
                          int nparts) {
    if (!b || !D || !J || !K) return set_err(RCHEM_ERR_INVALID, "null argument");
    rchem_jk_opts o;
    memset(&o, 0, sizeof(o));
    if (opts) o = *opts;
    if (o.where != RCHEM_HOST && o.where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", o.where);
    if (f32_boys_mode(o.emulated) < 0)
        return set_err(RCHEM_ERR_INVALID,
                       "emulated=%d (flags RCHEM_JK_EMULATED | RCHEM_JK_FP32_BOYS64 or RCHEM_JK_FP32_REC64)",
                       o.emulated);
    const double tau = (o.schwarz_tau == 0.0) ? 1e-12 : (o.schwarz_tau < 0.0 ? 0.0 : o.schwarz_tau);
    const double tau32 = (o.fp32_tau > 0.0) ? o.fp32_tau : 0.0;
    CKR(plan_tasks(b, tau, tau32, part, nparts));
    const size_t nn = (size_t)b->packed;
    CK(cudaEventRecord(b->ev_t0, b->stream));
    CK(cudaMemcpyAsync(b->d_D, D, nn * sizeof(double),
                       o.where == RCHEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, b->stream));
    bool any32 = false;
    for (int k = 0; k < RCHEM_NCLASS; ++k) any32 |= b->task_cnt[k][1] > 0;
    // replay the captured build; capture it again when the plan has changed.
    // The legacy default stream cannot be captured: run the launches directly there.
    const bool capturable = stream_capturable(b);
    if (!capturable) CKR(record_build(b, any32, (o.emulated & RCHEM_JK_EMULATED) != 0, f32_boys_mode(o.emulated)));
    else CKR(ensure_graph(b, any32, o.emulated));
    if (capturable) CK(cudaGraphLaunch(b->graph, b->stream));
    const cudaMemcpyKind out = o.where == RCHEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    CK(cudaMemcpyAsync(J, b->d_Jo, nn * sizeof(double), out, b->stream));
    CK(cudaMemcpyAsync(K, b->d_Ko, nn * sizeof(double), out, b->stream));
    CK(cudaEventRecord(b->ev_t1, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->last_stats = b->plan_stats;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, b->ev_t0, b->ev_t1) == cudaSuccess) b->last_stats.gpu_ms = ms;
    return RCHEM_OK;
}

extern "C" int rchem_jk_direct(rchem_basis b, const double *D, double *J, double *K, const rchem_jk_opts *opts) {
    NvtxRange nv("rchem_jk_direct");
    return jk_direct_impl(b, D, J, K, opts, 0, 1);
}

extern "C" int rchem_jk_direct_part(rchem_basis b, const double *D, double *J, double *K, const rchem_jk_opts *opts,
                                    int part, int nparts) {
    NvtxRange nv("rchem_jk_direct_part");
    if (nparts < 1 || part < 0 || part >= nparts)
        return set_err(RCHEM_ERR_INVALID, "part %d of %d", part, nparts);
    return jk_direct_impl(b, D, J, K, opts, part, nparts);
}

// every unique surviving quartet (bra pair >= ket pair in the class order), as
// for the Fock build, for the one-thread-per-quartet gradient kernel
// The gradient's work plan: the Schwarz-screened unique quartets of every
// (bra group, ket group) combination as segments, packed into warp tasks with
// G lanes per quartet (at least kGradPrimPerLane primitive quartets per lane:
// a derivative primitive quartet is ~100x a Fock one), heaviest tasks first.
// Component quartets from which a d class's gradient runs the warp-cooperative
// kernel: (dd|dp) and (dd|dd).  Measured on (H2O)4 6-31G**-shaped: every
// threshold from 1 to "never" gave 75 ms (1) ... 44 ms (216) ... 42.7 ms (648),
// 43.3 ms (never); below that the lanes of one quartet's warp stay idle.
static long long grad_wc_min() { return 648; }

static int plan_gradient(rchem_basis b, double tau, double tau32) {
    if (b->d_gtasks && b->gq_tau == tau && b->gq_tau32 == tau32) return RCHEM_OK;
    constexpr long long kGradPrimPerLane = 2;
    std::vector<EriSeg> segs;
    // lists: 2 k (+1 for FP32) for the s/p class k, 2 NCLASS (+1) for every class with a d shell
    std::vector<EriTask> per_class[GRAD_NLIST];
    const std::vector<ShellPair> &P = b->pairs;
    for (int gbi = 0; gbi < (int)b->groups.size(); ++gbi) {
        const PairGroup &gb = b->groups[gbi];
        for (int gki = b->geom_group_begin[gb.geom]; gki < b->geom_group_end[gb.geom]; ++gki) {
            const PairGroup &gk = b->groups[gki];
            if (gk.cls > gb.cls || (gk.cls == gb.cls && gki > gbi)) continue;
            const long long nprimq = (long long)gb.npp * gk.npp;
            const int L = gb.la + gb.lb + gk.la + gk.lb;
            // s/p classes get their specialised kernel, every class with a d shell the
            // run-time kernel (its lanes split primitive quartets x ket component pairs);
            // FP64 (or double-float) above tau32, FP32 below
            const int k = quartet_kernel(gb.cls, gk.cls);
            const int *l = rchem_class_l[k];
            // the s/p classes and the smallest d classes have compile-time kernels
            const bool sp = (l[0] <= 1 && l[1] <= 1 && l[2] <= 1 && l[3] <= 1) || k == 6 || k == 7 || k == 9 ||
                            k == 10;
            const long long units = sp ? nprimq : nprimq * ncart(gk.la) * ncart(gk.lb);
            // lanes per quartet: at least kGradPrimPerLane units per lane (for the run-time
            // d-class kernel at least one primitive quartet's ket component pairs, so a
            // lane's run of units shares its primitive-quartet tables)
            const long long per_lane = sp ? kGradPrimPerLane
                                          : std::max<long long>(kGradPrimPerLane, ncart(gk.la) * ncart(gk.lb));
            int lg = 0;
            while (lg < 5 && units >= per_lane << (lg + 1)) ++lg;
            // the larger d classes (at least kGradWcMin component quartets) run the
            // warp-cooperative kernel, one quartet per warp; the smaller ones keep
            // whole quartets per lane group, whose lanes the cooperative kernel
            // could not fill
            const bool wc = !sp && ((long long)ncart(gb.la) * ncart(gb.lb) * ncart(gk.la) * ncart(gk.lb) >=
                                        grad_wc_min() ||
                                    L + 1 > GR_RT_MAXL1 || gk.lb >= GR_RT_NJ);  // the per-lane kernel's table sizes
            if (wc) lg = 5;
            const long long work = (long long)(L + 2) * (L + 2) * (L + 2);  // ~ Hermite work per primitive quartet
            for (int prec = 0; prec < 2; ++prec) {
                const int s0 = (int)segs.size();
                long long total = 0;
                for (int ib = gb.begin; ib < gb.end; ++ib) {
                    const double Qb = P[ib].Q;
                    if (!(Qb > 0.0)) continue;
                    int nk = (tau > 0.0) ? count_ge(P, gk, tau / Qb) : (gk.end - gk.begin);
                    if (gki == gbi) nk = std::min(nk, ib - gb.begin + 1);
                    const int m = (tau32 > 0.0) ? std::min(nk, count_ge(P, gk, tau32 / Qb)) : nk;
                    const int lo = prec ? m : 0, hi = prec ? nk : m;
                    if (hi <= lo) continue;
                    segs.push_back(EriSeg{ib, gk.begin + lo, hi - lo, 0});
                    total += hi - lo;
                }
                if (total == 0) continue;
                pack_tasks(segs, s0, total, lg, ((units + (1 << lg) - 1) >> lg) * work,
                           per_class[sp ? 2 * k + prec : 2 * RCHEM_NCLASS + (wc ? 2 : 0) + prec]);
            }
        }
    }
    // one launch per class (its specialised kernel), heaviest tasks first
    std::vector<EriTask> tasks;
    for (int k = 0; k < GRAD_NLIST; ++k) {
        std::vector<EriTask> &L = per_class[k];
        std::stable_sort(L.begin(), L.end(), [](const EriTask &x, const EriTask &y) { return x.cost > y.cost; });
        b->gtask_off[k] = (long long)tasks.size();
        b->gtask_cnt[k] = (long long)L.size();
        b->gtask_cost[k] = 0.0;
        for (const EriTask &t : L) b->gtask_cost[k] += (double)t.cost;
        tasks.insert(tasks.end(), L.begin(), L.end());
    }
    if (b->d_gtasks) cudaFree(b->d_gtasks);
    if (b->d_gsegs) cudaFree(b->d_gsegs);
    b->d_gtasks = nullptr;
    b->d_gsegs = nullptr;
    b->gq_n = 0;
    CKR(upload(&b->d_gtasks, tasks, b->stream));
    CKR(upload(&b->d_gsegs, segs, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->gq_n = (long long)tasks.size();
    b->gq_tau = tau;
    b->gq_tau32 = tau32;
    return RCHEM_OK;
}
extern "C" int rchem_gradient(rchem_basis b, const double *D, const double *W, double *grad,
                              const rchem_jk_opts *opts) {
    NvtxRange nv("rchem_gradient");
    if (!b || !D || !W || !grad) return set_err(RCHEM_ERR_INVALID, "null argument");
    rchem_jk_opts o;
    memset(&o, 0, sizeof(o));
    if (opts) o = *opts;
    if (o.where != RCHEM_HOST && o.where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", o.where);
    const double tau = (o.schwarz_tau == 0.0) ? 1e-12 : (o.schwarz_tau < 0.0 ? 0.0 : o.schwarz_tau);
    const double tau32 = (o.fp32_tau > 0.0) ? o.fp32_tau : 0.0;
    CKR(plan_gradient(b, tau, tau32));
    const int na = b->natoms;
    const size_t nn = (size_t)b->packed;
    const cudaMemcpyKind in = o.where == RCHEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    CK(cudaMemcpyAsync(b->d_D, D, nn * sizeof(double), in, b->stream));
    CK(cudaMemcpyAsync(b->d_W, W, nn * sizeof(double), in, b->stream));
    // nuclear repulsion: dE/dR_A = -sum_C Z_A Z_C (R_A - R_C) / |R_A - R_C|^3
    std::vector<double> gnuc(3 * (size_t)na, 0.0);
    for (int a = 0; a < na; ++a)
        for (int c = 0; c < na; ++c) {
            if (a == c || b->atom_geom[a] != b->atom_geom[c]) continue;
            double d[3], r2 = 0.0;
            for (int x = 0; x < 3; ++x) {
                d[x] = b->R[3 * a + x] - b->R[3 * c + x];
                r2 += d[x] * d[x];
            }
            const double f = -(double)b->Z[a] * b->Z[c] / (r2 * std::sqrt(r2));
            for (int x = 0; x < 3; ++x) gnuc[3 * a + x] += f * d[x];
        }
    CK(cudaMemcpyAsync(b->d_grad, gnuc.data(), 3 * (size_t)na * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    if (b->gq_n > 0) {
        GradArgs g;
        g.segs = b->d_gsegs;
        g.pairs = b->d_pairs;
        g.prims = b->d_prims;
        g.prims32 = b->d_prims32;
        g.primsdf = b->d_primsdf;
        g.shell_atom = b->d_shell_atom;
        g.shell_l = b->d_shell_l;
        g.boys64 = b->tabs->boys64;
        g.boysfar = b->tabs->boysfar;
        g.boys32 = b->tabs->boys32;
        g.boysdf = b->tabs->boysdf;
        g.D = b->d_D;
        g.grad = b->d_grad;
        g.npq = pq_active(b);
        g.prim_eid = b->d_prim_eid;
        g.pq64 = b->d_pq64;
        g.pqdf = b->d_pqdf;
        // classes run concurrently: longest first, each onto the least-loaded stream
        std::vector<int> ks;
        for (int k = 0; k < GRAD_NLIST; ++k)
            if (b->gtask_cnt[k] > 0) ks.push_back(k);
        std::stable_sort(ks.begin(), ks.end(), [&](int x, int y) { return b->gtask_cost[x] > b->gtask_cost[y]; });
        const int nuse = std::min<int>((int)ks.size(), rchem_basis_s::NAUX);
        CK(cudaEventRecord(b->ev_fork, b->stream));
        for (int i = 0; i < nuse; ++i) CK(cudaStreamWaitEvent(b->aux[i], b->ev_fork, 0));
        double load[rchem_basis_s::NAUX] = {0};
        for (int k : ks) {
            int best = 0;
            for (int j = 1; j < nuse; ++j)
                if (load[j] < load[best]) best = j;
            load[best] += b->gtask_cost[k];
            cudaStream_t st = b->aux[best];
            g.tasks = b->d_gtasks + b->gtask_off[k];
            g.ntasks = (int)b->gtask_cnt[k];
            if (k < 2 * RCHEM_NCLASS) {  // an s/p class: its specialised kernel
                const unsigned blocks = (unsigned)((b->gtask_cnt[k] + 1) / 2);  // one warp per task
                const int cls = k / 2;
                const bool ok = (k & 1) ? (rchem_grad_sp_f32(cls, g, blocks, st) || rchem_grad_sd_f32(cls, g, blocks, st))
                                        : (((o.emulated & RCHEM_JK_EMULATED) && rchem_grad_sp_df64(cls, g, blocks, st)) ||
                                           rchem_grad_sp_f64(cls, g, blocks, st) || rchem_grad_pppp_f64(cls, g, blocks, st) ||
                                           rchem_grad_sd_f64(cls, g, blocks, st));
                if (!ok) return set_err(RCHEM_ERR_UNSUPPORTED, "gradient list %d has no specialised kernel", k);
                CK(cudaGetLastError());
                continue;
            }
            // classes with d shells (run-time angular momenta), FP32 below tau32 and FP64
            // above (also in the emulated form, which keeps these classes in FP64): the
            // smaller ones one lane group per quartet, the larger warp-cooperatively
            if (k < 2 * RCHEM_NCLASS + 2) {
                const unsigned blocks = (unsigned)((b->gtask_cnt[k] + 1) / 2);  // one warp per task
                if (k & 1) rchem_grad_rt_f32(g, blocks, st);
                else k_grad2e_rt<double><<<blocks, 64, 0, st>>>(g);
                CK(cudaGetLastError());
                continue;
            }
            const unsigned blocks = (unsigned)((b->gtask_cnt[k] + GW_WARPS - 1) / GW_WARPS);
            if (k & 1) {
                if (!rchem_grad_wc_f32(g, blocks, st))
                    return set_err(RCHEM_ERR_CUDA, "shared memory for the d-class gradient kernel");
            } else {
                const size_t smem = (size_t)GW_WARPS * GW_PER_WARP * sizeof(double);
                CK(cudaFuncSetAttribute(k_grad2e_wc<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                k_grad2e_wc<double><<<blocks, 32 * GW_WARPS, smem, st>>>(g);
            }
            CK(cudaGetLastError());
        }
        for (int i = 0; i < nuse; ++i) {
            CK(cudaEventRecord(b->ev_join[i], b->aux[i]));
            CK(cudaStreamWaitEvent(b->stream, b->ev_join[i], 0));
        }
    }
    const int th = 128;
    int maxnuc = 1;
    for (const GeomDev &gm : b->geoms) maxnuc = std::max(maxnuc, gm.natoms);
    const dim3 g1((unsigned)((nn + th - 1) / th), (unsigned)((maxnuc + GR1_NUCCHUNK - 1) / GR1_NUCCHUNK));
    k_grad1e<<<g1, th, 0, b->stream>>>(
        (long long)nn, b->ngeom, b->d_geom, reinterpret_cast<const AOGrad *>(b->d_ao),
        reinterpret_cast<const ShellGrad *>(b->d_sh), b->d_pexp, b->d_pcoef, na, b->d_Z, b->d_R, b->tabs->boys64,
        b->d_D, b->d_W, b->d_grad);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(grad, b->d_grad, 3 * (size_t)na * sizeof(double),
                       o.where == RCHEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return RCHEM_OK;
}

// Autotuner: for every class list of the Fock build, time the list alone under
// each candidate tile shape and keep the fastest.
extern "C" int rchem_set_tile_shape(rchem_basis b, int cls, int prec, int ppl) {
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    if (cls < 0 || cls >= RCHEM_NCLASS || prec < 0 || prec > 1)
        return set_err(RCHEM_ERR_INVALID, "class %d / precision %d out of range", cls, prec);
    // ppl > 0: one lane group per quartet; 0, -16, -8: the warp-cooperative
    // kernel with 32, 16 or 8 lanes per quartet
    if (ppl < 0 && ppl != -16 && ppl != -8) return set_err(RCHEM_ERR_INVALID, "primitive quartets per lane %d", ppl);
    if (ppl <= 0 && !rchem_class_wc[cls])
        return set_err(RCHEM_ERR_UNSUPPORTED, "class %d has no warp-cooperative kernel", cls);
    b->wc[cls][prec] = ppl > 0 ? 0 : (ppl == 0 ? 32 : -ppl);
    b->ppl[cls][prec] = ppl <= 0 ? kMinPrimPerLane : ppl;
    b->planned = false;  // the next build replans with this shape
    return RCHEM_OK;
}

extern "C" int rchem_set_exponent_table(rchem_basis b, int on) {
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    if (on && b->npq == 0)
        return set_err(RCHEM_ERR_UNSUPPORTED, "the basis has more than %d primitive-pair exponents: no table", kPqMax);
    b->pq_on = on != 0;
    b->planned = false;  // the next build replans and recaptures with the new setting
    return RCHEM_OK;
}

// One class list alone on the handle's stream: a warm-up launch, then one
// launch bracketed by CUDA events (its device time in *ms).
static int time_list(rchem_basis b, EriArgs a, int k, int prec, float *ms) {
    for (int rep = 0; rep < 2; ++rep) {  // first launch warms caches
        CK(cudaEventRecord(b->ev_t0, b->stream));
        rchem_eri_launchers[k](a, prec, EPI_JK, b->stream);
        CK(cudaEventRecord(b->ev_t1, b->stream));
        CK(cudaEventSynchronize(b->ev_t1));
        CK(cudaEventElapsedTime(ms, b->ev_t0, b->ev_t1));
    }
    CK(cudaGetLastError());
    return RCHEM_OK;
}

// One whole Fock build under the current tile shapes, as rchem_jk_direct runs
// it (the captured build, once to warm up, then timed): its device time in *ms.
static int time_build(rchem_basis b, double tau, double tau32, int flags, float *ms) {
    b->planned = false;
    CKR(plan_tasks(b, tau, tau32));
    bool any32 = false;
    for (int k = 0; k < RCHEM_NCLASS; ++k) any32 |= b->task_cnt[k][1] > 0;
    const bool capturable = stream_capturable(b);
    if (capturable) CKR(ensure_graph(b, any32, flags));
    for (int rep = 0; rep < 2; ++rep) {
        CK(cudaEventRecord(b->ev_t0, b->stream));
        if (capturable) CK(cudaGraphLaunch(b->graph, b->stream));
        else CKR(record_build(b, any32, (flags & RCHEM_JK_EMULATED) != 0, f32_boys_mode(flags)));
        CK(cudaEventRecord(b->ev_t1, b->stream));
        CK(cudaEventSynchronize(b->ev_t1));
    }
    CK(cudaEventElapsedTime(ms, b->ev_t0, b->ev_t1));
    return RCHEM_OK;
}

extern "C" int rchem_autotune(rchem_basis b, const rchem_jk_opts *opts, int *chosen) {
    NvtxRange nv("rchem_autotune");
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    rchem_jk_opts o;
    memset(&o, 0, sizeof(o));
    if (opts) o = *opts;
    if (f32_boys_mode(o.emulated) < 0) return set_err(RCHEM_ERR_INVALID, "emulated=%d", o.emulated);
    const double tau = (o.schwarz_tau == 0.0) ? 1e-12 : (o.schwarz_tau < 0.0 ? 0.0 : o.schwarz_tau);
    const double tau32 = (o.fp32_tau > 0.0) ? o.fp32_tau : 0.0;
    static const int cand[] = {4, 8, 16, 32, 64, 1 << 30};
    const int ncand = (int)(sizeof(cand) / sizeof(cand[0]));
    float best_ms[RCHEM_NCLASS][2], cls_ms[RCHEM_NCLASS][2];
    int best[RCHEM_NCLASS][2], best_wc[RCHEM_NCLASS][2], cls_ppl[RCHEM_NCLASS][2];
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < 2; ++p) {
            best_ms[k][p] = cls_ms[k][p] = 1e30f;
            best[k][p] = cls_ppl[k][p] = kMinPrimPerLane;
            best_wc[k][p] = 0;
        }
    const size_t nn = (size_t)b->packed;
    CK(cudaMemsetAsync(b->d_D, 0, nn * sizeof(double), b->stream));
    CK(cudaMemsetAsync(b->d_D32, 0, nn * sizeof(float), b->stream));
    CK(cudaMemsetAsync(b->d_Ddf, 0, nn * sizeof(float2), b->stream));
    // candidates: every lanes-per-quartet shape, then (c >= ncand) the
    // warp-cooperative kernel of the large classes with 32, 16 and 8 lanes per quartet
    static const int wc_lanes[] = {32, 16, 8};
    for (int c = 0; c < ncand + 3; ++c) {
        const bool wc = c >= ncand;
        const int ql = wc ? wc_lanes[c - ncand] : 0;
        for (int k = 0; k < RCHEM_NCLASS; ++k) {
            b->ppl[k][0] = b->ppl[k][1] = wc ? kMinPrimPerLane : cand[c];
            b->wc[k][0] = b->wc[k][1] = rchem_class_wc[k] ? ql : 0;
        }
        b->planned = false;
        CKR(plan_tasks(b, tau, tau32));
        EriArgs a = base_args(b);
        a.segs = b->d_segs;
        a.D = b->d_D;
        a.D32 = b->d_D32;
        a.Ddf = b->d_Ddf;
        a.J = b->d_Jh;
        a.K = b->d_Kh;
        a.f32_boys64 = f32_boys_mode(o.emulated);
        for (int k = 0; k < RCHEM_NCLASS; ++k)
            for (int p = 0; p < 2; ++p) {
                if (b->task_cnt[k][p] == 0 || (wc && !rchem_class_wc[k])) continue;
                a.tasks = b->d_tasks + b->task_off[k][p];
                a.ntasks = (int)b->task_cnt[k][p];
                a.wc = b->wc[k][p];
                float ms = 0.f;
                CKR(time_list(b, a, k, p == 1 ? 1 : ((o.emulated & RCHEM_JK_EMULATED) ? 2 : 0), &ms));
                if (ms < best_ms[k][p]) {
                    best_ms[k][p] = ms;
                    best[k][p] = wc ? kMinPrimPerLane : cand[c];
                    best_wc[k][p] = ql;
                }
                if (!wc && ms < cls_ms[k][p]) {
                    cls_ms[k][p] = ms;
                    cls_ppl[k][p] = cand[c];
                }
            }
    }
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < 2; ++p) {
            if (rchem_class_wc_only[k] && best_wc[k][p] == 0) {  // its one-lane-group shapes run 32 lanes per quartet
                best[k][p] = kMinPrimPerLane;
                best_wc[k][p] = 32;
            }
            b->ppl[k][p] = best[k][p];
            b->wc[k][p] = best_wc[k][p];
        }
    // In a build the class lists run concurrently, and a list's time alone
    // misjudges its cost there: a warp-cooperative kernel's shared memory takes
    // L1 from the kernels co-resident on its SMs (the (H2O)32 6-31G*-shaped
    // build: its (dd|ds) list with 8 lanes per quartet ran 9 % faster alone
    // than with one lane group per quartet, and made the build 11 % slower).
    // So each large-class list, the longest first, takes the shape of the
    // fastest whole build among its candidates (its best one-lane-group shape
    // and the warp-cooperative kernel with 32, 16, 8 lanes per quartet), the
    // other lists as chosen so far.
    struct Ref {
        int k, p;
        float ms;
    };
    std::vector<Ref> refs;
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < 2; ++p)
            if (rchem_class_wc[k] && b->task_cnt[k][p] > 0) refs.push_back(Ref{k, p, best_ms[k][p]});
    std::stable_sort(refs.begin(), refs.end(), [](const Ref &x, const Ref &y) { return x.ms > y.ms; });
    float cur = 0.f;
    if (!refs.empty()) CKR(time_build(b, tau, tau32, o.emulated, &cur));
    for (const Ref &r : refs) {
        const int k = r.k, p = r.p;
        int opt_ppl[4], opt_wc[4], nopt = 0;
        if (!rchem_class_wc_only[k]) {
            opt_ppl[nopt] = cls_ppl[k][p];
            opt_wc[nopt++] = 0;
        }
        for (int i = 0; i < 3; ++i) {
            opt_ppl[nopt] = kMinPrimPerLane;
            opt_wc[nopt++] = wc_lanes[i];
        }
        int win_ppl = b->ppl[k][p], win_wc = b->wc[k][p];
        for (int i = 0; i < nopt; ++i) {
            if (opt_wc[i] == win_wc && (opt_wc[i] != 0 || opt_ppl[i] == win_ppl)) continue;  // the current shape
            const int keep_ppl = b->ppl[k][p], keep_wc = b->wc[k][p];
            b->ppl[k][p] = opt_ppl[i];
            b->wc[k][p] = opt_wc[i];
            float ms = 0.f;
            CKR(time_build(b, tau, tau32, o.emulated, &ms));
            if (ms < cur) {
                cur = ms;
                win_ppl = opt_ppl[i];
                win_wc = opt_wc[i];
            } else {
                b->ppl[k][p] = keep_ppl;
                b->wc[k][p] = keep_wc;
            }
        }
        b->ppl[k][p] = win_ppl;
        b->wc[k][p] = win_wc;
    }
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < 2; ++p)
            if (chosen) chosen[2 * k + p] = b->wc[k][p] ? (b->wc[k][p] == 32 ? 0 : -b->wc[k][p]) : b->ppl[k][p];
    b->planned = false;
    CKR(plan_tasks(b, tau, tau32));
    return RCHEM_OK;
}

extern "C" int rchem_jk_list_times(rchem_basis b, const rchem_jk_opts *opts, float *ms) {
    NvtxRange nv("rchem_jk_list_times");
    if (!b || !ms) return set_err(RCHEM_ERR_INVALID, "null argument");
    rchem_jk_opts o;
    memset(&o, 0, sizeof(o));
    if (opts) o = *opts;
    if (f32_boys_mode(o.emulated) < 0) return set_err(RCHEM_ERR_INVALID, "emulated=%d", o.emulated);
    const double tau = (o.schwarz_tau == 0.0) ? 1e-12 : (o.schwarz_tau < 0.0 ? 0.0 : o.schwarz_tau);
    const double tau32 = (o.fp32_tau > 0.0) ? o.fp32_tau : 0.0;
    CKR(plan_tasks(b, tau, tau32));
    const size_t nn = (size_t)b->packed;
    const int th = 256;
    // the lower-precision copies of the density the FP32 / double-float lists read
    k_to_f32<<<(unsigned)((nn + th - 1) / th), th, 0, b->stream>>>((long long)nn, b->d_D, b->d_D32);
    k_to_df64<<<(unsigned)((nn + th - 1) / th), th, 0, b->stream>>>((long long)nn, b->d_D, b->d_Ddf);
    CK(cudaGetLastError());
    EriArgs a = base_args(b);
    a.segs = b->d_segs;
    a.D = b->d_D;
    a.D32 = b->d_D32;
    a.J = b->d_Jh;
    a.K = b->d_Kh;
    a.f32_boys64 = f32_boys_mode(o.emulated);
    for (int k = 0; k < RCHEM_NCLASS; ++k)
        for (int p = 0; p < 2; ++p) {
            ms[2 * k + p] = 0.f;
            if (b->task_cnt[k][p] == 0) continue;
            a.tasks = b->d_tasks + b->task_off[k][p];
            a.ntasks = (int)b->task_cnt[k][p];
            a.wc = b->wc[k][p];
            CKR(time_list(b, a, k, p == 1 ? 1 : ((o.emulated & RCHEM_JK_EMULATED) ? 2 : 0), &ms[2 * k + p]));
        }
    return RCHEM_OK;
}

extern "C" int rchem_jk_class_stats(rchem_basis b, int *class_l, long long *quartets, long long *prim_quartets,
                                    double *flops) {
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    if (!b->planned) return set_err(RCHEM_ERR_INVALID, "no Fock build has been planned yet");
    for (int k = 0; k < RCHEM_NCLASS; ++k) {
        for (int d = 0; d < 4; ++d)
            if (class_l) class_l[4 * k + d] = rchem_class_l[k][d];
        for (int p = 0; p < 2; ++p) {
            if (quartets) quartets[2 * k + p] = b->class_quartets[k][p];
            if (prim_quartets) prim_quartets[2 * k + p] = b->class_prims[k][p];
            if (flops) flops[2 * k + p] = b->list_flops[k][p];
        }
    }
    return RCHEM_OK;
}

extern "C" int rchem_jk_stats_get(rchem_basis b, rchem_jk_stats *out) {
    if (!b || !out) return set_err(RCHEM_ERR_INVALID, "null argument");
    *out = b->last_stats;
    return RCHEM_OK;
}

extern "C" int rchem_build_I(rchem_basis b, double *I, int where) {
    NvtxRange nv("rchem_build_I");
    if (!b || !I) return set_err(RCHEM_ERR_INVALID, "null argument");
    if (where != RCHEM_HOST && where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", where);
    if (b->ngeom != 1) return set_err(RCHEM_ERR_UNSUPPORTED, "build_I takes a single-geometry basis");
    const size_t n = b->nbf, n4 = n * n * n * n;
    if (n > 256) return set_err(RCHEM_ERR_UNSUPPORTED, "dense n^4 tensor for n=%zu", n);
    CKR(plan_tasks(b, 0.0, 0.0));  // every quartet, FP64
    double *d_I = I, *d_tmp = nullptr;
    if (where == RCHEM_HOST) {
        CK(cudaMalloc(&d_tmp, n4 * sizeof(double)));
        d_I = d_tmp;
    }
    CudaFreeGuard g_I(d_tmp);
    CK(cudaMemsetAsync(d_I, 0, n4 * sizeof(double), b->stream));
    EriArgs a = base_args(b);
    a.eri = d_I;
    CKR(launch_lists(b, a, EPI_STORE, false));
    if (where == RCHEM_HOST) return finish_out(b, d_I, I, n4, RCHEM_HOST);
    CK(cudaStreamSynchronize(b->stream));
    return RCHEM_OK;
}

// The 8-fold packed tensor: element rchem_eri_pack8(i,j,k,l) holds (ij|kl), one
// value per unique integral (npair (npair + 1) / 2 of them, npair = n (n + 1) / 2).
extern "C" int rchem_build_I_packed(rchem_basis b, double *I, int where) {
    NvtxRange nv("rchem_build_I_packed");
    if (!b || !I) return set_err(RCHEM_ERR_INVALID, "null argument");
    if (where != RCHEM_HOST && where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", where);
    if (b->ngeom != 1) return set_err(RCHEM_ERR_UNSUPPORTED, "build_I_packed takes a single-geometry basis");
    const size_t n = b->nbf, np = n * (n + 1) / 2, len = np * (np + 1) / 2;
    if (where == RCHEM_HOST) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        if (len * sizeof(double) > fr)
            return set_err(RCHEM_ERR_UNSUPPORTED, "packed ERI tensor of %zu bytes exceeds the free device memory (%zu)",
                           len * sizeof(double), fr);
    }
    CKR(plan_tasks(b, 0.0, 0.0));  // every quartet, FP64
    double *d_I = I, *d_tmp = nullptr;
    if (where == RCHEM_HOST) {
        CK(cudaMalloc(&d_tmp, len * sizeof(double)));
        d_I = d_tmp;
    }
    CudaFreeGuard g_I(d_tmp);
    CK(cudaMemsetAsync(d_I, 0, len * sizeof(double), b->stream));
    EriArgs a = base_args(b);
    a.eri = d_I;
    a.eri_packed = 1;
    CKR(launch_lists(b, a, EPI_STORE, false));
    if (where == RCHEM_HOST) return finish_out(b, d_I, I, len, RCHEM_HOST);
    CK(cudaStreamSynchronize(b->stream));
    return RCHEM_OK;
}

// J and K from the packed tensor, JK_inmem's definitions (src/basis.rs:462-484):
// J_mn = sum_ls (mn|ls) D_ls, K_mn = sum_ls (ml|ns) D_ls; one warp per m >= n
__global__ void k_jk_packed(int n, const double *__restrict__ I, const double *__restrict__ D, double *J, double *K) {
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (long long)n * (n + 1) / 2) return;  // whole warps
    int m = (int)((sqrt(8.0 * (double)w + 1.0) - 1.0) * 0.5);
    while ((long long)m * (m + 1) / 2 > w) --m;
    while ((long long)(m + 1) * (m + 2) / 2 <= w) ++m;
    const int nu = (int)(w - (long long)m * (m + 1) / 2);
    double j = 0.0, k = 0.0;
    for (int e = lane; e < n * n; e += 32) {
        const int l = e / n, s2 = e - l * n;
        const double d = D[e];
        j = fma(I[rchem_eri_pack8(m, nu, l, s2)], d, j);
        k = fma(I[rchem_eri_pack8(m, l, nu, s2)], d, k);
    }
    for (int o = 16; o > 0; o >>= 1) {
        j += __shfl_xor_sync(0xffffffffu, j, o);
        k += __shfl_xor_sync(0xffffffffu, k, o);
    }
    if (lane == 0) {
        J[(size_t)m * n + nu] = J[(size_t)nu * n + m] = j;
        K[(size_t)m * n + nu] = K[(size_t)nu * n + m] = k;
    }
}

extern "C" int rchem_jk_packed(int n, const double *I, const double *D, double *J, double *K, int where) {
    if (n <= 0 || !I || !D || !J || !K) return set_err(RCHEM_ERR_INVALID, "bad argument");
    if (where != RCHEM_HOST && where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", where);
    const size_t nn = (size_t)n * n, np = (size_t)n * (n + 1) / 2, len = np * (np + 1) / 2;
    const double *dI = I, *dD = D;
    double *dJ = J, *dK = K;
    CudaFreeList tmp;
    if (where == RCHEM_HOST) {
        double *a = nullptr, *d = nullptr, *j = nullptr, *k = nullptr;
        CK(cudaMalloc(&a, len * sizeof(double)));
        tmp.p.push_back(a);
        CK(cudaMalloc(&d, nn * sizeof(double)));
        tmp.p.push_back(d);
        CK(cudaMalloc(&j, nn * sizeof(double)));
        tmp.p.push_back(j);
        CK(cudaMalloc(&k, nn * sizeof(double)));
        tmp.p.push_back(k);
        CK(cudaMemcpy(a, I, len * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d, D, nn * sizeof(double), cudaMemcpyHostToDevice));
        dI = a;
        dD = d;
        dJ = j;
        dK = k;
    }
    const long long threads = (long long)np * 32;
    k_jk_packed<<<(unsigned)((threads + 127) / 128), 128>>>(n, dI, dD, dJ, dK);
    CK(cudaGetLastError());
    if (where == RCHEM_HOST) {
        CK(cudaMemcpy(J, dJ, nn * sizeof(double), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(K, dK, nn * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        CK(cudaDeviceSynchronize());
    }
    return RCHEM_OK;
}

// libpyquante2/cints.c:375-387 (declared in cints.h:72)
extern "C" int ijkl2intindex(int i, int j, int k, int l) { return (int)rchem_eri_pack8(i, j, k, l); }

extern "C" int rchem_jk_inmem(int n, const double *I, const double *D, double *J, double *K, int where) {
    if (n <= 0 || !I || !D || !J || !K) return set_err(RCHEM_ERR_INVALID, "bad argument");
    if (where != RCHEM_HOST && where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", where);
    const size_t nn = (size_t)n * n, n4 = nn * nn;
    const double *dI = I, *dD = D;
    double *dJ = J, *dK = K;
    double *a = nullptr, *b2 = nullptr, *c = nullptr, *d = nullptr;
    CudaFreeGuard ga(nullptr), gb(nullptr), gc(nullptr), gd(nullptr);
    if (where == RCHEM_HOST) {
        CK(cudaMalloc(&a, n4 * sizeof(double)));
        ga.p = a;
        CK(cudaMalloc(&b2, nn * sizeof(double)));
        gb.p = b2;
        CK(cudaMalloc(&c, nn * sizeof(double)));
        gc.p = c;
        CK(cudaMalloc(&d, nn * sizeof(double)));
        gd.p = d;
        CK(cudaMemcpy(a, I, n4 * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(b2, D, nn * sizeof(double), cudaMemcpyHostToDevice));
        dI = a;
        dD = b2;
        dJ = c;
        dK = d;
    }
    k_jk_inmem<<<(unsigned)((nn + 127) / 128), 128>>>(n, dI, dD, dJ, dK);
    CK(cudaGetLastError());
    if (where == RCHEM_HOST) {
        CK(cudaMemcpy(J, dJ, nn * sizeof(double), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(K, dK, nn * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        CK(cudaDeviceSynchronize());
    }
    return RCHEM_OK;
}

// ---------------------------------------------------------------------------
// cints-compatible scalar and batched entry points
// ---------------------------------------------------------------------------
template <typename T>
static int stage_in(const T *src, size_t n, int where, const T **dev, std::vector<void *> &tmp) {
    if (where == RCHEM_DEVICE) {
        *dev = src;
        return RCHEM_OK;
    }
    T *d = nullptr;
    CK(cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(T)));
    tmp.push_back(d);
    CK(cudaMemcpy(d, src, n * sizeof(T), cudaMemcpyHostToDevice));
    *dev = d;
    return RCHEM_OK;
}

static void free_all(std::vector<void *> &tmp) {
    for (void *p : tmp) cudaFree(p);
    tmp.clear();
}

extern "C" int rchem_eri_prim_batch(int count, const rchem_prim *prims, double *out, int where) {
    if (count < 0 || (count > 0 && (!prims || !out))) return set_err(RCHEM_ERR_INVALID, "bad argument");
    if (count == 0) return RCHEM_OK;
    if (where == RCHEM_HOST)
        for (int i = 0; i < 4 * count; ++i)
            if (prims[i].l < 0 || prims[i].m < 0 || prims[i].n < 0 || !(prims[i].alpha > 0.0))
                return set_err(RCHEM_ERR_INVALID, "primitive %d", i);
    if (where == RCHEM_HOST)
        for (int i = 0; i < count; ++i) {
            int L = 0;
            for (int k = 0; k < 4; ++k) L += prims[4 * i + k].l + prims[4 * i + k].m + prims[4 * i + k].n;
            if (L > MD_MAXL) return set_err(RCHEM_ERR_UNSUPPORTED, "quartet %d has total L=%d > %d", i, L, MD_MAXL);
        }
    const DevTables *t;
    CKR(get_tables(&t));
    std::vector<void *> tmp;
    const rchem_prim *dp;
    int rc = stage_in(prims, 4 * (size_t)count, where, &dp, tmp);
    if (rc) { free_all(tmp); return rc; }
    double *dout = out;
    if (where == RCHEM_HOST) {
        if (cudaMalloc(&dout, count * sizeof(double)) != cudaSuccess) { free_all(tmp); return set_err(RCHEM_ERR_NOMEM, "out"); }
        tmp.push_back(dout);
    }
    k_eri_prim_batch<<<(count + 63) / 64, 64>>>(count, dp, t->boys64, dout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && where == RCHEM_HOST) e = cudaMemcpy(out, dout, count * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && where == RCHEM_DEVICE) e = cudaDeviceSynchronize();
    free_all(tmp);
    if (e != cudaSuccess) return set_err(RCHEM_ERR_CUDA, "eri batch: %s", cudaGetErrorString(e));
    return RCHEM_OK;
}

extern "C" int rchem_onee_prim_batch(int kind, int count, const rchem_prim *prims, const double *centers, double *out,
                                     int where) {
    if (kind < 0 || kind > 2) return set_err(RCHEM_ERR_INVALID, "kind=%d", kind);
    if (count < 0 || (count > 0 && (!prims || !out || (kind == 2 && !centers))))
        return set_err(RCHEM_ERR_INVALID, "bad argument");
    if (count == 0) return RCHEM_OK;
    if (where == RCHEM_HOST)
        for (int i = 0; i < count; ++i) {
            const rchem_prim &a = prims[2 * i], &c = prims[2 * i + 1];
            if ((kind == 2 && a.l + a.m + a.n + c.l + c.m + c.n > MD_MAXL) || a.l + c.l + 2 > MD_MAXE ||
                a.m + c.m + 2 > MD_MAXE || a.n + c.n + 2 > MD_MAXE || a.l < 0 || a.m < 0 || a.n < 0 || c.l < 0 ||
                c.m < 0 || c.n < 0 || !(a.alpha > 0.0) || !(c.alpha > 0.0))
                return set_err(RCHEM_ERR_UNSUPPORTED, "pair %d angular momentum too high", i);
        }
    const DevTables *t;
    CKR(get_tables(&t));
    std::vector<void *> tmp;
    const rchem_prim *dp;
    const double *dc = nullptr;
    int rc = stage_in(prims, 2 * (size_t)count, where, &dp, tmp);
    if (!rc && kind == 2) rc = stage_in(centers, 3 * (size_t)count, where, &dc, tmp);
    if (rc) { free_all(tmp); return rc; }
    double *dout = out;
    if (where == RCHEM_HOST) {
        if (cudaMalloc(&dout, count * sizeof(double)) != cudaSuccess) { free_all(tmp); return set_err(RCHEM_ERR_NOMEM, "out"); }
        tmp.push_back(dout);
    }
    k_onee_prim_batch<<<(count + 63) / 64, 64>>>(kind, count, dp, dc, t->boys64, dout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && where == RCHEM_HOST) e = cudaMemcpy(out, dout, count * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && where == RCHEM_DEVICE) e = cudaDeviceSynchronize();
    free_all(tmp);
    if (e != cudaSuccess) return set_err(RCHEM_ERR_CUDA, "one-electron batch: %s", cudaGetErrorString(e));
    return RCHEM_OK;
}

extern "C" int rchem_boys_batch(int count, const int *m, const double *x, double *out, int precision, int where) {
    if (count < 0 || (count > 0 && (!m || !x || !out))) return set_err(RCHEM_ERR_INVALID, "bad argument");
    if (precision != 64 && precision != 32 && precision != 65)
        return set_err(RCHEM_ERR_INVALID, "precision=%d", precision);
    if (count == 0) return RCHEM_OK;
    const int mmax = precision == 65 ? BOYS_FAR_M - 1 : BOYS_MMAX;
    if (where == RCHEM_HOST)
        for (int i = 0; i < count; ++i)
            if (m[i] < 0 || m[i] > mmax || !(x[i] >= 0.0))
                return set_err(RCHEM_ERR_INVALID, "m=%d x=%g (0 <= m <= %d, x >= 0)", m[i], x[i], mmax);
    const DevTables *t;
    CKR(get_tables(&t));
    std::vector<void *> tmp;
    const int *dm;
    const double *dx;
    int rc = stage_in(m, count, where, &dm, tmp);
    if (!rc) rc = stage_in(x, count, where, &dx, tmp);
    if (rc) { free_all(tmp); return rc; }
    double *dout = out;
    if (where == RCHEM_HOST) {
        if (cudaMalloc(&dout, count * sizeof(double)) != cudaSuccess) { free_all(tmp); return set_err(RCHEM_ERR_NOMEM, "out"); }
        tmp.push_back(dout);
    }
    k_boys_batch<<<(count + 127) / 128, 128>>>(count, dm, dx, t->boys64, t->boys32, t->boysfar, precision, dout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && where == RCHEM_HOST) e = cudaMemcpy(out, dout, count * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && where == RCHEM_DEVICE) e = cudaDeviceSynchronize();
    free_all(tmp);
    if (e != cudaSuccess) return set_err(RCHEM_ERR_CUDA, "boys batch: %s", cudaGetErrorString(e));
    return RCHEM_OK;
}

static rchem_prim mkprim(double x, double y, double z, double norm, int l, int m, int n, double alpha) {
    rchem_prim p;
    p.x = x; p.y = y; p.z = z; p.norm = norm; p.alpha = alpha; p.l = l; p.m = m; p.n = n; p.pad = 0;
    return p;
}

extern "C" double coulomb_repulsion(double xa, double ya, double za, double norma, int la, int ma, int na,
                                    double alphaa, double xb, double yb, double zb, double normb, int lb, int mb,
                                    int nb, double alphab, double xc, double yc, double zc, double normc, int lc,
                                    int mc, int nc, double alphac, double xd, double yd, double zd, double normd,
                                    int ld, int md, int nd, double alphad) {
    rchem_prim q[4] = {mkprim(xa, ya, za, norma, la, ma, na, alphaa), mkprim(xb, yb, zb, normb, lb, mb, nb, alphab),
                       mkprim(xc, yc, zc, normc, lc, mc, nc, alphac), mkprim(xd, yd, zd, normd, ld, md, nd, alphad)};
    double v = NAN;
    if (rchem_eri_prim_batch(1, q, &v, RCHEM_HOST) != RCHEM_OK) return NAN;
    return v;
}

extern "C" double overlap(double alpha1, int l1, int m1, int n1, double xa, double ya, double za, double alpha2,
                          int l2, int m2, int n2, double xb, double yb, double zb) {
    rchem_prim q[2] = {mkprim(xa, ya, za, 1.0, l1, m1, n1, alpha1), mkprim(xb, yb, zb, 1.0, l2, m2, n2, alpha2)};
    double v = NAN;
    if (rchem_onee_prim_batch(0, 1, q, nullptr, &v, RCHEM_HOST) != RCHEM_OK) return NAN;
    return v;
}

extern "C" double kinetic(double alpha1, int l1, int m1, int n1, double xa, double ya, double za, double alpha2,
                          int l2, int m2, int n2, double xb, double yb, double zb) {
    rchem_prim q[2] = {mkprim(xa, ya, za, 1.0, l1, m1, n1, alpha1), mkprim(xb, yb, zb, 1.0, l2, m2, n2, alpha2)};
    double v = NAN;
    if (rchem_onee_prim_batch(1, 1, q, nullptr, &v, RCHEM_HOST) != RCHEM_OK) return NAN;
    return v;
}

extern "C" double nuclear_attraction(double x1, double y1, double z1, double norm1, int l1, int m1, int n1,
                                     double alpha1, double x2, double y2, double z2, double norm2, int l2, int m2,
                                     int n2, double alpha2, double x3, double y3, double z3) {
    rchem_prim q[2] = {mkprim(x1, y1, z1, norm1, l1, m1, n1, alpha1), mkprim(x2, y2, z2, norm2, l2, m2, n2, alpha2)};
    const double c[3] = {x3, y3, z3};
    double v = NAN;
    if (rchem_onee_prim_batch(2, 1, q, c, &v, RCHEM_HOST) != RCHEM_OK) return NAN;
    return v;
}

extern "C" double Fgamma(double m, double x) {
    const int mi = (int)(m + 0.5);
    double v = NAN;
    if (rchem_boys_batch(1, &mi, &x, &v, 64, RCHEM_HOST) != RCHEM_OK) return NAN;
    return v;
}

extern "C" double contr_coulomb(int ia, double *aexps, double *acoefs, double *anorms, double xa, double ya,
                                double za, int la, int ma, int na, int ib, double *bexps, double *bcoefs,
                                double *bnorms, double xb, double yb, double zb, int lb, int mb, int nb, int ic,
                                double *cexps, double *ccoefs, double *cnorms, double xc, double yc, double zc,
                                int lc, int mc, int nc, int id, double *dexps, double *dcoefs, double *dnorms,
                                double xd, double yd, double zd, int ld, int md, int nd) {
    if (ia <= 0 || ib <= 0 || ic <= 0 || id <= 0) {
        set_err(RCHEM_ERR_INVALID, "empty contraction");
        return NAN;
    }
    const int count = ia * ib * ic * id;
    std::vector<rchem_prim> q((size_t)count * 4);
    std::vector<double> w(count), v(count);
    int k = 0;
    for (int i = 0; i < ia; ++i)
        for (int j = 0; j < ib; ++j)
            for (int c = 0; c < ic; ++c)
                for (int d = 0; d < id; ++d, ++k) {
                    q[4 * k + 0] = mkprim(xa, ya, za, anorms[i], la, ma, na, aexps[i]);
                    q[4 * k + 1] = mkprim(xb, yb, zb, bnorms[j], lb, mb, nb, bexps[j]);
                    q[4 * k + 2] = mkprim(xc, yc, zc, cnorms[c], lc, mc, nc, cexps[c]);
                    q[4 * k + 3] = mkprim(xd, yd, zd, dnorms[d], ld, md, nd, dexps[d]);
                    w[k] = acoefs[i] * bcoefs[j] * ccoefs[c] * dcoefs[d];
                }
    if (rchem_eri_prim_batch(count, q.data(), v.data(), RCHEM_HOST) != RCHEM_OK) return NAN;
    double s = 0.0;
    for (int i = 0; i < count; ++i) s += w[i] * v[i];
    return s;
}

// ---------------------------------------------------------------------------
// Fock build that allocates nothing
// ---------------------------------------------------------------------------
// rchem_jk_direct keeps its J-hat/K-hat accumulators in buffers the basis
// handle allocated when it was created, and may allocate again when the work
// plan changes.  Some callers cannot allocate device memory at the point where
// they need a Fock build: code running under an external memory manager that
// owns the whole device (a pooled allocator that forbids cudaMalloc after
// start-up), or a long-running service whose steady-state loop must never
// allocate.  rchem_jk_direct_noalloc serves them: its scratch (J-hat, K-hat and the
// single-precision copy of D of the mixed form) lives in the file-scope device
// array below, sized for up to RCHEM_NOALLOC_MAX_NBF basis functions
// (2*640^2 doubles + 640^2 floats, about 8 MiB); every GPU that loads this
// library holds that array until the process exits.
#define RCHEM_NOALLOC_MAX_NBF 640
#define RCHEM_NOALLOC_DOUBLES (2 * RCHEM_NOALLOC_MAX_NBF * RCHEM_NOALLOC_MAX_NBF + \
                               RCHEM_NOALLOC_MAX_NBF * RCHEM_NOALLOC_MAX_NBF / 2)
static __device__ __align__(256) double g_noalloc_scratch[RCHEM_NOALLOC_DOUBLES];

// The array's device address, looked up once per device.  On the host the
// symbol g_noalloc_scratch is only a stand-in: a kernel given it would fault,
// or silently touch the wrong memory where the GPU can reach host memory, so
// kernels are always handed this looked-up address.
static double *g_noalloc_ptr[64];
static std::mutex g_noalloc_mu;

static int noalloc_scratch(double **out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_err(RCHEM_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return set_err(RCHEM_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = (double *)p;
    }
    *out = g_noalloc_ptr[dev];
    return RCHEM_OK;
}

extern "C" int rchem_jk_direct_noalloc(rchem_basis b, const double *D, double *J, double *K,
                                       const rchem_jk_opts *opts) {
    NvtxRange nv("rchem_jk_direct_noalloc");
    if (!b || !D || !J || !K || !opts) return set_err(RCHEM_ERR_INVALID, "null argument");
    if (opts->where != RCHEM_DEVICE)
        return set_err(RCHEM_ERR_INVALID, "rchem_jk_direct_noalloc takes device arrays only (opts->where = RCHEM_DEVICE)");
    if (b->ngeom != 1) return set_err(RCHEM_ERR_UNSUPPORTED, "rchem_jk_direct_noalloc takes a single-geometry basis");
    const int n = b->nbf;
    if (n > RCHEM_NOALLOC_MAX_NBF)
        return set_err(RCHEM_ERR_UNSUPPORTED, "nbf=%d exceeds the no-allocation limit of %d basis functions", n,
                       RCHEM_NOALLOC_MAX_NBF);
    const double tau = (opts->schwarz_tau == 0.0) ? 1e-12 : (opts->schwarz_tau < 0.0 ? 0.0 : opts->schwarz_tau);
    const double tau32 = (opts->fp32_tau > 0.0) ? opts->fp32_tau : 0.0;
    if (!b->planned || tau != b->plan_tau || tau32 != b->plan_tau32 || b->plan_nparts != 1)
        return set_err(RCHEM_ERR_INVALID,
                       "the basis has no work plan for these thresholds: call rchem_jk_direct once with the same "
                       "options first (planning may allocate)");
    // the scratch address and the handle's stream both belong to the handle's device
    int cur = -1;
    CK(cudaGetDevice(&cur));
    if (cur != b->dev)
        return set_err(RCHEM_ERR_INVALID, "the current device is %d, the handle's device is %d: make it current first",
                       cur, b->dev);
    double *scratch = nullptr;
    CKR(noalloc_scratch(&scratch));
    const size_t nn = (size_t)n * n;
    double *Jh = scratch, *Kh = scratch + nn;
    float *D32 = (float *)(scratch + 2 * nn);
    // the array keeps the previous call's contents: clear the accumulators
    CK(cudaMemsetAsync(Jh, 0, 2 * nn * sizeof(double), b->stream));
    bool any32 = false;
    for (int k = 0; k < RCHEM_NCLASS; ++k) any32 |= b->task_cnt[k][1] > 0;
    const int th = 256;
    if (any32) {
        k_to_f32<<<(unsigned)((nn + th - 1) / th), th, 0, b->stream>>>((long long)nn, D, D32);
        CK(cudaGetLastError());
    }
    EriArgs a = base_args(b);
    a.D = D;
    a.D32 = D32;
    a.J = Jh;
    a.K = Kh;
    CKR(launch_lists(b, a, EPI_JK, any32));
    k_symmetrize<<<(unsigned)((nn + th - 1) / th), th, 0, b->stream>>>((long long)nn, 1, b->d_geom, Jh, Kh, J, K);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(b->stream));
    b->last_stats = b->plan_stats;
    return RCHEM_OK;
}

// ---------------------------------------------------------------------------
// batched symmetric eigensolver (the batched SCF's diagonalisations)
// ---------------------------------------------------------------------------
extern "C" int rchem_eigh_batched(int n, int batch, const double *A, double *w, double *V, void *stream) {
    if (n < 1 || n > RCHEM_EIGH_MAXN)
        return set_err(RCHEM_ERR_UNSUPPORTED, "rchem_eigh_batched: n = %d outside 1..%d", n, RCHEM_EIGH_MAXN);
    if (batch < 0) return set_err(RCHEM_ERR_INVALID, "rchem_eigh_batched: batch = %d", batch);
    if (batch == 0) return RCHEM_OK;
    if (!A || !w || !V) return set_err(RCHEM_ERR_INVALID, "rchem_eigh_batched: null array");
    const void *ptrs[3] = {A, w, V};
    for (const void *ptr : ptrs) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess ||
            (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return set_err(RCHEM_ERR_INVALID, "rchem_eigh_batched: A, w and V must be device arrays");
        }
    }
    const size_t smem = eigh_smem_bytes(n);
    CK(cudaFuncSetAttribute(k_eigh_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_eigh_jacobi<<<batch, RCHEM_EIGH_THREADS, smem, (cudaStream_t)stream>>>(n, A, w, V, nullptr);
    CK(cudaGetLastError());
    return RCHEM_OK;
}

// ---------------------------------------------------------------------------
// native RHF driver: every geometry of the handle at once (scf_batch.cuh)
// ---------------------------------------------------------------------------
extern "C" int rchem_rhf(rchem_basis b, const rchem_scf_opts *opts, const int *nocc_in, double *e_elec,
                         double *e_nuc, double *D_out, double *W_out, int *iterations, int *converged) {
    NvtxRange nv("rchem_rhf");
    if (!b) return set_err(RCHEM_ERR_INVALID, "null handle");
    rchem_scf_opts o;
    memset(&o, 0, sizeof(o));
    o.thresh_e = 1e-10;
    o.thresh_d = 1e-7;
    o.max_iter = 128;
    o.diis = RCHEM_DIIS_MAX;
    if (opts) o = *opts;
    if (o.diis < 0 || o.diis > RCHEM_DIIS_MAX) return set_err(RCHEM_ERR_INVALID, "diis = %d (0..%d)", o.diis, RCHEM_DIIS_MAX);
    if (o.max_iter < 1) return set_err(RCHEM_ERR_INVALID, "max_iter = %d", o.max_iter);
    if (o.jk.where != RCHEM_HOST && o.jk.where != RCHEM_DEVICE) return set_err(RCHEM_ERR_INVALID, "where=%d", o.jk.where);
    if (f32_boys_mode(o.jk.emulated) < 0)
        return set_err(RCHEM_ERR_INVALID, "jk.emulated=%d", o.jk.emulated);
    const int ng = b->ngeom;
    const long long packed = b->packed;
    int nmax = 0;
    std::vector<int> nocc(ng);
    for (int g = 0; g < ng; ++g) {
        const GeomDev &gm = b->geoms[g];
        nmax = std::max(nmax, gm.n);
        if (nocc_in) {
            nocc[g] = nocc_in[g];
        } else {
            int ne = 0;
            for (int a = gm.atom0; a < gm.atom0 + gm.natoms; ++a) ne += b->Z[a];
            if (ne % 2) return set_err(RCHEM_ERR_INVALID, "geometry %d has an odd electron count (%d)", g, ne);
            nocc[g] = ne / 2;
        }
        if (nocc[g] < 0 || nocc[g] > gm.n) return set_err(RCHEM_ERR_INVALID, "geometry %d: nocc %d", g, nocc[g]);
    }
    if (nmax > RCHEM_EIGH_MAXN)
        return set_err(RCHEM_ERR_UNSUPPORTED, "rchem_rhf diagonalises n <= %d per geometry (largest: %d)",
                       RCHEM_EIGH_MAXN, nmax);
    cudaStream_t st = b->stream;
    const size_t bytes = (size_t)packed * sizeof(double);
    // device buffers, freed on every return path
    enum { S_, H_, X_, T1_, T2_, F_, FX_, D_, DO_, J_, K_, W_, CV_, CV2_, EPS_, NB_ };
    double *buf[NB_] = {};
    CudaFreeList guards;
    for (int k = 0; k < NB_; ++k) {
        CK(cudaMalloc(&buf[k], bytes));
        guards.p.push_back(buf[k]);
    }
    const int nh = std::max(o.diis, 1);
    double *Fh = nullptr, *Eh = nullptr, *d_e = nullptr, *d_dm = nullptr, *d_coef = nullptr;
    int *d_nocc = nullptr;
    CK(cudaMalloc(&Fh, bytes * nh));
    guards.p.push_back(Fh);
    CK(cudaMalloc(&Eh, bytes * nh));
    guards.p.push_back(Eh);
    CK(cudaMalloc(&d_e, ng * sizeof(double)));
    guards.p.push_back(d_e);
    CK(cudaMalloc(&d_dm, ng * sizeof(double)));
    guards.p.push_back(d_dm);
    CK(cudaMalloc(&d_coef, (size_t)ng * RCHEM_DIIS_MAX * sizeof(double)));
    guards.p.push_back(d_coef);
    CK(cudaMalloc(&d_nocc, ng * sizeof(int)));
    guards.p.push_back(d_nocc);
    CK(cudaMemcpyAsync(d_nocc, nocc.data(), ng * sizeof(int), cudaMemcpyHostToDevice, st));
    double *S = buf[S_], *H = buf[H_], *X = buf[X_], *T1 = buf[T1_], *T2 = buf[T2_], *F = buf[F_], *Fx = buf[FX_],
           *D = buf[D_], *Dold = buf[DO_], *J = buf[J_], *K = buf[K_], *Wm = buf[W_], *Cv = buf[CV_],
           *Cn = buf[CV2_], *eps = buf[EPS_];
    const size_t esm = eigh_smem_bytes(nmax);
    CK(cudaFuncSetAttribute(k_scf_eigh, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esm));
    const int th = RCHEM_SCF_THREADS;
    const unsigned eb = (unsigned)((packed + th - 1) / th);
    const GeomDev *geo = b->d_geom;
    // S, H = T + V, X = S^-1/2 (the eigenvalues go to eps, the vectors to T1)
    CKR(onee(b, RCHEM_ONEE_S, nullptr, 0, 0, 0, S, RCHEM_DEVICE));
    CKR(onee(b, RCHEM_ONEE_H, nullptr, 0, 0, 0, H, RCHEM_DEVICE));
    k_scf_eigh<<<ng, RCHEM_EIGH_THREADS, esm, st>>>(geo, S, eps, T1);
    k_scf_invsqrt<<<ng, th, 0, st>>>(geo, eps, T1, X);
    CK(cudaGetLastError());
    // Roothaan step, warm-started: with the previous orbitals C (S-orthonormal;
    // C = X before the first step) F'' = C^T F C is diagonalised, F'' = V e V^T,
    // and the new orbitals are C V.  This is X^T F X expressed in the basis of
    // the previous orbitals, so the eigenpairs are those of the plain step; once
    // the orbitals settle F'' is nearly diagonal and Jacobi needs 2-3 sweeps
    // instead of 8-10.  Then D = C_occ C_occ^T (and W).
    CK(cudaMemcpyAsync(Cv, X, bytes, cudaMemcpyDeviceToDevice, st));
    auto density = [&](const double *Fin, double *Dd, double *Ww) -> int {
        k_scf_gemm<<<ng, th, 0, st>>>(geo, Cv, 1, Fin, 0, T1, 1.0, 0.0);
        k_scf_gemm<<<ng, th, 0, st>>>(geo, T1, 0, Cv, 0, T2, 1.0, 0.0);
        k_scf_eigh<<<ng, RCHEM_EIGH_THREADS, esm, st>>>(geo, T2, eps, T1);
        k_scf_gemm<<<ng, th, 0, st>>>(geo, Cv, 0, T1, 0, Cn, 1.0, 0.0);
        k_scf_copy<<<ng, th, 0, st>>>(geo, Cn, Cv);  // the new orbitals (a copy keeps the pointers fixed for capture)
        k_scf_density<<<ng, th, 0, st>>>(geo, d_nocc, Cv, eps, Dd, Ww);
        CK(cudaGetLastError());
        return RCHEM_OK;
    };
    CKR(density(H, D, nullptr));  // core-Hamiltonian guess
    rchem_jk_opts jo = o.jk;
    jo.where = RCHEM_DEVICE;
    std::vector<double> eg(ng);
    // the iteration's state lives on the device (ring slot, count, stop flag)
    ScfState *d_st = nullptr;
    double *d_eprev = nullptr;
    CK(cudaMalloc(&d_st, sizeof(ScfState)));
    guards.p.push_back(d_st);
    CK(cudaMalloc(&d_eprev, ng * sizeof(double)));
    guards.p.push_back(d_eprev);
    CK(cudaMemsetAsync(d_st, 0, sizeof(ScfState), st));
    CK(cudaMemsetAsync(d_eprev, 0, ng * sizeof(double), st));
    const double tau = (jo.schwarz_tau == 0.0) ? 1e-12 : (jo.schwarz_tau < 0.0 ? 0.0 : jo.schwarz_tau);
    const double tau32 = (jo.fp32_tau > 0.0) ? jo.fp32_tau : 0.0;
    CKR(plan_tasks(b, tau, tau32));
    bool any32 = false;
    for (int k = 0; k < RCHEM_NCLASS; ++k) any32 |= b->task_cnt[k][1] > 0;
    const bool emul = (jo.emulated & RCHEM_JK_EMULATED) != 0;
    const int boys64 = f32_boys_mode(jo.emulated);
    // One iteration, every argument fixed (state-driven), so the same launches
    // can be captured once and replayed:  J, K of D (the Fock build on the
    // handle's buffers), F = H + 2J - K, the energies, the DIIS step, the
    // Roothaan step, max |D - Dold|, then k_scf_check.
    auto iteration = [&](cudaGraphConditionalHandle h, int use_h) -> int {
        CK(cudaMemcpyAsync(b->d_D, D, bytes, cudaMemcpyDeviceToDevice, st));
        CKR(record_build(b, any32, emul, boys64));
        k_scf_fock<<<eb, th, 0, st>>>(packed, H, b->d_Jo, b->d_Ko, F);
        k_scf_energy<<<ng, th, 0, st>>>(geo, H, F, D, nullptr, d_e, d_dm);
        const double *Fuse = F;
        if (o.diis > 0) {
            // error X^T (FDS - SDF) X into this iteration's ring slot, F beside it
            k_scf_diis_slot<<<1, 32, 0, st>>>(d_st, o.diis);
            k_scf_gemm<<<ng, th, 0, st>>>(geo, F, 0, D, 0, T1, 1.0, 0.0);
            k_scf_gemm<<<ng, th, 0, st>>>(geo, T1, 0, S, 0, T2, 1.0, 0.0);
            k_scf_antisym<<<ng, th, 0, st>>>(geo, T2, T1);
            k_scf_gemm<<<ng, th, 0, st>>>(geo, X, 1, T1, 0, T2, 1.0, 0.0);
            k_scf_gemm<<<ng, th, 0, st>>>(geo, T2, 0, X, 0, Eh, 1.0, 0.0, d_st, packed);
            k_scf_store_slot<<<ng, th, 0, st>>>(geo, F, Fh, packed, d_st);
            k_scf_diis<<<ng, th, 0, st>>>(geo, Eh, packed, d_st, d_coef);
            k_scf_extrapolate<<<ng, th, 0, st>>>(geo, Fh, packed, d_st, d_coef, Fx);
            Fuse = Fx;
            CK(cudaGetLastError());
        }
        k_scf_copy<<<ng, th, 0, st>>>(geo, D, Dold);
        CKR(density(Fuse, D, nullptr));
        // change of the density: max |D - Dold| (the pass's energy sum lands in scratch)
        k_scf_energy<<<ng, th, 0, st>>>(geo, H, F, D, Dold, d_coef, d_dm);
        k_scf_check<<<1, th, 0, st>>>(d_st, ng, d_e, d_eprev, d_dm, o.thresh_e, o.thresh_d, o.max_iter, h, use_h);
        CK(cudaGetLastError());
        return RCHEM_OK;
    };
    // The whole loop as one graph launch: the iteration captured into the body
    // of a WHILE conditional node whose condition k_scf_check clears on
    // convergence or at max_iter.  Where that cannot be built (the legacy
    // default stream cannot be captured), the host launches one iteration at a
    // time and reads the stop flag after each.
    bool done_in_graph = false;
    const bool capturable = st != nullptr && st != cudaStreamLegacy;
    if (capturable) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        cudaGraphConditionalHandle h = 0;
        bool built = cudaGraphCreate(&g, 0) == cudaSuccess &&
                     cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
        cudaGraph_t body = nullptr;
        if (built) {
            // zeroed raw storage: the struct's union of node kinds has no default constructor
            alignas(cudaGraphNodeParams) unsigned char npbuf[sizeof(cudaGraphNodeParams)];
            memset(npbuf, 0, sizeof(npbuf));
            cudaGraphNodeParams &np = *reinterpret_cast<cudaGraphNodeParams *>(npbuf);
            np.type = cudaGraphNodeTypeConditional;
            np.conditional.handle = h;
            np.conditional.type = cudaGraphCondTypeWhile;
            np.conditional.size = 1;
            cudaGraphNode_t node = nullptr;
            built = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) == cudaSuccess;
            if (built) body = np.conditional.phGraph_out[0];
        }
        if (built && cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                         cudaSuccess) {
            const int rc = iteration(h, 1);
            const cudaError_t ec = cudaStreamEndCapture(st, &body);
            built = rc == RCHEM_OK && ec == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
        } else {
            built = false;
        }
        if (built) {
            NvtxRange nv_loop("scf loop (one graph launch)");
            const cudaError_t el = cudaGraphLaunch(ge, st);
            const cudaError_t es = el == cudaSuccess ? cudaStreamSynchronize(st) : el;
            cudaGraphExecDestroy(ge);
            cudaGraphDestroy(g);
            if (es != cudaSuccess) return set_err(RCHEM_ERR_CUDA, "SCF loop graph: %s", cudaGetErrorString(es));
            done_in_graph = true;
        } else {
            if (ge) cudaGraphExecDestroy(ge);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();  // clear a construction error; the host-driven loop follows
        }
    }
    ScfState hs;
    memset(&hs, 0, sizeof(hs));
    if (done_in_graph) {
        CK(cudaMemcpy(&hs, d_st, sizeof(ScfState), cudaMemcpyDeviceToHost));
    } else {
        for (int k = 0; k < o.max_iter && !hs.stop; ++k) {
            NvtxRange nv_it("scf iteration");
            CKR(iteration(0, 0));
            CK(cudaMemcpyAsync(&hs, d_st, sizeof(ScfState), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
    }
    b->last_stats = b->plan_stats;
    int it = hs.it;
    const bool conv = hs.converged != 0;
    if (it > o.max_iter) it = o.max_iter;
    // energies at the final density with its own Fock matrix; W from that F's orbitals
    CKR(rchem_jk_direct(b, D, J, K, &jo));
    k_scf_fock<<<eb, th, 0, st>>>(packed, H, J, K, F);
    k_scf_energy<<<ng, th, 0, st>>>(geo, H, F, D, nullptr, d_e, d_dm);
    CKR(density(F, Fx, Wm));  // the final D stays; Fx takes the unused new density
    CK(cudaMemcpyAsync(eg.data(), d_e, ng * sizeof(double), cudaMemcpyDeviceToHost, st));
    const cudaMemcpyKind out = o.jk.where == RCHEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (D_out) CK(cudaMemcpyAsync(D_out, D, bytes, out, st));
    if (W_out) CK(cudaMemcpyAsync(W_out, Wm, bytes, out, st));
    CK(cudaStreamSynchronize(st));
    for (int g = 0; g < ng; ++g) {
        if (e_elec) e_elec[g] = eg[g];
        if (e_nuc) {
            const GeomDev &gm = b->geoms[g];
            double en = 0.0;
            for (int a = gm.atom0; a < gm.atom0 + gm.natoms; ++a)
                for (int c = gm.atom0; c < a; ++c) {
                    double r2 = 0.0;
                    for (int x = 0; x < 3; ++x) {
                        const double d = b->R[3 * a + x] - b->R[3 * c + x];
                        r2 += d * d;
                    }
                    en += (double)b->Z[a] * b->Z[c] / std::sqrt(r2);
                }
            e_nuc[g] = en;
        }
    }
    if (iterations) *iterations = it;
    if (converged) *converged = conv ? 1 : 0;
    return RCHEM_OK;
}
