// onee_cls.cu -- launcher of the shell-pair one-electron kernels (onee_cls.cuh).
#define RCHEM_GRAD_NO_KERNELS  // the gradient kernels live in rchem_gpu.cu and grad_sp_*.cu
#include "onee_cls.cuh"

template <int LA, int LB, int KIND>
static void launch_one(int n, const OneePair *pairs, const ShellGrad *sh, const double *pexp, const double *pcoef,
                       const double *Z, const double *R, const double *boys, double *out, cudaStream_t st) {
    if (n <= 0) return;
    const int th = 128;
    k_onee_cls<LA, LB, KIND><<<(unsigned)((n + th - 1) / th), th, 0, st>>>(n, pairs, sh, pexp, pcoef, Z, R, boys, out);
}

template <int KIND>
static void launch_kind(const int *begin, const OneePair *pairs, const ShellGrad *sh, const double *pexp,
                        const double *pcoef, const double *Z, const double *R, const double *boys, double *out,
                        cudaStream_t st) {
#define RCHEM_ONEE_CLS(la, lb)                                                                                     \
    launch_one<la, lb, KIND>(begin[la * 3 + lb + 1] - begin[la * 3 + lb], pairs + begin[la * 3 + lb], sh, pexp, \
                             pcoef, Z, R, boys, out, st)
    RCHEM_ONEE_CLS(0, 0);
    RCHEM_ONEE_CLS(0, 1);
    RCHEM_ONEE_CLS(0, 2);
    RCHEM_ONEE_CLS(1, 0);
    RCHEM_ONEE_CLS(1, 1);
    RCHEM_ONEE_CLS(1, 2);
    RCHEM_ONEE_CLS(2, 0);
    RCHEM_ONEE_CLS(2, 1);
    RCHEM_ONEE_CLS(2, 2);
#undef RCHEM_ONEE_CLS
}

// kind: RCHEM_ONEE_S, _T, _V or _H; pairs of class la*3+lb at [begin[c], begin[c+1]).
// false for another kind.
bool rchem_onee_cls_launch(int kind, const int *begin, const OneePair *pairs, const ShellGrad *sh,
                           const double *pexp, const double *pcoef, const double *Z, const double *R,
                           const double *boys, double *out, cudaStream_t st) {
    switch (kind) {
        case RCHEM_ONEE_S: launch_kind<RCHEM_ONEE_S>(begin, pairs, sh, pexp, pcoef, Z, R, boys, out, st); return true;
        case RCHEM_ONEE_T: launch_kind<RCHEM_ONEE_T>(begin, pairs, sh, pexp, pcoef, Z, R, boys, out, st); return true;
        case RCHEM_ONEE_V: launch_kind<RCHEM_ONEE_V>(begin, pairs, sh, pexp, pcoef, Z, R, boys, out, st); return true;
        case RCHEM_ONEE_H: launch_kind<RCHEM_ONEE_H>(begin, pairs, sh, pexp, pcoef, Z, R, boys, out, st); return true;
        default: return false;
    }
}
