// grad_sd_f64.cu -- the specialised gradient kernels of the smallest classes with
// a d shell, in double arithmetic (a translation unit of their own so they compile
// in parallel with the s/p set).
#include "grad_sp_launch.cuh"

bool rchem_grad_sd_f64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<double, 6, 11>(k, g, blocks, st);
}
