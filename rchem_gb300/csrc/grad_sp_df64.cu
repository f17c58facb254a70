// grad_sp_df64.cu -- the s/p gradient kernels in double-float arithmetic.
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_df64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<df64>(k, g, blocks, st);
}
