// grad_sp_df64.cu -- the gradient kernels in df64 arithmetic (s/p classes and the
// run-time-l kernel of the classes with d shells).
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_df64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<df64>(k, g, blocks, st);
}

void rchem_grad_rt_df64(const GradArgs &g, unsigned blocks, cudaStream_t st) {
    k_grad2e_rt<df64><<<blocks, 64, 0, st>>>(g);
}
