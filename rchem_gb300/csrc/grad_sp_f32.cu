// grad_sp_f32.cu -- the gradient kernels in float arithmetic (s/p classes and the
// run-time-l kernel of the classes with d shells).
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_f32(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<float>(k, g, blocks, st);
}

void rchem_grad_rt_f32(const GradArgs &g, unsigned blocks, cudaStream_t st) {
    k_grad2e_rt<float><<<blocks, 64, 0, st>>>(g);
}
