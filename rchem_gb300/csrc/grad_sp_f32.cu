// grad_sp_f32.cu -- the s/p gradient kernels in float arithmetic.
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_f32(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<float>(k, g, blocks, st);
}
