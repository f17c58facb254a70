// grad_sp_f32.cu -- the gradient kernels in float arithmetic (s/p classes and the
// two kernels of the classes with d shells).
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_f32(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<float>(k, g, blocks, st);
}

// the smaller d classes, one lane group per quartet
void rchem_grad_rt_f32(const GradArgs &g, unsigned blocks, cudaStream_t st) {
    k_grad2e_rt<float><<<blocks, 64, 0, st>>>(g);
}

// the larger d classes, one quartet per warp (blocks of GW_WARPS warps); false if the
// shared-memory limit cannot be raised
bool rchem_grad_wc_f32(const GradArgs &g, unsigned blocks, cudaStream_t st) {
    const size_t smem = (size_t)GW_WARPS * GW_PER_WARP * sizeof(float);
    if (cudaFuncSetAttribute(k_grad2e_wc<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return false;
    k_grad2e_wc<float><<<blocks, 32 * GW_WARPS, smem, st>>>(g);
    return true;
}
