// grad_sp_df64.cu -- the s/p gradient kernels in double-float arithmetic,
// classes 0..3 here and (pp|ps) in grad_sp_df64b.cu (compiled in parallel);
// false for (pp|pp), which runs FP64.
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_df64b(int k, const GradArgs &g, unsigned blocks, cudaStream_t st);

bool rchem_grad_sp_df64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<df64, 0, 4>(k, g, blocks, st) || rchem_grad_sp_df64b(k, g, blocks, st);
}
