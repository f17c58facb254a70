// grad_sp_f64.cu -- the s/p gradient kernels in double arithmetic but (pp|pp),
// which grad_pppp_f64.cu builds.
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_f64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<double, 0, 5>(k, g, blocks, st);
}
