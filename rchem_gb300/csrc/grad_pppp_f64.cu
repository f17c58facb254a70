// grad_pppp_f64.cu -- the (pp|pp) gradient kernel in double arithmetic, a
// translation unit of its own: build.py compiles it with ptxas -O1, where it
// keeps ~6 KB of local memory per thread instead of ~30 KB at -O3.
#include "grad_sp_launch.cuh"

bool rchem_grad_pppp_f64(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<double, 5, 6>(k, g, blocks, st);
}
