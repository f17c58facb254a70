// grad_sp_df64b.cu -- the (pp|ps) gradient kernel in double-float arithmetic
// (its own translation unit so it compiles beside the others; (pp|pp) has no
// double-float instantiation -- it alone would take minutes to compile -- and
// runs FP64 in the emulated form).
#include "grad_sp_launch.cuh"

bool rchem_grad_sp_df64b(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    return grad_sp_launch<df64, 4, 5>(k, g, blocks, st);
}
