// grad_sp_launch.cuh -- launcher of the specialised s/p gradient kernels for
// one arithmetic type; each grad_sp_*.cu translation unit instantiates it for
// its type so the three sets compile in parallel.
#pragma once
#define RCHEM_GRAD_NO_KERNELS  // the run-time-l and one-electron kernels live in rchem_gpu.cu
#include "eri_kernel.cuh"
#include "grad_cls.cuh"

// class index k of the generated class table, launched if lo <= k < hi (the
// s/p classes are 0..5); false otherwise
template <typename R, int lo = 0, int hi = 6>
bool grad_sp_launch(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    if (k < lo || k >= hi) return false;
    if constexpr (lo <= 0 && 0 < hi) if (k == 0) { k_grad2e_cls<0, 0, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 1 && 1 < hi) if (k == 1) { k_grad2e_cls<1, 0, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 2 && 2 < hi) if (k == 2) { k_grad2e_cls<1, 0, 1, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 3 && 3 < hi) if (k == 3) { k_grad2e_cls<1, 1, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 4 && 4 < hi) if (k == 4) { k_grad2e_cls<1, 1, 1, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 5 && 5 < hi) if (k == 5) { k_grad2e_cls<1, 1, 1, 1, R><<<blocks, 64, 0, st>>>(g); return true; }
    return false;
}
