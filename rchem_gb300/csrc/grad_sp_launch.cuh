// grad_sp_launch.cuh -- launcher of the specialised gradient kernels for one
// arithmetic type; each grad_sp_*.cu / grad_sd_*.cu translation unit
// instantiates it for its type and class range so the sets compile in parallel.
#pragma once
#define RCHEM_GRAD_NO_KERNELS  // the run-time-l and one-electron kernels live in rchem_gpu.cu
#include "eri_kernel.cuh"
#include "grad_cls.cuh"

// class index k of the generated class table, launched if lo <= k < hi and the
// class has a specialised kernel (the s/p classes 0..5; 6, 7, 9, 10); false otherwise
template <typename R, int lo = 0, int hi = 6>
bool grad_sp_launch(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    if (k < lo || k >= hi) return false;
    if constexpr (lo <= 0 && 0 < hi) if (k == 0) { k_grad2e_cls<0, 0, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 1 && 1 < hi) if (k == 1) { k_grad2e_cls<1, 0, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 2 && 2 < hi) if (k == 2) { k_grad2e_cls<1, 0, 1, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 3 && 3 < hi) if (k == 3) { k_grad2e_cls<1, 1, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 4 && 4 < hi) if (k == 4) { k_grad2e_cls<1, 1, 1, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 5 && 5 < hi) if (k == 5) { k_grad2e_cls<1, 1, 1, 1, R><<<blocks, 64, 0, st>>>(g); return true; }
    // the smallest classes with a d shell: (ds|ss), (ds|ps), (ds|ds), (dp|ss)
    if constexpr (lo <= 6 && 6 < hi) if (k == 6) { k_grad2e_cls<2, 0, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 7 && 7 < hi) if (k == 7) { k_grad2e_cls<2, 0, 1, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 9 && 9 < hi) if (k == 9) { k_grad2e_cls<2, 0, 2, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    if constexpr (lo <= 10 && 10 < hi) if (k == 10) { k_grad2e_cls<2, 1, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true; }
    return false;
}
