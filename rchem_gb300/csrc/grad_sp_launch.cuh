// grad_sp_launch.cuh -- launcher of the specialised s/p gradient kernels for
// one arithmetic type; each grad_sp_*.cu translation unit instantiates it for
// its type so the three sets compile in parallel.
#pragma once
#define RCHEM_GRAD_NO_KERNELS  // the run-time-l and one-electron kernels live in rchem_gpu.cu
#include "eri_kernel.cuh"
#include "grad_cls.cuh"

// class index k of the generated class table (s/p classes only); false if k is
// not an s/p class
template <typename R>
bool grad_sp_launch(int k, const GradArgs &g, unsigned blocks, cudaStream_t st) {
    switch (k) {
        case 0: k_grad2e_cls<0, 0, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true;
        case 1: k_grad2e_cls<1, 0, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true;
        case 2: k_grad2e_cls<1, 0, 1, 0, R><<<blocks, 64, 0, st>>>(g); return true;
        case 3: k_grad2e_cls<1, 1, 0, 0, R><<<blocks, 64, 0, st>>>(g); return true;
        case 4: k_grad2e_cls<1, 1, 1, 0, R><<<blocks, 64, 0, st>>>(g); return true;
        case 5: k_grad2e_cls<1, 1, 1, 1, R><<<blocks, 64, 0, st>>>(g); return true;
        default: return false;
    }
}
