// peak.cu -- FMA-throughput probe used by the benchmark as the roofline
// denominator of the FP64 / FP32 CUDA-core pipes (the ERI kernels are bound by
// FP64 FMA issue, not by HBM or tensor cores).  Each thread runs 8
// independent FMA chains; the grid fills every SM several times over.
#include <cuda_runtime.h>

#include "../../include/rchem_bench.h"

template <typename R>
__global__ void k_fma_loop(int iters, R seed, R *sink) {
    R a0 = seed + threadIdx.x, a1 = a0 + R(1), a2 = a0 + R(2), a3 = a0 + R(3);
    R a4 = a0 + R(4), a5 = a0 + R(5), a6 = a0 + R(6), a7 = a0 + R(7);
    const R m = R(0.999999), c = R(1e-7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
            a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
        }
    }
    const R s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == R(-12345)) sink[0] = s;  // keeps the chains live; never true
}

extern "C" int rchem_peak_fma(int precision, double *tflops) {
    if (!tflops || (precision != 64 && precision != 32)) return 1;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 3;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 3;
    void *sink = nullptr;
    if (cudaMalloc(&sink, 16) != cudaSuccess) return 4;
    const int threads = 256, blocks = sms * 8;
    const int iters = precision == 64 ? 256 : 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (precision == 64) k_fma_loop<double><<<blocks, threads>>>(iters, 1.0, (double *)sink);
        else k_fma_loop<float><<<blocks, threads>>>(iters, 1.0f, (float *)sink);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // first launch is a warm-up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (cudaGetLastError() != cudaSuccess) return 3;
    const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return 0;
}
