/*
 * rchem_bench.h -- measurement helpers of librchem_gpu.so (no counterpart in
 * the reference, which has no GPU code).
 */
#ifndef RCHEM_BENCH_H
#define RCHEM_BENCH_H

#ifdef __cplusplus
extern "C" {
#endif

/* Sustained FMA throughput of the current device's CUDA cores, in TFLOP/s
 * (FMA = 2 FLOP), precision 64 or 32: the roofline denominator of the ERI
 * kernels.  Returns 0 on success. */
int rchem_peak_fma(int precision, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* RCHEM_BENCH_H */
