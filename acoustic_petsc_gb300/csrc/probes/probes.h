/* probes.h -- test and measurement support built into libhype_probes.so, kept out of the
 * library's public C ABI (include/hype_gpu.h).  Neither entry point is on the solver path. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
/* Measured FMA issue ceiling of the FP64 (precision 0) or FP32 (precision 1) pipe of the
 * current device, in TFLOP/s (about 20 ms of GPU time). */
int hype_probe_fma_peak(int precision, double* tflops);
/* Double-float primitives of df64.cuh, elementwise: for each x[q], y[q] (|x|, |y| in the
 * FP32 normal range), out[7q..7q+6] = the FP32 pair (hi, lo) of x as FP64 values, hi + lo,
 * and x + y, x - y, x * y, x / y in double-float arithmetic, each converted back to FP64. */
int hype_df64_probe(const double* x, const double* y, long long n, double* out);
#ifdef __cplusplus
}
#endif
