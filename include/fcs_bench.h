/*
 * fcs_bench.h -- measurement helpers exported by libfcs_cuda.so.  They have no
 * counterpart in the reference (which has no GPU code); bench.py uses them to
 * measure the roofline denominators of the integrator on the GPU it runs on.
 */
#ifndef FCS_BENCH_H
#define FCS_BENCH_H
#ifdef __cplusplus
extern "C" {
#endif

/* Dense FP64 FMA throughput of the device (TFLOP/s, 2 flops per FMA),
 * measured with independent FMA chains on every SM for about `ms` ms. */
int fcs_bench_fp64_peak(int device, double ms, double* tflops);

/* Same for FP32 FMAs. */
int fcs_bench_fp32_peak(int device, double ms, double* tflops);

/* Evaluates the integrator's table-driven FP64 exp and CUDA's exp on n host
 * arguments (validation of the integrator's exp against CUDA's results). */
int fcs_check_exp(int device, long long n, const double* x, double* fast, double* cuda_exp);

#ifdef __cplusplus
}
#endif
#endif
