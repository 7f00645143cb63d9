// fcs_peak.cu -- FMA throughput probes (include/fcs_bench.h): 8 independent
// FMA chains per thread, enough resident warps per SM to cover the pipe
// latency, timed with CUDA events.  The result is the FP64 / FP32 roofline
// denominator of the integrator kernels.
#include <cuda_runtime.h>
#include "../../include/fcs_bench.h"
#include "fcs_device.cuh"

namespace {

template<class T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == T(-1)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains alive
}

template<class T>
int peak(int device, double ms, double* tflops) {
    if (!tflops) return 1;
    if (cudaSetDevice(device) != cudaSuccess) return 2;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 256, grid = sms * 8;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * block * grid) != cudaSuccess) return 3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int iters = 64;
    double best = 0;
    for (int rep = 0; rep < 12; rep++) {
        cudaEventRecord(e0);
        fma_chains<T><<<grid, block>>>(out, iters, T(0.999999), T(1e-7));
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        const double flops = 2.0 * 64.0 * iters * (double)block * grid;
        const double tf = flops / (t * 1e-3) / 1e12;
        if (tf > best) best = tf;
        if (t < ms && iters < (1 << 24)) iters *= 2;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    *tflops = best;
    return cudaGetLastError() == cudaSuccess ? 0 : 4;
}

}  // namespace

extern "C" int fcs_bench_fp64_peak(int device, double ms, double* tflops) { return peak<double>(device, ms, tflops); }
extern "C" int fcs_bench_fp32_peak(int device, double ms, double* tflops) { return peak<float>(device, ms, tflops); }

namespace {
__global__ void exp_pair(const double* x, double* a, double* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        a[i] = fcs::fast_exp(x[i]);
        b[i] = exp(x[i]);
    }
}
}  // namespace

extern "C" int fcs_check_exp(int device, long long n, const double* x, double* fast, double* cuda_exp) {
    if (n <= 0 || !x || !fast || !cuda_exp) return 1;
    if (cudaSetDevice(device) != cudaSuccess) return 2;
    double *dx = nullptr, *da = nullptr, *db = nullptr;
    if (cudaMalloc(&dx, n * 8) != cudaSuccess || cudaMalloc(&da, n * 8) != cudaSuccess ||
        cudaMalloc(&db, n * 8) != cudaSuccess) {
        cudaFree(dx); cudaFree(da); cudaFree(db);
        return 3;
    }
    cudaMemcpy(dx, x, n * 8, cudaMemcpyHostToDevice);
    exp_pair<<<1024, 256>>>(dx, da, db, n);
    cudaMemcpy(fast, da, n * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(cuda_exp, db, n * 8, cudaMemcpyDeviceToHost);
    cudaFree(dx); cudaFree(da); cudaFree(db);
    return cudaGetLastError() == cudaSuccess ? 0 : 4;
}
