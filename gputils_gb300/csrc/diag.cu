// diag.cu -- arithmetic-throughput probe used for the roofline denominators
// of the CUDA-core-bound kernels (the measured peak figures cover HBM
// bandwidth and BF16 tensor throughput only, not FP32 FFMA or FP64 DFMA).
#include "common.cuh"

namespace gbla {

// 8 independent FMA chains per thread keep the pipes full.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(int iters, T seed, T *out) {
    T a[8];
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = seed + T(threadIdx.x + i);
    const T x = T(0.999999), y = T(1e-7);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 16; u++)
#pragma unroll
            for (int i = 0; i < 8; i++) a[i] = fma(a[i], x, y);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += a[i];
    if (s == T(-12345)) out[blockIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_diag_fma_throughput(int precision, int iters, double *gflops, double *ms) {
    if (!gflops || iters <= 0 || (precision != 32 && precision != 64)) return GBLA_INVALID_VALUE;
    int blocks = sm_count() * 8;
    void *out = nullptr;
    cudaEvent_t e0, e1;
    gbla_status s = from_cuda(cudaMalloc(&out, sizeof(double) * blocks));
    if (s != GBLA_SUCCESS) return s;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int rep = 0; rep < 2; rep++) {  // first run warms up
        cudaEventRecord(e0);
        if (precision == 32) k_fma_probe<float><<<blocks, 256>>>(iters, 1.0f, (float *)out);
        else k_fma_probe<double><<<blocks, 256>>>(iters, 1.0, (double *)out);
        cudaEventRecord(e1);
    }
    s = from_cuda(cudaEventSynchronize(e1));
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * 16 * 8 * (double)iters * blocks * 256;
    *gflops = flops / (t * 1e-3) / 1e9;
    if (ms) *ms = t;
    return s;
}
