// peak_probe.cu -- FMA throughput probe for the benchmark's roofline
// denominators of the CUDA-core-bound kernels (the machine's measured peaks
// cover HBM bandwidth and BF16 tensor throughput only, not FP32 FFMA or FP64
// DFMA).  Built into its own bench-only library (baseline/libpeak_probe.so);
// nothing in libgbla.so calls it.  bench.py runs it at start-up while it
// samples the SM clock, and reports the rate beside that clock.
#include <cuda_runtime.h>

namespace {

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

}  // namespace

// Measured FMA rate of the current device (precision 32 or 64) in GFLOP/s:
// 8 blocks of 256 threads per SM, each thread 8 independent FMA chains; the
// second of two runs is timed.  Returns 0 or a cudaError_t code.
extern "C" __attribute__((visibility("default"))) int peak_fma_throughput(int precision, int iters, double *gflops,
                                                                          double *ms) {
    if (!gflops || iters <= 0 || (precision != 32 && precision != 64)) return (int)cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8;
    void *out = nullptr;
    cudaEvent_t e0, e1;
    cudaError_t err = cudaMalloc(&out, sizeof(double) * blocks);
    if (err != cudaSuccess) return (int)err;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int rep = 0; rep < 2; rep++) {  // first run warms up
        cudaEventRecord(e0);
        if (precision == 32) k_fma_probe<float><<<blocks, 256>>>(iters, 1.0f, (float *)out);
        else k_fma_probe<double><<<blocks, 256>>>(iters, 1.0, (double *)out);
        cudaEventRecord(e1);
    }
    err = cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * 16 * 8 * (double)iters * blocks * 256;
    *gflops = flops / (t * 1e-3) / 1e9;
    if (ms) *ms = t;
    return (int)err;
}
