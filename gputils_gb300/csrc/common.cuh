// common.cuh -- shared helpers for the sm_103a batched linear-algebra kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "gbla.h"

#define GBLA_API extern "C" __attribute__((visibility("default")))

namespace gbla {

constexpr unsigned FULL = 0xffffffffu;

// Map a CUDA runtime error to the ABI status, remembering the last one for
// gbla_last_cuda_error().
gbla_status from_cuda(cudaError_t e);

// Check the launch that was just enqueued.
inline gbla_status launch_status() { return from_cuda(cudaGetLastError()); }

template <typename T>
__device__ __forceinline__ T shfl(T v, int src, int width = 32) {
    return __shfl_sync(FULL, v, src, width);
}

template <typename T>
__device__ __forceinline__ T shfl_xor(T v, int mask, int width = 32) {
    return __shfl_xor_sync(FULL, v, mask, width);
}

// Sum over a group of `width` consecutive lanes (width a power of two <= 32);
// every lane of the group receives the total.
template <typename T>
__device__ __forceinline__ T group_sum(T v, int width) {
    for (int o = width >> 1; o > 0; o >>= 1) v += shfl_xor(v, o, width);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += shfl_xor(v, o);
    return v;
}

template <typename T> __device__ __forceinline__ T dev_sqrt(T x);
template <> __device__ __forceinline__ float dev_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double dev_sqrt<double>(double x) { return sqrt(x); }

template <typename T> __device__ __forceinline__ T dev_rsqrt(T x);
template <> __device__ __forceinline__ float dev_rsqrt<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double dev_rsqrt<double>(double x) { return rsqrt(x); }

// Number of SMs of the current device (cached per device ordinal).
int sm_count();

// Grid for a persistent kernel: the blocks that can be resident at once
// (occupancy of `func` at this block size and dynamic shared memory, times
// the SM count), at most `work` and at least 1.
int64_t persistent_grid(const void *func, int threads, size_t smem, int64_t work);

// Round x up to a multiple of m.
__host__ __device__ constexpr int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

}  // namespace gbla
