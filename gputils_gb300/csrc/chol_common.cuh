// chol_common.cuh -- Cholesky building blocks shared by the uniform-batch
// kernels (chol.cu) and the ragged solver (chol_ragged.cu).
#pragma once
#include "common.cuh"

namespace gbla {

enum CholMode { CH_FACTOR = 1, CH_SOLVE = 2 };

// ------------------------------------------------- lane-row (n <= 32) pieces
template <typename T, int NB>
__device__ __forceinline__ void lr_factor(T (&a)[NB], T &dinv, int &fail, int n, int r) {
#pragma unroll
    for (int k = 0; k < NB; k++) {
        if (k < n) {
            T d = shfl(a[k], k, NB);
            if (!(d > T(0)) && fail == 0) fail = k + 1;
            T l, il;
            if constexpr (sizeof(T) == 4) {
                // reciprocal square root with one Newton step (about 1 ulp),
                // l = d / sqrt(d): a short dependency chain per pivot
                float y = rsqrtf(d);
                y = y * fmaf(-0.5f * d * y, y, 1.5f);
                il = y;
                l = d * y;
            } else {
                l = dev_sqrt<T>(d);
                il = T(1) / l;
            }
            if (r == k) { a[k] = l; dinv = il; }
            else if (r > k) a[k] *= il;
#pragma unroll
            for (int j = k + 1; j < NB; j++) {
                if (j < n) {
                    T ljk = shfl(a[k], j, NB);
                    if (r >= j) a[j] -= a[k] * ljk;
                }
            }
        }
    }
}

// Solve L L^T x = b for one right-hand side held one row per lane.
template <typename T, int NB>
__device__ __forceinline__ T lr_solve(const T (&a)[NB], T dinv, T b, int n, int r) {
#pragma unroll
    for (int k = 0; k < NB; k++) {
        if (k < n) {
            if (r == k) b *= dinv;
            T yk = shfl(b, k, NB);
            if (r > k) b -= a[k] * yk;
        }
    }
#pragma unroll
    for (int k = NB - 1; k >= 0; k--) {
        if (k < n) {
            T part = (r > k && r < n) ? a[k] * b : T(0);
            T s = group_sum(part, NB);
            if (r == k) b = (b - s) * dinv;
        }
    }
    return b;
}

// Solve L L^T x = b with L available both by rows (a: row r in lane r) and by
// columns (at[k] = L(k, r) in lane r): both substitutions are column-oriented,
// one broadcast and one fma per step.
template <typename T, int NB>
__device__ __forceinline__ T lr_solve_cols(const T (&a)[NB], const T (&at)[NB], T dinv, T b, int n, int r) {
#pragma unroll
    for (int k = 0; k < NB; k++) {
        if (k < n) {
            if (r == k) b *= dinv;
            T yk = shfl(b, k, NB);
            if (r > k) b -= a[k] * yk;
        }
    }
#pragma unroll
    for (int k = NB - 1; k >= 0; k--) {
        if (k < n) {
            if (r == k) b *= dinv;
            T xk = shfl(b, k, NB);
            if (r < k) b -= at[k] * xk;
        }
    }
    return b;
}

// ------------------------------------------------------- CTA (n > 32) pieces
constexpr int CTA_THREADS = 256;
constexpr int CTA_WARPS = CTA_THREADS / 32;
constexpr int CTA_RHS_CHUNK = CTA_WARPS;  // one warp per right-hand side

__host__ __device__ inline int cta_ld(int n) { return n | 1; }

// Solve L L^T x = b for the column x (length n, shared memory) with one warp.
template <typename T>
__device__ __forceinline__ void cta_solve_col(const T *__restrict__ a, int ld, const T *__restrict__ dinv,
                                              T *__restrict__ x, int n, int lane) {
    for (int k = 0; k < n; k++) {
        T xk = x[k] * dinv[k];
        for (int i = k + 1 + lane; i < n; i += 32) x[i] -= a[(int64_t)k * ld + i] * xk;
        __syncwarp();
        if (lane == 0) x[k] = xk;
        __syncwarp();
    }
    for (int k = n - 1; k >= 0; k--) {
        T xk = x[k] * dinv[k];
        for (int i = lane; i < k; i += 32) x[i] -= a[(int64_t)i * ld + k] * xk;  // L(k, i)
        __syncwarp();
        if (lane == 0) x[k] = xk;
        __syncwarp();
    }
}

}  // namespace gbla
