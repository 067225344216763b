// gemm.cu -- batched GEMM, FFMA path (any shape, float and double) and the
// dispatcher that routes eligible single-precision shapes to the tcgen05
// split-precision kernel (gemm_tc.cu).
//
// FFMA kernel: one 64x64 tile of C per block, 256 threads, 4x4 register tile
// per thread, K staged through shared memory in slabs of 16 with a
// register double buffer for the next slab.
#include "common.cuh"

namespace gbla {

// implemented in gemm_tc.cu
bool tc_gemm_eligible(int m, int n, int k, int64_t sA, int64_t sB, int64_t sC, const void *A, const void *B,
                      const void *C);
gbla_status tc_sgemm_bf16x6(int m, int n, int k, float alpha, const float *A, int64_t sA, const float *B,
                            int64_t sB, float beta, float *C, int64_t sC, int batch, cudaStream_t st);

constexpr int GB_M = 64, GB_N = 64, GB_K = 16, GB_THREADS = 256;

template <typename T>
__global__ void __launch_bounds__(GB_THREADS) k_gemm_ffma(int m, int n, int k, T alpha, const T *__restrict__ A,
                                                          int64_t sA, const T *__restrict__ B, int64_t sB, T beta,
                                                          T *__restrict__ C, int64_t sC, int batch) {
    __shared__ __align__(16) T As[GB_K][GB_M + 4];
    __shared__ __align__(16) T Bs[GB_K][GB_N + 4];
    const int t = threadIdx.x;
    const int rg = t % 16, cg = t / 16;  // rows rg*4..+3, cols cg*4..+3
    const int i0 = blockIdx.y * GB_M, j0 = blockIdx.x * GB_N;
    // tile loaders: A tile 64 x 16 (4 elements / thread), B tile 16 x 64
    const int la_i = t % 64, la_k = t / 64;   // A: rows along threads, k = la_k + 4*s
    const int lb_k = t % 16, lb_j = t / 16;   // B: k along threads, j = lb_j + 16*s
    for (int64_t b = blockIdx.z; b < batch; b += gridDim.z) {
        const T *a = A + b * sA;
        const T *bb = B + b * sB;
        T acc[4][4];
#pragma unroll
        for (int x = 0; x < 4; x++)
#pragma unroll
            for (int y = 0; y < 4; y++) acc[x][y] = T(0);
        T ra[4], rb[4];
        auto load = [&](int kk0) {
#pragma unroll
            for (int s = 0; s < 4; s++) {
                int i = i0 + la_i, kk = kk0 + la_k + 4 * s;
                ra[s] = (i < m && kk < k) ? a[(int64_t)kk * m + i] : T(0);
                int j = j0 + lb_j + 16 * s, kb = kk0 + lb_k;
                rb[s] = (j < n && kb < k) ? bb[(int64_t)j * k + kb] : T(0);
            }
        };
        load(0);
        for (int kk0 = 0; kk0 < k; kk0 += GB_K) {
            __syncthreads();
#pragma unroll
            for (int s = 0; s < 4; s++) {
                As[la_k + 4 * s][la_i] = ra[s];
                Bs[lb_k][lb_j + 16 * s] = rb[s];
            }
            __syncthreads();
            if (kk0 + GB_K < k) load(kk0 + GB_K);
#pragma unroll
            for (int kk = 0; kk < GB_K; kk++) {
                T av[4], bv[4];
#pragma unroll
                for (int x = 0; x < 4; x++) av[x] = As[kk][rg * 4 + x];
#pragma unroll
                for (int y = 0; y < 4; y++) bv[y] = Bs[kk][cg * 4 + y];
#pragma unroll
                for (int x = 0; x < 4; x++)
#pragma unroll
                    for (int y = 0; y < 4; y++) acc[x][y] = fma(av[x], bv[y], acc[x][y]);
            }
        }
        T *c = C + b * sC;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            int j = j0 + cg * 4 + y;
            if (j >= n) continue;
#pragma unroll
            for (int x = 0; x < 4; x++) {
                int i = i0 + rg * 4 + x;
                if (i >= m) continue;
                T v = alpha * acc[x][y];
                if (beta != T(0)) v = fma(beta, c[(int64_t)j * m + i], v);
                c[(int64_t)j * m + i] = v;
            }
        }
    }
}

template <typename T>
__global__ void k_gemm_scale_c(int64_t mn, T beta, T *__restrict__ C, int64_t sC, int batch) {
    for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
        for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mn; e += (int64_t)gridDim.x * blockDim.x)
            C[b * sC + e] = beta == T(0) ? T(0) : beta * C[b * sC + e];
}

static bool overlaps(const void *p, int64_t bytes_p, const void *q, int64_t bytes_q) {
    const char *a = (const char *)p, *b = (const char *)q;
    return a < b + bytes_q && b < a + bytes_p;
}

template <typename T>
static gbla_status gemm_ffma(int m, int n, int k, T alpha, const T *A, int64_t sA, const T *B, int64_t sB, T beta,
                             T *C, int64_t sC, int batch, cudaStream_t st) {
    if (k == 0 || alpha == T(0)) {
        dim3 grid((unsigned)((int64_t)m * n + 255) / 256 < 4096 ? (unsigned)(((int64_t)m * n + 255) / 256) : 4096,
                  batch < 65535 ? batch : 65535);
        k_gemm_scale_c<T><<<grid, 256, 0, st>>>((int64_t)m * n, beta, C, sC, batch);
        return launch_status();
    }
    dim3 grid((n + GB_N - 1) / GB_N, (m + GB_M - 1) / GB_M, batch < 65535 ? batch : 65535);
    k_gemm_ffma<T><<<grid, GB_THREADS, 0, st>>>(m, n, k, alpha, A, sA, B, sB, beta, C, sC, batch);
    return launch_status();
}

template <typename T>
static gbla_status gemm_check(int m, int n, int k, const T *A, int64_t sA, const T *B, int64_t sB, T *C,
                              int64_t sC, int batch) {
    if (m < 0 || n < 0 || k < 0 || batch < 0) return GBLA_INVALID_VALUE;
    if ((int64_t)m * n == 0 || batch == 0) return GBLA_SUCCESS;
    if (!C || sC < (int64_t)m * n) return GBLA_INVALID_VALUE;
    if (k > 0 && (!A || !B || sA < (int64_t)m * k || sB < (int64_t)k * n)) return GBLA_INVALID_VALUE;
    if (k > 0) {
        int64_t bytesC = ((int64_t)(batch - 1) * sC + (int64_t)m * n) * (int64_t)sizeof(T);
        int64_t bytesA = ((int64_t)(batch - 1) * sA + (int64_t)m * k) * (int64_t)sizeof(T);
        int64_t bytesB = ((int64_t)(batch - 1) * sB + (int64_t)k * n) * (int64_t)sizeof(T);
        if (overlaps(C, bytesC, A, bytesA) || overlaps(C, bytesC, B, bytesB)) return GBLA_INVALID_VALUE;
    }
    return GBLA_SUCCESS;
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_sgemm_batched(int m, int n, int k, float alpha, const float *A, int64_t sA, const float *B,
                                        int64_t sB, float beta, float *C, int64_t sC, int batch, gbla_gemm_mode mode,
                                        cudaStream_t st) {
    gbla_status s = gemm_check<float>(m, n, k, A, sA, B, sB, C, sC, batch);
    if (s != GBLA_SUCCESS || (int64_t)m * n == 0 || batch == 0) return s;
    if (mode != GBLA_GEMM_AUTO && mode != GBLA_GEMM_FP32 && mode != GBLA_GEMM_BF16X6) return GBLA_INVALID_VALUE;
    bool tc_ok = k > 0 && alpha != 0.0f && tc_gemm_eligible(m, n, k, sA, sB, sC, A, B, C);
    if (mode == GBLA_GEMM_BF16X6 && !tc_ok) return GBLA_NOT_SUPPORTED;
    if (tc_ok && mode != GBLA_GEMM_FP32) return tc_sgemm_bf16x6(m, n, k, alpha, A, sA, B, sB, beta, C, sC, batch, st);
    return gemm_ffma<float>(m, n, k, alpha, A, sA, B, sB, beta, C, sC, batch, st);
}

GBLA_API gbla_status gbla_dgemm_batched(int m, int n, int k, double alpha, const double *A, int64_t sA,
                                        const double *B, int64_t sB, double beta, double *C, int64_t sC, int batch,
                                        cudaStream_t st) {
    gbla_status s = gemm_check<double>(m, n, k, A, sA, B, sB, C, sC, batch);
    if (s != GBLA_SUCCESS || (int64_t)m * n == 0 || batch == 0) return s;
    return gemm_ffma<double>(m, n, k, alpha, A, sA, B, sB, beta, C, sC, batch, st);
}
