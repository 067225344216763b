// ref_path.cu -- the reference's library call sequence, for measurement only.
//
// GPUtils' hot path is a thin layer over cuBLAS / cuSOLVER (include/tensor.cuh).
// The reference source is not available where the benchmark runs, so this
// file re-issues the same library calls with the same arguments that
// tensor.cuh makes, so that bench.py can time "the reference's
// cuBLAS/cuSOLVER-backed build" on the same GPU and inputs.  It is never
// linked into libgbla.so and nothing in the product calls it.
//
//   refp_sgemm_batched  cublasSgemmBatched(N, N, ...) with pointer arrays  tensor.cuh:1321-1328
//   refp_sgels_batched  DTensor<int> info alloc + cublasSgelsBatched       tensor.cuh:1369-1393
//   refp_spotrf_batched cusolverDnSpotrfBatched(LOWER)                      tensor.cuh:2149-2159
//   refp_spotrs_batched cusolverDnSpotrsBatched(LOWER, nrhs = 1)            tensor.cuh:2180-2197
//   refp_sgesvd_loop    host loop of cusolverDnSgesvd('A'|'N', 'A')          tensor.cuh:1651-1676
//   refp_spotrf         CholeskyFactoriser<float>: workspace sized once
//                       (cusolverDnSpotrf_bufferSize), factorise = cusolverDnSpotrf(LOWER)
//                                                                            tensor.cuh:1703-1709, 1735-1740, 1754-1761
//   refp_spotrs         CholeskyFactoriser<float>::solve: cusolverDnSpotrs   tensor.cuh:1775-1783
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#define REFP_API extern "C" __attribute__((visibility("default")))

static cublasHandle_t g_blas = nullptr;
static cusolverDnHandle_t g_solver = nullptr;

REFP_API int refp_init(void *stream) {
    if (!g_blas && cublasCreate(&g_blas) != CUBLAS_STATUS_SUCCESS) return 1;
    if (!g_solver && cusolverDnCreate(&g_solver) != CUSOLVER_STATUS_SUCCESS) return 2;
    if (cublasSetStream(g_blas, (cudaStream_t)stream) != CUBLAS_STATUS_SUCCESS) return 3;
    if (cusolverDnSetStream(g_solver, (cudaStream_t)stream) != CUSOLVER_STATUS_SUCCESS) return 4;
    return 0;
}

REFP_API int refp_sgemm_batched(int m, int n, int k, float alpha, const float **A, const float **B, float beta,
                                float **C, int batch) {
    return (int)cublasSgemmBatched(g_blas, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &alpha, A, m, B, k, &beta, C, m, batch);
}

// one leastSquaresBatched call: nrhs = 1, with the per-call info array the
// reference allocates and frees (tensor.cuh:1381)
REFP_API int refp_sgels_batched(int m, int n, float **A, float **B, int batch, int *host_info) {
    int *dinfo = nullptr;
    if (cudaMalloc(&dinfo, sizeof(int) * (size_t)batch) != cudaSuccess) return 100;
    int info = 0;
    int st = (int)cublasSgelsBatched(g_blas, CUBLAS_OP_N, m, n, 1, A, m, B, m, &info, dinfo, batch);
    cudaFree(dinfo);
    if (host_info) *host_info = info;
    return st;
}

REFP_API int refp_spotrf_batched(int n, float **A, int *info, int batch) {
    return (int)cusolverDnSpotrfBatched(g_solver, CUBLAS_FILL_MODE_LOWER, n, A, n, info, batch);
}

REFP_API int refp_spotrs_batched(int n, float **A, float **B, int *info, int batch) {
    return (int)cusolverDnSpotrsBatched(g_solver, CUBLAS_FILL_MODE_LOWER, n, 1, A, n, B, n, info, batch);
}

REFP_API int refp_spotrf_bufsize(int n, int *lwork) {
    return (int)cusolverDnSpotrf_bufferSize(g_solver, CUBLAS_FILL_MODE_LOWER, n, nullptr, n, lwork);
}

REFP_API int refp_spotrf(int n, float *A, float *work, int lwork, int *info) {
    return (int)cusolverDnSpotrf(g_solver, CUBLAS_FILL_MODE_LOWER, n, A, n, work, lwork, info);
}

// CholeskyFactoriser<float>::solve: cusolverDnSpotrs(LOWER, nrhs = 1)      tensor.cuh:1775-1783
REFP_API int refp_spotrs(int n, const float *A, float *B, int *info) {
    return (int)cusolverDnSpotrs(g_solver, CUBLAS_FILL_MODE_LOWER, n, 1, A, n, B, n, info);
}

REFP_API int refp_dpotrf_batched(int n, double **A, int *info, int batch) {
    return (int)cusolverDnDpotrfBatched(g_solver, CUBLAS_FILL_MODE_LOWER, n, A, n, info, batch);
}

REFP_API int refp_dpotrs_batched(int n, double **A, double **B, int *info, int batch) {
    return (int)cusolverDnDpotrsBatched(g_solver, CUBLAS_FILL_MODE_LOWER, n, 1, A, n, B, n, info, batch);
}

REFP_API int refp_sgesvd_lwork(int m, int n) {
    int lwork = 0;
    if (cusolverDnSgesvd_bufferSize(g_solver, m, n, &lwork) != CUSOLVER_STATUS_SUCCESS) return -1;
    return lwork;
}

// Svd<float>::factorise: one gesvd per matrix on the same workspace
REFP_API int refp_sgesvd_loop(int m, int n, float *A, float *S, float *U, float *Vt, float *work, int lwork,
                              int *info, int batch, int computeU) {
    int minmn = m < n ? m : n;
    for (int i = 0; i < batch; i++) {
        int st = (int)cusolverDnSgesvd(g_solver, computeU ? 'A' : 'N', 'A', m, n, A + (size_t)i * m * n, m,
                                       S + (size_t)i * minmn, computeU ? U + (size_t)i * m * m : nullptr, m,
                                       Vt + (size_t)i * n * n, n, work, lwork, nullptr, info + i);
        if (st) return st;
    }
    return 0;
}
