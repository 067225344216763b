// svd_big.cuh -- launcher of the one-sided Jacobi SVD for the shapes beyond
// the warp and 64-column block kernels of svd.cu (defined in svd_big.cu).
#pragma once
#include "common.cuh"

namespace gbla {

// Columns of the largest matrix the big-shape kernel takes (V stays in shared memory).
constexpr int SVD_BIG_MAX_N = 128;

// One-sided Jacobi SVD of m x n matrices (m >= n, n <= SVD_BIG_MAX_N), one
// block per matrix; arguments as svd_launch in svd.cu (validated by the
// caller), no warm start.  A is destroyed.
template <typename T>
gbla_status svd_big_launch(int m, int n, T *A, int64_t sA, T *S, int64_t sS, T *Vt, int64_t sVt, T *U, int64_t sU,
                           T tol, int max_sweeps, int *info, int *sweeps, int batch, cudaStream_t st);

}  // namespace gbla
