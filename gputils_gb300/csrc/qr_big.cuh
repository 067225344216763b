// qr_big.cuh -- QR launchers for the shapes beyond the warp kernels
// (any m >= n), defined in qr_cta.cu, and the flags shared by all QR kernels.
#pragma once
#include "common.cuh"

namespace gbla {

enum QrFlags { QR_WRITE_FACTORS = 1, QR_WRITE_TAU = 2, QR_SOLVE = 4 };

// Householder QR (and, with QR_SOLVE, least squares) of m x n matrices, one
// block per matrix; arguments as qr_launch in qr_common.cuh (already
// validated by the caller).  GBLA_NOT_SUPPORTED when single-precision
// refinement is requested for a matrix too large for shared memory.
template <typename T>
gbla_status qr_big_launch(int m, int n, int nrhs, T *A, int64_t sA, T *B, int64_t sB, T *tau, int64_t sTau,
                          int *info, int flags, int refine, int batch, cudaStream_t st);

// C_i <- Q_i^T C_i (trans) or Q_i C_i for any m; arguments as ormqr_launch.
template <typename T>
gbla_status ormqr_big_launch(int trans, int m, int nc, int k, const T *A, int64_t sA, const T *tau, int64_t sTau,
                             T *Cm, int64_t sC, int batch, cudaStream_t st);

}  // namespace gbla
