// qr_f64.cu -- FP64 batched QR through the C ABI: geqrf and least squares
// (one warp per matrix; FP64 needs no refinement), ormqr and the
// upper-triangular solve.
#include "qr_common.cuh"

using namespace gbla;

GBLA_API gbla_status gbla_dgeqrf_batched(int m, int n, double *A, int64_t sA, double *tau, int64_t sTau, int *info,
                                         int batch, cudaStream_t st) {
    return qr_launch<double>(m, n, 0, A, sA, nullptr, 0, tau, sTau, info, QR_WRITE_FACTORS | QR_WRITE_TAU, 0, batch,
                             st);
}
GBLA_API gbla_status gbla_dgels_batched(int m, int n, int nrhs, double *A, int64_t sA, double *B, int64_t sB,
                                        int *info, int batch, cudaStream_t st) {
    return qr_launch<double>(m, n, nrhs, A, sA, B, sB, nullptr, 0, info, QR_WRITE_FACTORS | QR_SOLVE, 0, batch, st);
}
GBLA_API gbla_status gbla_dormqr_batched(int trans, int m, int nc, int k, const double *A, int64_t sA,
                                         const double *tau, int64_t sTau, double *Cm, int64_t sC, int batch,
                                         cudaStream_t st) {
    return ormqr_launch<double>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, batch, st);
}
GBLA_API gbla_status gbla_dtrsm_upper_batched(int n, int nc, const double *Rm, int64_t ldr, int64_t sR, double *Bm,
                                              int64_t ldb, int64_t sB, int batch, cudaStream_t st) {
    return trsm_launch<double>(n, nc, Rm, ldr, sR, Bm, ldb, sB, batch, st);
}
