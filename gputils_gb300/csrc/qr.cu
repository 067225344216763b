// qr.cu -- FP32 batched QR through the C ABI: geqrf (one warp per matrix,
// factor-only variant), ormqr, the upper-triangular solve, and the
// two-kernel least squares (warp factorisation into a workspace, then one
// block per system solving from shared memory).
#include "qr_common.cuh"

namespace gbla {

// workspace of gbla_sgels_batched_ws: factors (batch x m x n) + taus (batch x 32)
static size_t gels_ws_bytes(int m, int n, int batch) {
    if (m < 0 || n < 0 || batch < 0) return 0;
    return sizeof(float) * ((size_t)batch * m * n + (size_t)batch * 32) + 256;
}

static gbla_status gels_ws_launch(int m, int n, int nrhs, float *A, int64_t sA, float *B, int64_t sB, int *info,
                                  int refine, void *ws, size_t ws_bytes, int batch, cudaStream_t st) {
    if (m < 0 || n < 0 || nrhs < 0 || batch < 0 || refine < 0 || m < n) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0) return GBLA_SUCCESS;
    if (!A || sA < (int64_t)m * n || (nrhs > 0 && (!B || sB < (int64_t)m * nrhs))) return GBLA_INVALID_VALUE;
    if (m > 128 || n > 32) return GBLA_NOT_SUPPORTED;
    if (!ws || ws_bytes < gels_ws_bytes(m, n, batch)) return GBLA_WORKSPACE_TOO_SMALL;
    float *F = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(ws) + 15) & ~uintptr_t(15));
    float *tau = F + (size_t)batch * m * n;
    const int R = (m + 31) / 32;
    const unsigned g1 = (unsigned)((batch + 3) / 4);
    const size_t smem2 = sizeof(float) * ((size_t)32 * (32 * R + 1) + (refine > 0 ? 32 * 32 * R : 0) + 32);
    auto go = [&](auto kf, auto ks) -> gbla_status {
        kf<<<g1, 128, 0, st>>>(m, n, 0, A, sA, nullptr, 0, tau, 32, info, QR_WRITE_FACTORS | QR_WRITE_TAU, batch, F,
                               (int64_t)m * n);
        gbla_status s = launch_status();
        if (s != GBLA_SUCCESS) return s;
        if (smem2 > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
            if (e != cudaSuccess) return from_cuda(e);
        }
        ks<<<(unsigned)batch, 128, smem2, st>>>(m, n, nrhs, A, sA, F, tau, B, sB, refine, batch);
        return launch_status();
    };
    switch (R) {
        case 1: return go(k_qr_warp<float, 1, false>, k_ls_solve<1>);
        case 2: return go(k_qr_warp<float, 2, false>, k_ls_solve<2>);
        case 3: return go(k_qr_warp<float, 3, false>, k_ls_solve<3>);
        default: return go(k_qr_warp<float, 4, false>, k_ls_solve<4>);
    }
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_sgeqrf_batched(int m, int n, float *A, int64_t sA, float *tau, int64_t sTau, int *info,
                                         int batch, cudaStream_t st) {
    return qr_launch<float>(m, n, 0, A, sA, nullptr, 0, tau, sTau, info, QR_WRITE_FACTORS | QR_WRITE_TAU, 0, batch, st);
}
GBLA_API size_t gbla_sgels_batched_workspace_bytes(int m, int n, int batch) { return gels_ws_bytes(m, n, batch); }
GBLA_API gbla_status gbla_sgels_batched_ws(int m, int n, int nrhs, float *A, int64_t sA, float *B, int64_t sB,
                                           int *info, int refine, void *workspace, size_t workspace_bytes, int batch,
                                           cudaStream_t st) {
    return gels_ws_launch(m, n, nrhs, A, sA, B, sB, info, refine, workspace, workspace_bytes, batch, st);
}
GBLA_API gbla_status gbla_sormqr_batched(int trans, int m, int nc, int k, const float *A, int64_t sA, const float *tau,
                                         int64_t sTau, float *Cm, int64_t sC, int batch, cudaStream_t st) {
    return ormqr_launch<float>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, batch, st);
}
GBLA_API gbla_status gbla_strsm_upper_batched(int n, int nc, const float *Rm, int64_t ldr, int64_t sR, float *Bm,
                                              int64_t ldb, int64_t sB, int batch, cudaStream_t st) {
    return trsm_launch<float>(n, nc, Rm, ldr, sR, Bm, ldb, sB, batch, st);
}
