// gels.cu -- FP32 least squares through the C ABI: the fused
// one-block-per-system kernel (k_gels_cta in qr_common.cuh).
#include "qr_common.cuh"

namespace gbla {

// Single-precision least squares, one block per system (k_gels_cta).
static gbla_status gels_cta_launch(int m, int n, int nrhs, float *A, int64_t sA, float *B, int64_t sB, int *info,
                                   int refine, int batch, cudaStream_t st) {
    if (m < 0 || n < 0 || nrhs < 0 || batch < 0 || refine < 0 || m < n) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0) return GBLA_SUCCESS;
    if (!A || sA < (int64_t)m * n || (nrhs > 0 && (!B || sB < (int64_t)m * nrhs))) return GBLA_INVALID_VALUE;
    if (m > 128 || n > 32)
        return qr_big_launch<float>(m, n, nrhs, A, sA, B, sB, nullptr, 0, info, QR_WRITE_FACTORS | QR_SOLVE, refine,
                                    batch, st);
    const int R = (m + 31) / 32;
    // factors, two Householder vectors, taus, and the original A when refining
    const size_t smem = sizeof(float) * ((size_t)32 * (32 * R + 1) + (refine > 0 ? 32 * 32 * R : 0) + 2 * 32 * R + 32);
    auto go = [&](auto kern) -> gbla_status {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return from_cuda(e);
        }
        kern<<<(unsigned)batch, 128, smem, st>>>(m, n, nrhs, A, sA, B, sB, info, refine, batch);
        return launch_status();
    };
    switch (R) {
        case 1: return go(k_gels_cta<1>);
        case 2: return go(k_gels_cta<2>);
        case 3: return go(k_gels_cta<3>);
        default: return go(k_gels_cta<4>);
    }
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_sgels_batched(int m, int n, int nrhs, float *A, int64_t sA, float *B, int64_t sB, int *info,
                                        int refine, int batch, cudaStream_t st) {
    return gels_cta_launch(m, n, nrhs, A, sA, B, sB, info, refine, batch, st);
}
