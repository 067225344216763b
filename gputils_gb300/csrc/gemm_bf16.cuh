// gemm_bf16.cuh -- in-library interface of the BF16 tcgen05 GEMM
// (gemm_bf16.cu): C[M x N] = alpha * A[M x K] * B[N x K]^T, K-major BF16
// operands, FP32 accumulation, fused epilogue.
#pragma once
#include "common.cuh"

namespace gbla {

// Epilogue extras for in-library callers (not part of the ABI struct):
// out_f32 = alpha * acc + beta * out_f32 (the old value is read when beta is
// nonzero), and with `lower` only the elements with column index n >= row
// index m are written -- for a symmetric C stored into a column-major matrix
// (out_f32[m * ld + n] is element (n, m)), its lower triangle -- and tiles
// entirely above the diagonal are not computed.
struct Bf16EpiX {
    float beta;
    int lower;
};

gbla_status gemm_bf16_tn(int M, int N, int K, const void *A, int64_t lda, const void *B, int64_t ldb,
                         const gbla_bf16_epilogue &epi, cudaStream_t st);
gbla_status gemm_bf16_tn_ex(int M, int N, int K, const void *A, int64_t lda, const void *B, int64_t ldb,
                            const gbla_bf16_epilogue &epi, const Bf16EpiX &ex, cudaStream_t st);

}  // namespace gbla
