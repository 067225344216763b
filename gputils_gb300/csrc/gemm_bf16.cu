// gemm_bf16.cu -- general BF16 GEMM on the 5th-generation tensor cores:
//   C[M x N] = alpha * A[M x K] * B[N x K]^T      (both operands K-major)
// with FP32 accumulation in tensor memory and a fused epilogue (bias, ReLU,
// ReLU-derivative mask, FP32 / BF16 / transposed-BF16 outputs).  It carries
// the warm-start network's forward and backward passes.
//
// Per CTA one 128 x 128 output tile; K is walked in 64-element stages through
// a 3-deep shared-memory ring filled by TMA (cp.async.bulk.tensor, 128-byte
// swizzle), so two CTAs fit on an SM and one CTA's epilogue overlaps the
// other's main loop.  Warp roles (192 threads):
//   warp 0    TMA producer (one lane): waits "empty[s]", arms "full[s]" with
//             the stage's byte count, issues the A and B box loads;
//   warp 1    TMEM owner and MMA issuer (one lane): waits "full[s]", issues
//             four K=16 tcgen05.mma, commits to "empty[s]"; after the last
//             stage commits to "done";
//   warps 2-5 epilogue: wait "done", tcgen05.ld their 32-lane quarter of the
//             accumulator, apply the epilogue, store.
// Every wait is bounded.  On a timeout the CTA sets g_bf16_gemm_error, waits
// (bounded) for its TMA loads in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include "common.cuh"
#include "gemm_bf16.cuh"

namespace gbla {

constexpr int BG_BM = 128, BG_BN = 128, BG_BK = 64, BG_STAGES = 3;
constexpr int BG_THREADS = 192;
constexpr int BG_TILE_BYTES = BG_BM * BG_BK * 2;                  // 16 KB per operand per stage
constexpr int BG_STAGE_BYTES = 2 * BG_TILE_BYTES;                 // A + B
constexpr int BG_SMEM = BG_STAGES * BG_STAGE_BYTES + 1024 + 256;  // + alignment slack + barriers
constexpr uint32_t BG_TMEM_COLS = 128;
constexpr uint32_t BG_SPIN_LIMIT = 1u << 26;

__device__ int g_bf16_gemm_error = 0;


namespace {

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < BG_SPIN_LIMIT; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// K-major operand tile, 128-byte swizzle: rows of 64 bf16 (128 B), 8-row
// groups 1024 B apart (SBO); the leading offset is unused for this layout.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                        // LBO (ignored for swizzled K-major)
    d |= (uint64_t)((1024u >> 4) & 0x3FFF) << 32;  // SBO: next 8-row group
    d |= (uint64_t)1 << 46;                        // tcgen05 descriptor version
    d |= (uint64_t)2 << 61;                        // layout: 128-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: D fp32, A = B = bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace

__global__ void __launch_bounds__(BG_THREADS, 2)
    k_gemm_bf16_tn(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int M, int N,
                   int K, const gbla_bf16_epilogue epi, const Bf16EpiX ex) {
    extern __shared__ unsigned char bg_raw[];
    // 1024-byte alignment for the 128-byte swizzle pattern
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(bg_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + BG_STAGES * BG_STAGE_BYTES);
    uint64_t *empty = full + BG_STAGES;
    uint64_t *done = empty + BG_STAGES;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // N tiles vary fastest: the CTAs that share an A row panel run together and
    // read it once from DRAM (through L2)
    const int m0 = blockIdx.y * BG_BM, n0 = blockIdx.x * BG_BN;
    const int KT = (K + BG_BK - 1) / BG_BK;
    if (ex.lower && n0 + BG_BN <= m0) return;  // every element of the tile has n < m (whole CTA, before any setup)

    if (tid == 0) {
        for (int s = 0; s < BG_STAGES; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(full + s)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(empty + s)));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(done)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        s_abort = 0;
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_tmem)),
                     "r"(BG_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = s_tmem;
    int issued = 0;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        for (int kt = 0; kt < KT; kt++) {
            const int s = kt % BG_STAGES;
            if (kt >= BG_STAGES && !bar_wait(su32(empty + s), ((kt / BG_STAGES) + 1) & 1)) {
                s_abort = 1;
                break;
            }
            if (*(volatile int *)&s_abort) break;
            const uint32_t fb = su32(full + s);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(BG_STAGE_BYTES)
                         : "memory");
            const uint32_t sa = su32(smem + s * BG_STAGE_BYTES);
            tma_load_2d(sa, &mapA, kt * BG_BK, m0, fb);
            tma_load_2d(sa + BG_TILE_BYTES, &mapB, kt * BG_BK, n0, fb);
            issued = kt + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        constexpr uint32_t idesc = idesc_bf16(BG_BM, BG_BN);
        bool ok = true;
        for (int kt = 0; kt < KT; kt++) {
            const int s = kt % BG_STAGES;
            if (!bar_wait(su32(full + s), (kt / BG_STAGES) & 1)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t sa = su32(smem + s * BG_STAGE_BYTES), sb = sa + BG_TILE_BYTES;
#pragma unroll
            for (int k = 0; k < BG_BK / 16; k++) {
                const uint64_t ad = desc_sw128(sa + k * 32), bd = desc_sw128(sb + k * 32);
                const uint32_t acc = (kt > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             su32(empty + s))
                         : "memory");
        }
        if (!ok) s_abort = 1;
        // "done" fires when every MMA issued so far has completed
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(done))
                     : "memory");
    } else if (warp >= 2) {
        // ---------------- epilogue
        const bool ok = bar_wait(su32(done), 0);
        asm volatile("tcgen05.fence::after_thread_sync;");
        const int quad = warp & 3;
        const int m = m0 + quad * 32 + lane;
        if (!ok) s_abort = 1;
        // tcgen05.ld is warp-collective: decide per warp
        if (__all_sync(FULL, ok && !*(volatile int *)&s_abort)) {
            for (int c = 0; c < BG_BN / 32; c++) {
                uint32_t v[32];
                tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(c * 32), v);
                if (m >= M) continue;
                const int nb = n0 + c * 32;
                float x[32];
#pragma unroll
                for (int e = 0; e < 32; e++) {
                    const int n = nb + e;
                    float t = epi.alpha * __uint_as_float(v[e]);
                    if (epi.bias && n < N) t += epi.bias[n];
                    if (epi.relu) t = fmaxf(t, 0.0f);
                    if (epi.mask && n < N &&
                        !(__bfloat162float(__ushort_as_bfloat16(epi.mask[(int64_t)m * epi.ld_mask + n])) > 0.0f))
                        t = 0.0f;
                    x[e] = t;
                }
                const bool whole = nb + 32 <= N;
                if (epi.out_f32 && !(ex.lower && nb + 32 <= m)) {
                    float *dst = epi.out_f32 + (int64_t)m * epi.ld_f32 + nb;
                    if (whole && (!ex.lower || nb >= m) && ((uintptr_t)dst & 15) == 0) {
#pragma unroll
                        for (int e = 0; e < 32; e += 4) {
                            float4 o = make_float4(x[e], x[e + 1], x[e + 2], x[e + 3]);
                            if (ex.beta != 0.0f) {
                                const float4 c = *reinterpret_cast<const float4 *>(dst + e);
                                o.x = fmaf(ex.beta, c.x, o.x);
                                o.y = fmaf(ex.beta, c.y, o.y);
                                o.z = fmaf(ex.beta, c.z, o.z);
                                o.w = fmaf(ex.beta, c.w, o.w);
                            }
                            *reinterpret_cast<float4 *>(dst + e) = o;
                        }
                    } else {
                        for (int e = 0; e < 32; e++)
                            if (nb + e < N && (!ex.lower || nb + e >= m))
                                dst[e] = ex.beta != 0.0f ? fmaf(ex.beta, dst[e], x[e]) : x[e];
                    }
                }
                if (epi.out_bf16) {
                    __nv_bfloat16 *dst = reinterpret_cast<__nv_bfloat16 *>(epi.out_bf16) + (int64_t)m * epi.ld_bf16 + nb;
                    if (whole && ((uintptr_t)dst & 15) == 0) {
#pragma unroll
                        for (int e = 0; e < 32; e += 8) {
                            __nv_bfloat162 p0 = __floats2bfloat162_rn(x[e], x[e + 1]);
                            __nv_bfloat162 p1 = __floats2bfloat162_rn(x[e + 2], x[e + 3]);
                            __nv_bfloat162 p2 = __floats2bfloat162_rn(x[e + 4], x[e + 5]);
                            __nv_bfloat162 p3 = __floats2bfloat162_rn(x[e + 6], x[e + 7]);
                            uint4 u;
                            u.x = *reinterpret_cast<uint32_t *>(&p0);
                            u.y = *reinterpret_cast<uint32_t *>(&p1);
                            u.z = *reinterpret_cast<uint32_t *>(&p2);
                            u.w = *reinterpret_cast<uint32_t *>(&p3);
                            *reinterpret_cast<uint4 *>(dst + e) = u;
                        }
                    } else {
                        for (int e = 0; e < 32; e++)
                            if (nb + e < N) dst[e] = __float2bfloat16_rn(x[e]);
                    }
                }
                if (epi.out_bf16_t) {
                    // C^T: for a fixed column the warp's 32 rows are consecutive
                    for (int e = 0; e < 32; e++)
                        if (nb + e < N)
                            epi.out_bf16_t[(int64_t)(nb + e) * epi.ld_bf16_t + m] =
                                __bfloat16_as_ushort(__float2bfloat16_rn(x[e]));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (s_abort) {
        if (tid == 0) atomicExch(&g_bf16_gemm_error, 1);
        if (warp == 0 && lane == 0) {
            // let the loads this CTA issued land before the CTA exits
            for (int kt = issued - BG_STAGES > 0 ? issued - BG_STAGES : 0; kt < issued; kt++)
                bar_wait(su32(full + kt % BG_STAGES), (kt / BG_STAGES) & 1);
        }
        if (warp == 1 && lane == 0) bar_wait(su32(done), 0);
        __syncthreads();
    }
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BG_TMEM_COLS));
    }
}

// ------------------------------------------------------------------ host
namespace {

typedef CUresult (*encode_tiled_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

encode_tiled_fn encoder() {
    static encode_tiled_fn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<encode_tiled_fn>(p);
    }
    return fn;
}

// rows x cols bf16, row stride ld elements; box 64 (cols) x 128 (rows), 128-byte swizzle
bool make_map(CUtensorMap *map, const void *base, int64_t rows, int64_t cols, int64_t ld) {
    encode_tiled_fn enc = encoder();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {BG_BK, BG_BM};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

gbla_status gemm_bf16_tn_ex(int M, int N, int K, const void *A, int64_t lda, const void *B, int64_t ldb,
                            const gbla_bf16_epilogue &epi, const Bf16EpiX &ex, cudaStream_t st) {
    if (M < 0 || N < 0 || K < 0) return GBLA_INVALID_VALUE;
    if (M == 0 || N == 0) return GBLA_SUCCESS;
    if (!A || !B || K == 0) return GBLA_INVALID_VALUE;
    // TMA: 16-byte aligned bases and row strides
    if (((uintptr_t)A & 15) || ((uintptr_t)B & 15) || (lda & 7) || (ldb & 7) || lda < K || ldb < K)
        return GBLA_INVALID_VALUE;
    if (!epi.out_f32 && !epi.out_bf16 && !epi.out_bf16_t) return GBLA_INVALID_VALUE;
    if ((epi.out_f32 && epi.ld_f32 < N) || (epi.out_bf16 && epi.ld_bf16 < N) || (epi.out_bf16_t && epi.ld_bf16_t < M) ||
        (epi.mask && epi.ld_mask < N))
        return GBLA_INVALID_VALUE;
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, lda) || !make_map(&mb, B, N, K, ldb)) return GBLA_CUDA_ERROR;
    static bool attr_done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, BG_SMEM);
        if (e != cudaSuccess) return from_cuda(e);
        attr_done[dev] = true;
    }
    dim3 grid((unsigned)((N + BG_BN - 1) / BG_BN), (unsigned)((M + BG_BM - 1) / BG_BM));
    if (grid.y > 65535) return GBLA_INVALID_VALUE;
    k_gemm_bf16_tn<<<grid, BG_THREADS, BG_SMEM, st>>>(ma, mb, M, N, K, epi, ex);
    return launch_status();
}

gbla_status gemm_bf16_tn(int M, int N, int K, const void *A, int64_t lda, const void *B, int64_t ldb,
                         const gbla_bf16_epilogue &epi, cudaStream_t st) {
    return gemm_bf16_tn_ex(M, N, K, A, lda, B, ldb, epi, Bf16EpiX{0.0f, 0}, st);
}

}  // namespace gbla

GBLA_API gbla_status gbla_gemm_bf16_tn(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb,
                                       const gbla_bf16_epilogue *epi, cudaStream_t stream) {
    if (!epi) return GBLA_INVALID_VALUE;
    return gbla::gemm_bf16_tn(M, N, K, A, lda, B, ldb, *epi, stream);
}
