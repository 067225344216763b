// gemm_tc.cu -- batched 64x64x64 single-precision GEMM on the 5th-generation
// tensor cores (tcgen05) with a three-way BF16 split of both operands.
//
// Precision: x = x_hi + x_mid + x_lo exactly (three bf16 terms, 24 bits), and
// C = A_hi B_hi + A_hi B_mid + A_mid B_hi + A_hi B_lo + A_mid B_mid + A_lo B_hi
// is accumulated in FP32 in tensor memory; the dropped terms are O(2^-24)
// relative, so the result carries FP32-level error.
//
// Shape mapping: two independent pairs (i, j) form one M=128, N=128 MMA,
//   D = [A_i; A_j] (128 x K) * [B_i B_j] (K x 128),
// and only the diagonal 64x64 blocks of D are stored (the off-diagonal blocks
// cost tensor time but no memory traffic).  This keeps the accumulator in the
// plain M=128 layout: row r of D lives in TMEM lane r.
//
// Pipeline per block (256 threads, persistent, one block per SM):
//   cp.async copies raw fp32 operands into one of two shared-memory stages
//   (64 KB each, one pair-of-pairs); all warps: raw stage -> split -> BF16
//   operand tiles (K-major core-matrix layout, no swizzle); fence.proxy.async;
//   barrier; the stage is refilled with the pair-of-pairs two steps ahead; one
//   thread issues the 24 tcgen05.mma into one of two TMEM accumulators and
//   commits to an mbarrier.  Once the MMAs of pair-of-pairs q are done, the
//   warps split q + grid and issue its MMAs into the other accumulator, then
//   read q's accumulator with tcgen05.ld and store C while those MMAs run.
//   Every wait is bounded; on a timeout the block records an error flag, waits
//   for its copies, frees its TMEM and exits.
#include <cuda_bf16.h>
#include "common.cuh"

namespace gbla {

constexpr int TC_THREADS = 256;
constexpr int TC_TILE_BYTES = 128 * 64 * 2;    // one operand split: 128 rows x 64 K bf16 = 16 KB
constexpr int TC_RAW_BYTES = 4 * 64 * 64 * 4;   // fp32 A_i, A_j, B_i, B_j of one pair-of-pairs = 64 KB
// A and B, 3 splits each; two raw fp32 stages; barrier
constexpr int TC_SMEM = 6 * TC_TILE_BYTES + 2 * TC_RAW_BYTES + 64;
constexpr int TC_TMEM_COLS = 256;  // two 128-column accumulators
constexpr uint32_t TC_SPIN_LIMIT = 1u << 26;

__device__ int g_tc_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// K-major, no-swizzle canonical layout: core matrix = 8 rows x 16 bytes,
// LBO = 128 B between core matrices along K, SBO = 1024 B between 8-row groups.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;   // leading-dimension byte offset (K direction)
    d |= (uint64_t)((1024u >> 4) & 0x3FFF) << 32;  // stride-dimension byte offset (M/N direction)
    d |= (uint64_t)1 << 46;                        // descriptor version for tcgen05
    return d;                                      // base offset 0, no swizzle
}

// Instruction descriptor, kind::f16: D fp32, A = B = bf16, both K-major, M = N = 128.
__host__ __device__ constexpr uint32_t make_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (row, k) in a K-major 128 x 64 bf16 tile
__device__ __forceinline__ uint32_t kmajor_off(int row, int kgroup) {
    return (uint32_t)((row >> 3) * 1024 + kgroup * 128 + (row & 7) * 16);
}

// Exact three-way BF16 split of two values at once: each cvt.rn.bf16x2
// rounds and packs a pair (element 0 in the low half), and a BF16 value
// widens back to FP32 by placing its bits in the high half of a word.
__device__ __forceinline__ uint32_t bf16x2_rn(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ void split3x2(float x0, float x1, uint32_t &H, uint32_t &M, uint32_t &L) {
    H = bf16x2_rn(x0, x1);
    const float r0 = x0 - __uint_as_float(H << 16), r1 = x1 - __uint_as_float(H & 0xffff0000u);
    M = bf16x2_rn(r0, r1);
    const float s0 = r0 - __uint_as_float(M << 16), s1 = r1 - __uint_as_float(M & 0xffff0000u);
    L = bf16x2_rn(s0, s1);
}

// Split 8 K-consecutive fp32 values of one operand row into three 16-byte
// core-matrix rows.
__device__ __forceinline__ void store_split_row(unsigned char *base, uint32_t off, const float (&v)[8]) {
    uint32_t h[4], m[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; e++) split3x2(v[2 * e], v[2 * e + 1], h[e], m[e], l[e]);
    *reinterpret_cast<uint4 *>(base + 0 * TC_TILE_BYTES + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(base + 1 * TC_TILE_BYTES + off) = make_uint4(m[0], m[1], m[2], m[3]);
    *reinterpret_cast<uint4 *>(base + 2 * TC_TILE_BYTES + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < TC_SPIN_LIMIT; it++) {
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

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_gemm_tc_bf16x6(float alpha, const float *__restrict__ A, int64_t sA, const float *__restrict__ B, int64_t sB,
                     float beta, float *__restrict__ C, int64_t sC, int batch) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sAop = smem;                      // 3 splits x 16 KB
    unsigned char *sBop = smem + 3 * TC_TILE_BYTES;  // 3 splits x 16 KB
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 6 * TC_TILE_BYTES + 2 * TC_RAW_BYTES);
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t bar_a = smem_u32(bar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a));
        asm volatile("fence.mbarrier_init.release.cluster;");
        s_abort = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = s_tmem;
    constexpr uint32_t idesc = make_idesc_bf16(128, 128);
    uint32_t phase = 0;

    const int npp = (batch + 1) / 2;  // pair-of-pairs count
    // Raw fp32 operands of one pair-of-pairs (stage layout: A_i, A_j, B_i, B_j,
    // 16 KB each) are copied into shared memory with 16-byte cp.async, two
    // stages deep, so the copies of pair-of-pairs q + 2 grid run while q is
    // split, multiplied and stored.  A_p is column-major (element (r, k) at
    // k * 64 + r) and kept linear: the split reads it down a column, lanes on
    // consecutive rows.  B_p (element (k, n) at n * 64 + k) is read along k by
    // lanes on consecutive n, so its 16-byte chunk kc of row n is stored at
    // chunk position kc ^ (n & 7) of that row: eight consecutive rows then hit
    // eight different bank groups.
    unsigned char *raw0 = smem + 6 * TC_TILE_BYTES;
    auto issue_raw = [&](int qq, int stage) {
        if (qq < npp) {
            unsigned char *dst0 = raw0 + stage * TC_RAW_BYTES;
#pragma unroll
            for (int u = 0; u < 16; u++) {
                const int idx = (u & 7) * TC_THREADS + tid;  // 0..2047 within the operand
                const int half = idx >> 10, c = idx & 1023;  // pair 2 qq + half, chunk c
                const int pr = 2 * qq + half;
                const bool ok = pr < batch;
                const float *src;
                uint32_t doff;
                if (u < 8) {
                    src = A + (int64_t)(ok ? pr : 0) * sA + c * 4;
                    doff = (uint32_t)(half * 16384 + c * 16);
                } else {
                    const int n = c >> 4, kc = c & 15;
                    src = B + (int64_t)(ok ? pr : 0) * sB + c * 4;
                    doff = (uint32_t)(32768 + half * 16384 + n * 256 + ((kc ^ (n & 7)) << 4));
                }
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst0 + doff)),
                             "l"(src), "r"(ok ? 16 : 0)
                             : "memory");
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");  // (possibly empty) group per call
    };
    issue_raw(blockIdx.x, 0);
    issue_raw(blockIdx.x + gridDim.x, 1);
    // split: raw fp32 (shared) -> three BF16 K-major operand tiles
    auto split = [&](int stg) {
        const unsigned char *rs = raw0 + stg * TC_RAW_BYTES;
#pragma unroll
        for (int it = 0; it < 4; it++) {
            const int item = tid + it * TC_THREADS;  // 0..1023 = 128 rows x 8 kgroups
            const int row = item & 127, kg = item >> 7;
            const int half = row >> 6, r = row & 63;
            const float *ra = reinterpret_cast<const float *>(rs + half * 16384);
            float va[8], vb[8];
#pragma unroll
            for (int e = 0; e < 8; e++) va[e] = ra[(kg * 8 + e) * 64 + r];
            const unsigned char *rb = rs + 32768 + half * 16384 + r * 256;
            const float4 b0 = *reinterpret_cast<const float4 *>(rb + (((2 * kg) ^ (r & 7)) << 4));
            const float4 b1 = *reinterpret_cast<const float4 *>(rb + (((2 * kg + 1) ^ (r & 7)) << 4));
            vb[0] = b0.x; vb[1] = b0.y; vb[2] = b0.z; vb[3] = b0.w;
            vb[4] = b1.x; vb[5] = b1.y; vb[6] = b1.z; vb[7] = b1.w;
            const uint32_t off = kmajor_off(row, kg);
            store_split_row(sAop, off, va);
            store_split_row(sBop, off, vb);
        }
    };
    // one thread issues the 24 MMAs of a pair-of-pairs into accumulator buffer buf
    auto issue_mma = [&](int buf) {
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a0 = smem_u32(sAop), b0 = smem_u32(sBop);
            const uint32_t d = tmem + (uint32_t)(buf * 128);
            uint32_t acc = 0;
#pragma unroll
            for (int s = 0; s < 4; s++) {  // K slices of 16
                const uint32_t ko = s * 256;
                // (a split, b split) products, smallest first
                const int pa[6] = {2, 1, 0, 1, 0, 0};
                const int pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
                for (int p = 0; p < 6; p++) {
                    uint64_t ad = make_desc(a0 + pa[p] * TC_TILE_BYTES + ko);
                    uint64_t bd = make_desc(b0 + pb[p] * TC_TILE_BYTES + ko);
                    mma_bf16(d, ad, bd, idesc, acc);
                    acc = 1;
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_a)
                         : "memory");
        }
    };
    // Accumulators are double-buffered in tensor memory (2 x 128 columns): the
    // MMAs of pair-of-pairs q + grid run while the epilogue of q reads its
    // buffer.  The operand tiles are single-buffered, so the split of q + grid
    // waits for the MMAs of q.
    int stage = 0, buf = 0;
    const int q0 = blockIdx.x;
    if (q0 < npp) {
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        __syncthreads();
        split(stage);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        issue_raw(q0 + 2 * gridDim.x, stage);
        issue_mma(buf);
    }
    for (int q = q0; q < npp; q += gridDim.x) {
        const int p0 = 2 * q;
        const bool has1 = p0 + 1 < batch;
        // the MMAs of q are done: its accumulator is ready and the operand tiles are free
        bool ok = mbar_wait(bar_a, phase);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) { atomicExch(&g_tc_error, 1); s_abort = 1; }
            break;
        }
        phase ^= 1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const int qn = q + gridDim.x;
        if (qn < npp) {
            stage ^= 1;
            asm volatile("cp.async.wait_group 1;" ::: "memory");  // qn's stage landed; the other may be in flight
            __syncthreads();
            split(stage);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            // this stage is consumed: start the copies of the pair-of-pairs two steps ahead
            issue_raw(qn + 2 * gridDim.x, stage);
            issue_mma(buf ^ 1);
        }
        // ---- epilogue of q (buffer buf): warp w reads lanes 32*(w%4).., 32 columns of its pair's diagonal block
        {
            const int quad = warp & 3, half = warp >> 2;
            const int row = quad * 32 + lane;          // D row = TMEM lane
            const int pair = p0 + (row >> 6);
            const int col0 = (row >> 6) * 64 + half * 32;  // diagonal block, 32 of its 64 columns
            uint32_t v[32];
            uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * 128 + col0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (pair < batch && (row < 64 || has1)) {
                float *c = C + (int64_t)pair * sC;
                const int r = row & 63, cb = half * 32;
#pragma unroll
                for (int e = 0; e < 32; e++) {
                    float val = alpha * __uint_as_float(v[e]);
                    float *dst = c + (int64_t)(cb + e) * 64 + r;
                    if (beta != 0.0f) val = fmaf(beta, *dst, val);
                    *dst = val;
                }
            }
        }
        // every read of buffer buf is done before the MMAs of q + 2 grid overwrite it
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        buf ^= 1;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");  // no copy may land after the block is gone
    __syncthreads();
    if (s_abort) mbar_wait(bar_a, phase);  // give an MMA still in flight a bounded chance to land
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
    }
}

bool tc_gemm_eligible(int m, int n, int k, int64_t sA, int64_t sB, int64_t sC, const void *A, const void *B,
                      const void *C) {
    if (m != 64 || n != 64 || k != 64) return false;
    // 16-byte copies of whole matrices: both operands 16-byte aligned, strides multiples of 4 floats
    if (((uintptr_t)A & 15) != 0 || (sA % 4) != 0) return false;
    if (((uintptr_t)B & 15) != 0 || (sB % 4) != 0) return false;
    (void)sC; (void)C;
    return true;
}

gbla_status tc_sgemm_bf16x6(int m, int n, int k, float alpha, const float *A, int64_t sA, const float *B, int64_t sB,
                            float beta, float *C, int64_t sC, int batch, cudaStream_t st) {
    (void)m; (void)n; (void)k;
    static bool attr_done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc_bf16x6, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
        if (e != cudaSuccess) return from_cuda(e);
        attr_done[dev] = true;
    }
    int npp = (batch + 1) / 2;
    int grid = sm_count();  // persistent: one block per SM, loads of the next pair-of-pairs overlap the current
    if (grid > npp) grid = npp;
    k_gemm_tc_bf16x6<<<grid, TC_THREADS, TC_SMEM, st>>>(alpha, A, sA, B, sB, beta, C, sC, batch);
    return launch_status();
}

}  // namespace gbla

GBLA_API int gbla_device_error_flags(void) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, gbla::g_tc_error, sizeof(int)) != cudaSuccess) return -1;
    int z = 0;
    cudaMemcpyToSymbol(gbla::g_tc_error, &z, sizeof(int));
    return v;
}
