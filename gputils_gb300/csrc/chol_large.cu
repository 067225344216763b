// chol_large.cu -- Cholesky factorisation of one large SPD matrix (FP32) on
// the whole GPU, for the sizes where one thread block per matrix (chol.cu)
// leaves all but one SM idle.
//
// Right-looking blocked algorithm, panels of CL_NB = 128 columns.  For the
// panel at column k0 (width w, n2 rows below it):
//   1. k_potrf_diag, one CTA: L11 = chol(A11) with the block in registers
//      (an 8 x 8 tile per thread, one barrier per column), written back into
//      the lower triangle of A11; info = first non-positive pivot;
//   2. k_trsm_panel, n2 / 64 CTAs: L21 = A21 L11^-T row by row (four threads
//      per row, each keeping every fourth entry of the row in registers; one
//      4-lane reduction per column), written back into A21 and, split once
//      into BF16 parts in shared memory, as the row-major operands of step 3;
//   3. the trailing update A22 -= L21 L21^T on the tensor cores: one
//      tcgen05 GEMM (gemm_bf16.cu) with K = 6 w over the stacked three-way
//      split x = h + m + l (exact for FP32 x; h, m, l BF16):
//      [h h m h l m] . [h m h l h m]^T = hh' + hm' + mh' + hl' + lh' + mm',
//      the products below 2^-24 of |x|^2 dropped, FP32 accumulation in
//      tensor memory; the epilogue subtracts the product from the lower
//      triangle of A22 in place (tiles above the diagonal are skipped).
//      The update of the next panel's 128 columns runs on the caller's
//      stream; the rest runs on a side stream, overlapping the next panel's
//      steps 1 and 2 (look-ahead).
// The strict upper triangle of A is never written.
//
// The solve with one such factor (gbla_spotrs_large) is blocked the same
// way: per 128-row block a one-CTA triangular solve and a many-CTA update of
// the remaining rows (below it forward, above it backward).
//
// Replaces cusolverDnSpotrf and cusolverDnSpotrs for one matrix (the
// reference's CholeskyFactoriser: workspace include/tensor.cuh:1703-1709,
// factorise :1754-1761, solve :1775-1783).
#include <cuda_bf16.h>
#include "common.cuh"
#include "gemm_bf16.cuh"

namespace gbla {

constexpr int CL_NB = 128;          // panel width
constexpr int CL_LD = CL_NB + 1;    // shared-memory column stride of a 128 x 128 block (odd: conflict-free)
constexpr int CL_K = 6 * CL_NB;     // stacked split products per row of L21
constexpr int CL_TROWS = 64;        // rows of L21 per CTA of the panel solve
constexpr int CL_THREADS = 256;
constexpr int CL_PLD = CL_NB + 8;   // row stride of the BF16 part rows in shared memory (16-byte rows, no conflicts)

// ------------------------------------------------------------ diagonal block
// A: top-left element of the w x w diagonal block (w <= 128), column stride
// lda.  Thread t = ti + 16 tj keeps the 8 x 8 register tile of elements
// (ti + 16 r, tj + 16 c) of the lower triangle.  Step k updates a(i, j) -=
// a(i, k) a(j, k) / d_k for k < j <= i with column k read from a shared
// buffer (unscaled; d_k = a(k, k)), and the owners of column k + 1 publish
// it in the other buffer: one barrier per column.  Column j is scaled by
// 1 / sqrt(d_j) at the end.  Steps k = 16 KC + kr run in diag_steps<KC>, so
// every register index is a compile-time constant.
struct DiagShared {
    float colb[2][CL_NB];  // the pivot column of the step, double-buffered
    float dsq[CL_NB];      // sqrt(d_j)
    int fail;
};

template <int KC>
__device__ __forceinline__ void diag_steps(float (&a)[8][8], DiagShared &sh, int w, int ti, int tj, int tid) {
    const int kend = w - 16 * KC < 16 ? w - 16 * KC : 16;  // <= 0 past the last column
    for (int kr = 0; kr < kend; kr++) {
        const int k = 16 * KC + kr;
        const float *col = sh.colb[k & 1];
        const float d = col[k];
        if (tid == 0) {
            sh.dsq[k] = sqrtf(d);
            if (!(d > 0.f) && sh.fail == 0) sh.fail = k + 1;
        }
        const float id = 1.f / d;
        float ci[8], cj[8];
#pragma unroll
        for (int r = KC; r < 8; r++) ci[r] = col[ti + 16 * r];
#pragma unroll
        for (int c = KC; c < 8; c++) cj[c] = col[tj + 16 * c] * id;
        // j = tj + 16 c > k and i = ti + 16 r >= j
#pragma unroll
        for (int c = KC; c < 8; c++)
#pragma unroll
            for (int r = c; r < 8; r++) {
                const bool upd = (c > KC || tj > kr) && (r > c || ti >= tj);
                if (upd) a[r][c] = fmaf(-ci[r], cj[c], a[r][c]);
            }
        // publish column k + 1: owners tj == (k + 1) mod 16, local column KC or KC + 1
        if (k + 1 < w) {
            float *nxt = sh.colb[(k + 1) & 1];
            if (kr < 15) {
                if (tj == kr + 1) {
#pragma unroll
                    for (int r = 0; r < 8; r++) nxt[ti + 16 * r] = a[r][KC];
                }
            } else if (KC < 7) {
                if (tj == 0) {
#pragma unroll
                    for (int r = 0; r < 8; r++) nxt[ti + 16 * r] = a[r][KC < 7 ? KC + 1 : KC];
                }
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(CL_THREADS, 1)
    k_potrf_diag(float *__restrict__ A, int64_t lda, int w, int k0, int *__restrict__ info) {
    __shared__ DiagShared sh;
    const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
    float a[8][8];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int i = ti + 16 * r, j = tj + 16 * c;
            a[r][c] = (i < w && j <= i) ? A[(int64_t)j * lda + i] : 0.f;
        }
    if (tid == 0) sh.fail = 0;
    if (tj == 0) {
#pragma unroll
        for (int r = 0; r < 8; r++) sh.colb[0][ti + 16 * r] = a[r][0];
    }
    __syncthreads();
    diag_steps<0>(a, sh, w, ti, tj, tid);
    diag_steps<1>(a, sh, w, ti, tj, tid);
    diag_steps<2>(a, sh, w, ti, tj, tid);
    diag_steps<3>(a, sh, w, ti, tj, tid);
    diag_steps<4>(a, sh, w, ti, tj, tid);
    diag_steps<5>(a, sh, w, ti, tj, tid);
    diag_steps<6>(a, sh, w, ti, tj, tid);
    diag_steps<7>(a, sh, w, ti, tj, tid);
    // L(j, j) = sqrt(d_j), L(i, j) = a(i, j) / sqrt(d_j) below it
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int i = ti + 16 * r, j = tj + 16 * c;
            if (i < w && j <= i) A[(int64_t)j * lda + i] = i == j ? sh.dsq[j] : a[r][c] / sh.dsq[j];
        }
    if (tid == 0 && info && sh.fail && *info == 0) *info = k0 + sh.fail;
}

// --------------------------------------------------------------- panel solve
// A: the matrix (column stride lda); the panel is columns [k0, k0 + 128),
// L11 its diagonal block (already factored), A21 rows [k0 + 128, k0 + 128 +
// n2).  SA, SB: n2 x CL_K row-major BF16 operands of the trailing update.
__device__ __forceinline__ void bf16_split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
    h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);  // exact
    m = __float2bfloat16_rn(r1);
    l = __float2bfloat16_rn(r1 - __bfloat162float(m));  // exact: r1 - m has at most 8 significant bits
}

__global__ void __launch_bounds__(CL_THREADS, 2)
    k_trsm_panel(float *__restrict__ A, int64_t lda, int k0, int n2, __nv_bfloat16 *__restrict__ SA,
                 __nv_bfloat16 *__restrict__ SB) {
    extern __shared__ float cl_s[];
    float *L = cl_s;                   // 128 x CL_LD: L11, column-major (lower triangle)
    float *dinv = L + CL_NB * CL_LD;   // 128: 1 / L_jj
    // the solved rows split into h, m, l: 3 x CL_TROWS rows of CL_PLD BF16, row-major
    __nv_bfloat16 *P = reinterpret_cast<__nv_bfloat16 *>(dinv + CL_NB);
    const int tid = threadIdx.x, row = tid >> 2, sub = tid & 3;
    const float *a11 = A + k0 + (int64_t)k0 * lda;
    // the whole 128 x 128 block, 64 values a thread with 16 loads in flight
    // (the strict upper triangle is loaded but not read)
#pragma unroll 16
    for (int e = tid; e < CL_NB * CL_NB; e += CL_THREADS) {
        const int j = e >> 7, i = e & (CL_NB - 1);
        L[j * CL_LD + i] = a11[(int64_t)j * lda + i];
    }
    __syncthreads();
    if (tid < CL_NB) dinv[tid] = 1.f / L[tid * CL_LD + tid];
    __syncthreads();
    const int r0 = blockIdx.x * CL_TROWS;
    const int r = r0 + row;  // row of L21
    const bool live = r < n2;
    float *a21 = A + (k0 + CL_NB) + (int64_t)k0 * lda;  // A21(r, i) = a21[r + i lda]
    float x[CL_NB / 4];  // entries i = sub + 4 s of the row
#pragma unroll
    for (int s = 0; s < CL_NB / 4; s++) x[s] = live ? a21[r + (int64_t)(sub + 4 * s) * lda] : 0.f;
    // forward substitution x L11^T = a: x_j = (a_j - sum_{i<j} x_i L_ji) / L_jj
#pragma unroll
    for (int j = 0; j < CL_NB; j++) {
        float p = 0.f;
#pragma unroll
        for (int s = 0; s <= (j >> 2); s++)
            if (4 * s + 3 < j || sub + 4 * s < j) p = fmaf(x[s], L[(sub + 4 * s) * CL_LD + j], p);
        p += shfl_xor(p, 1);  // the four threads of a row are lanes 4 q .. 4 q + 3
        p += shfl_xor(p, 2);
        if (sub == (j & 3)) x[j >> 2] = (x[j >> 2] - p) * dinv[j];
    }
#pragma unroll
    for (int s = 0; s < CL_NB / 4; s++) {
        const int i = sub + 4 * s;
        if (live) a21[r + (int64_t)i * lda] = x[s];
        __nv_bfloat16 h, m, l;
        bf16_split3(x[s], h, m, l);
        P[(0 * CL_TROWS + row) * CL_PLD + i] = h;
        P[(1 * CL_TROWS + row) * CL_PLD + i] = m;
        P[(2 * CL_TROWS + row) * CL_PLD + i] = l;
    }
    __syncthreads();
    // the operands, in 16-byte chunks: a row of SA / SB is six sections of
    // 128 values (h h m h l m / h m h l h m), 16 chunks of 8 each
    constexpr int CHUNKS = CL_K / 8;  // 96 per row and operand
    // part of section s (0 = h, 1 = m, 2 = l) in bits 2 s, 2 s + 1
    constexpr unsigned PART_A = 0u | 0u << 2 | 1u << 4 | 0u << 6 | 2u << 8 | 1u << 10;  // h h m h l m
    constexpr unsigned PART_B = 0u | 1u << 2 | 0u << 4 | 2u << 6 | 0u << 8 | 1u << 10;  // h m h l h m
    for (int c = tid; c < CL_TROWS * 2 * CHUNKS; c += CL_THREADS) {
        const int rr = c / (2 * CHUNKS), q = c % (2 * CHUNKS);
        if (r0 + rr >= n2) continue;
        const int op = q / CHUNKS, ch = q % CHUNKS, sec = ch / 16, i0 = (ch % 16) * 8;
        const unsigned part = ((op == 0 ? PART_A : PART_B) >> (2 * sec)) & 3u;
        const uint4 v = *reinterpret_cast<const uint4 *>(P + (part * CL_TROWS + rr) * CL_PLD + i0);
        *reinterpret_cast<uint4 *>((op == 0 ? SA : SB) + (int64_t)(r0 + rr) * CL_K + ch * 8) = v;
    }
}

// ------------------------------------------------------------ blocked solve
// L L^T X = B for one large factor (column stride lda) and nrhs columns of B
// (column stride ldb), in 128-row blocks: forward, the diagonal block solves
// its rows (one CTA, a warp per right-hand side) and then every row below
// subtracts the block's contribution (many CTAs, a thread per row, reading
// rows of the column block: coalesced); backward, the transposed diagonal
// block solves and then every row above subtracts its contribution (a
// thread per row i, reading L(k0 .. k0 + w, i), a contiguous piece of
// column i).  No workspace; each element of X is written by one thread.
constexpr int CS_WARPS = 4;     // right-hand sides per CTA of the diagonal solves
constexpr int CS_THREADS = 128; // rows per CTA of the updates

// Diagonal block of rows [k0, k0 + w): forward (L_kk y = b) or backward
// (L_kk^T x = y), in place in B.
template <bool FORWARD>
__global__ void __launch_bounds__(32 * CS_WARPS)
    k_trsv_diag(const float *__restrict__ L, int64_t lda, float *__restrict__ B, int64_t ldb, int k0, int w,
                int nrhs) {
    extern __shared__ float lb[];  // CL_NB x CL_LD: L_kk, column-major (lower triangle)
    __shared__ float xs[CS_WARPS][CL_NB];
    __shared__ float dinv[CL_NB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float *lk = L + k0 + (int64_t)k0 * lda;
    // the w x w block, 16 loads in flight a thread (the strict upper triangle
    // is loaded but not read)
#pragma unroll 16
    for (int e = tid; e < w * w; e += 32 * CS_WARPS) {
        const int j = e / w, i = e - j * w;
        lb[j * CL_LD + i] = lk[(int64_t)j * lda + i];
    }
    __syncthreads();
    for (int i = tid; i < w; i += 32 * CS_WARPS) dinv[i] = 1.f / lb[i * CL_LD + i];
    __syncthreads();
    const int c = blockIdx.x * CS_WARPS + warp;
    if (c >= nrhs) return;  // whole warp; no block barriers below
    float *x = xs[warp];
    float *bc = B + (int64_t)c * ldb + k0;
    for (int i = lane; i < w; i += 32) x[i] = bc[i];
    __syncwarp();
    if (FORWARD) {
        for (int j = 0; j < w; j++) {
            const float xj = x[j] * dinv[j];
            for (int i = j + 1 + lane; i < w; i += 32) x[i] = fmaf(-lb[j * CL_LD + i], xj, x[i]);
            __syncwarp();
            if (lane == 0) x[j] = xj;
            __syncwarp();
        }
    } else {
        for (int j = w - 1; j >= 0; j--) {
            const float xj = x[j] * dinv[j];
            for (int i = lane; i < j; i += 32) x[i] = fmaf(-lb[i * CL_LD + j], xj, x[i]);  // L(j, i)
            __syncwarp();
            if (lane == 0) x[j] = xj;
            __syncwarp();
        }
    }
    for (int i = lane; i < w; i += 32) bc[i] = x[i];
}

// Forward: rows i in [r0, n) lose L(i, k0 .. k0 + w) . y(k0 .. k0 + w).
__global__ void __launch_bounds__(CS_THREADS)
    k_trsv_fwd_update(const float *__restrict__ L, int64_t lda, float *__restrict__ B, int64_t ldb, int k0, int w,
                      int r0, int n, int nrhs) {
    __shared__ float ys[CL_NB];
    const int i = r0 + blockIdx.x * CS_THREADS + threadIdx.x;
    for (int c = 0; c < nrhs; c++) {
        __syncthreads();
        for (int j = threadIdx.x; j < w; j += CS_THREADS) ys[j] = B[(int64_t)c * ldb + k0 + j];
        __syncthreads();
        if (i < n) {
            const float *li = L + i + (int64_t)k0 * lda;
            float sp[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 16
            for (int j = 0; j < w; j++) sp[j & 3] = fmaf(li[(int64_t)j * lda], ys[j], sp[j & 3]);
            B[(int64_t)c * ldb + i] -= (sp[0] + sp[1]) + (sp[2] + sp[3]);
        }
    }
}

// Backward: rows i in [0, k0) lose L(k0 .. k0 + w, i) . x(k0 .. k0 + w).
__global__ void __launch_bounds__(CS_THREADS)
    k_trsv_bwd_update(const float *__restrict__ L, int64_t lda, float *__restrict__ B, int64_t ldb, int k0, int w,
                      int nrhs) {
    __shared__ float xs[CL_NB];
    const int i = blockIdx.x * CS_THREADS + threadIdx.x;
    for (int c = 0; c < nrhs; c++) {
        __syncthreads();
        for (int j = threadIdx.x; j < w; j += CS_THREADS) xs[j] = B[(int64_t)c * ldb + k0 + j];
        __syncthreads();
        if (i < k0) {
            const float *li = L + k0 + (int64_t)i * lda;  // column i from row k0: contiguous
            float sp[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 16
            for (int j = 0; j < w; j++) sp[j & 3] = fmaf(li[j], xs[j], sp[j & 3]);
            B[(int64_t)c * ldb + i] -= (sp[0] + sp[1]) + (sp[2] + sp[3]);
        }
    }
}

static gbla_status potrs_large(int n, int nrhs, const float *L, int64_t lda, float *B, int64_t ldb, cudaStream_t st) {
    if (n < 0 || nrhs < 0 || lda < n || ldb < n || (n > 0 && nrhs > 0 && (!L || !B))) return GBLA_INVALID_VALUE;
    if (n == 0 || nrhs == 0) return GBLA_SUCCESS;
    const unsigned gd = (unsigned)((nrhs + CS_WARPS - 1) / CS_WARPS);
    const size_t smem = sizeof(float) * (size_t)CL_NB * CL_LD;
    static bool attr_done[64] = {false};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    if (dev < 0 || dev >= 64 || !attr_done[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_trsv_diag<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_trsv_diag<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return from_cuda(e);
        if (dev >= 0 && dev < 64) attr_done[dev] = true;
    }
    for (int k0 = 0; k0 < n; k0 += CL_NB) {
        const int w = n - k0 < CL_NB ? n - k0 : CL_NB;
        k_trsv_diag<true><<<gd, 32 * CS_WARPS, smem, st>>>(L, lda, B, ldb, k0, w, nrhs);
        gbla_status s = launch_status();
        if (s != GBLA_SUCCESS) return s;
        const int r0 = k0 + w;
        if (r0 < n) {
            k_trsv_fwd_update<<<(unsigned)((n - r0 + CS_THREADS - 1) / CS_THREADS), CS_THREADS, 0, st>>>(
                L, lda, B, ldb, k0, w, r0, n, nrhs);
            s = launch_status();
            if (s != GBLA_SUCCESS) return s;
        }
    }
    for (int k0 = (n - 1) / CL_NB * CL_NB; k0 >= 0; k0 -= CL_NB) {
        const int w = n - k0 < CL_NB ? n - k0 : CL_NB;
        k_trsv_diag<false><<<gd, 32 * CS_WARPS, smem, st>>>(L, lda, B, ldb, k0, w, nrhs);
        gbla_status s = launch_status();
        if (s != GBLA_SUCCESS) return s;
        if (k0 > 0) {
            k_trsv_bwd_update<<<(unsigned)((k0 + CS_THREADS - 1) / CS_THREADS), CS_THREADS, 0, st>>>(L, lda, B, ldb,
                                                                                                  k0, w, nrhs);
            s = launch_status();
            if (s != GBLA_SUCCESS) return s;
        }
    }
    return GBLA_SUCCESS;
}

// ---------------------------------------------------------------------- host
// Two sets of BF16 operands (panels alternate), each n x CL_K for SA and SB.
static size_t potrf_large_ws_bytes(int n) {
    return n <= CL_NB ? 0 : (size_t)4 * n * CL_K * sizeof(__nv_bfloat16) + 256;  // one panel needs no update
}

// Side stream and events of the look-ahead, created on the first call of a
// host thread on a device and kept (one set per thread, so that concurrent
// callers never share an event).
struct LookAhead {
    cudaStream_t side = nullptr;
    cudaEvent_t panel_done = nullptr, rest_done = nullptr;
};

static gbla_status look_ahead(LookAhead *&out) {
    thread_local LookAhead tab[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GBLA_CUDA_ERROR;
    LookAhead &la = tab[dev];
    if (!la.side) {
        cudaError_t e = cudaStreamCreateWithFlags(&la.side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&la.panel_done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&la.rest_done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            la.side = nullptr;
            return from_cuda(e);
        }
    }
    out = &la;
    return GBLA_SUCCESS;
}

// Panel p (columns k0 .. k0 + w) on the caller's stream: diagonal block,
// panel solve into operand set p & 1, then the trailing update of the next
// panel's 128 columns (every row below them).  The rest of the trailing
// update (columns and rows past k0 + 2 * 128) runs on the side stream, where
// it overlaps the next panel's diagonal block and solve; the caller's stream
// waits for it before the next partial update, which writes into the same
// columns, and at the end.  Operand set p & 1 is next written by panel p + 2,
// after that wait.
static gbla_status potrf_large(int n, float *A, int64_t lda, int *info, void *ws, size_t ws_bytes, cudaStream_t st) {
    if (n < 0 || lda < n || (n > 0 && !A)) return GBLA_INVALID_VALUE;
    if (info) {
        cudaError_t e = cudaMemsetAsync(info, 0, sizeof(int), st);
        if (e != cudaSuccess) return from_cuda(e);
    }
    if (n == 0) return GBLA_SUCCESS;
    if (n > CL_NB && (!ws || ws_bytes < potrf_large_ws_bytes(n))) return GBLA_WORKSPACE_TOO_SMALL;
    const size_t smem_t = sizeof(float) * ((size_t)CL_NB * CL_LD + CL_NB) + sizeof(__nv_bfloat16) * 3 * CL_TROWS * CL_PLD;
    static bool attr_done[64] = {false};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    if (dev < 0 || dev >= 64 || !attr_done[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_trsm_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t);
        if (e != cudaSuccess) return from_cuda(e);
        if (dev >= 0 && dev < 64) attr_done[dev] = true;
    }
    LookAhead *la = nullptr;
    if (n > 2 * CL_NB) {
        gbla_status s = look_ahead(la);
        if (s != GBLA_SUCCESS) return s;
    }
    __nv_bfloat16 *base = reinterpret_cast<__nv_bfloat16 *>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    gbla_bf16_epilogue epi = {};
    epi.alpha = -1.0f;
    epi.ld_f32 = lda;
    const Bf16EpiX ex = {1.0f, 1};
    bool pending = false;  // a side-stream update not yet waited for
    gbla_status s = GBLA_SUCCESS;
    for (int k0 = 0, p = 0; k0 < n && s == GBLA_SUCCESS; k0 += CL_NB, p++) {
        const int w = n - k0 < CL_NB ? n - k0 : CL_NB;
        const int n2 = n - k0 - w;
        k_potrf_diag<<<1, CL_THREADS, 0, st>>>(A + k0 + (int64_t)k0 * lda, lda, w, k0, info);
        s = launch_status();
        if (s != GBLA_SUCCESS || n2 == 0) break;
        __nv_bfloat16 *SA = base + (size_t)(p & 1) * 2 * n * CL_K, *SB = SA + (size_t)n * CL_K;
        k_trsm_panel<<<(unsigned)((n2 + CL_TROWS - 1) / CL_TROWS), CL_THREADS, smem_t, st>>>(A, lda, k0, n2, SA, SB);
        s = launch_status();
        if (s != GBLA_SUCCESS) break;
        float *a22 = A + (k0 + CL_NB) + (int64_t)(k0 + CL_NB) * lda;
        const int m1 = n2 < CL_NB ? n2 : CL_NB;
        if (n2 > CL_NB) {
            // the rest of the update on the side stream, once the operands are written
            cudaError_t e = cudaEventRecord(la->panel_done, st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(la->side, la->panel_done, 0);
            if (e != cudaSuccess) {
                s = from_cuda(e);
                break;
            }
        }
        if (pending) {
            cudaError_t e = cudaStreamWaitEvent(st, la->rest_done, 0);
            pending = false;
            if (e != cudaSuccess) {
                s = from_cuda(e);
                break;
            }
        }
        // columns [0, 128) of A22, every row at or below the diagonal
        epi.out_f32 = a22;
        s = gemm_bf16_tn_ex(m1, n2, CL_K, SA, CL_K, SB, CL_K, epi, ex, st);
        if (s != GBLA_SUCCESS || n2 <= CL_NB) continue;
        // A22[128:, 128:]
        epi.out_f32 = a22 + CL_NB + (int64_t)CL_NB * lda;
        s = gemm_bf16_tn_ex(n2 - CL_NB, n2 - CL_NB, CL_K, SA + (size_t)CL_NB * CL_K, CL_K, SB + (size_t)CL_NB * CL_K,
                            CL_K, epi, ex, la->side);
        if (s != GBLA_SUCCESS) break;
        cudaError_t e = cudaEventRecord(la->rest_done, la->side);
        if (e != cudaSuccess) {
            s = from_cuda(e);
            break;
        }
        pending = true;
    }
    if (pending) {  // join the side stream
        cudaError_t e = cudaStreamWaitEvent(st, la->rest_done, 0);
        if (s == GBLA_SUCCESS && e != cudaSuccess) s = from_cuda(e);
    }
    return s;
}

}  // namespace gbla

using namespace gbla;

GBLA_API size_t gbla_spotrf_large_workspace_bytes(int n) { return potrf_large_ws_bytes(n); }

GBLA_API gbla_status gbla_spotrs_large(int n, int nrhs, const float *L, int64_t lda, float *B, int64_t ldb,
                                       cudaStream_t st) {
    return potrs_large(n, nrhs, L, lda, B, ldb, st);
}

GBLA_API gbla_status gbla_spotrf_large(int n, float *A, int64_t lda, int *info, void *workspace,
                                       size_t workspace_bytes, cudaStream_t st) {
    return potrf_large(n, A, lda, info, workspace, workspace_bytes, st);
}
