// wsnet.cu -- learned warm start for the one-sided Jacobi SVD.
//
// A network maps an n x n matrix A to the strictly-upper entries o of a skew
// matrix S; the warm-start frame is V0 = Vb (I - S)^{-1} (I + S) =
// Vb (2 X - I) with X = (I - S)^{-1} (a Cayley transform about a fixed base
// frame Vb), so V0 is orthogonal by construction whatever the network says.
//
// Network: n^2 -> h -> h -> P (P = n(n-1)/2), ReLU after the hidden layers.
// Weights and activations are BF16, products accumulate in FP32 on the
// tensor cores (gbla_gemm_bf16_tn), master weights and Adam state are FP32.
// Activations are row-major [batch][features]; the backward weight products
// contract over the batch, so the forward pass also writes each activation
// transposed ([features][batch]) from the GEMM epilogue and every product
// keeps both operands K-major.
//
// Loss per matrix: || V0 - V Pi D ||_F^2 with V the converged Jacobi frame;
// the permutation Pi and signs D match each predicted column to a true one
// greedily (largest |V0^T V| entry first), i.e. the distance to the nearest
// exact eigenbasis -- Jacobi does not care about column order or sign.
// Gradient through the Cayley transform: dX = X dS X, so
//   dL/dS = 2 X^T (Vb^T dL/dV0) X^T,   dL/do_ij = dL/dS_ij - dL/dS_ji.
// One block per matrix does the whole chain in shared memory (k_ws_loss).
#include <cuda_bf16.h>
#include <new>
#include "common.cuh"

namespace gbla {
gbla_status gemm_bf16_tn(int M, int N, int K, const void *A, int64_t lda, const void *B, int64_t ldb,
                         const gbla_bf16_epilogue &epi, cudaStream_t st);
}

struct gbla_wsnet {
    int n, h, P, in, maxb, ldb;
    int64_t np, o_w1, o_b1, o_w2, o_b2, o_w3, o_b3;
    float *param, *grad, *adam_m, *adam_v, *vbase, *out, *loss_mat;
    uint16_t *w1, *w2, *w2t, *w3, *w3t;
    uint16_t *x, *xt, *h1, *h1t, *h2, *h2t, *dout, *doutt, *dh2, *dh2t, *dh1t;
    int64_t step;
};

namespace gbla {
namespace {

constexpr int WS_T = 256;   // threads of the per-matrix kernels
constexpr int WS_LD = 68;   // shared-memory column stride (16-byte rows, spread banks)
constexpr int WS_MAT = 64 * WS_LD;

__device__ __forceinline__ float bf(uint16_t u) { return __bfloat162float(__ushort_as_bfloat16(u)); }
__device__ __forceinline__ uint16_t tobf(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }

// index of S(i, j), i < j, in the output vector (row-major upper triangle)
__device__ __forceinline__ int upper_index(int i, int j, int n) { return i * n - i * (i + 1) / 2 + (j - i - 1); }

__device__ __forceinline__ uint64_t splitmix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------- element-wise
__global__ void k_ws_init(float *p, int64_t np, int64_t o_b1, int64_t o_w2, int64_t o_b2, int in, int h,
                          uint64_t seed) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < np; e += (int64_t)gridDim.x * blockDim.x) {
        float bound = 0.0f;
        if (e < o_b1) bound = sqrtf(6.0f / in);                  // W1: He-uniform
        else if (e >= o_w2 && e < o_b2) bound = sqrtf(6.0f / h);  // W2
        const float u = (float)(splitmix(seed ^ (uint64_t)(e * 0x2545F4914F6CDD1Dull)) >> 40) * (1.0f / 16777216.0f);
        p[e] = bound * (2.0f * u - 1.0f);
    }
}

// BF16 copies of the weights, W2 and W3 also transposed
__global__ void k_ws_refresh(const float *p, int64_t o_w2, int64_t o_w3, int in, int h, int P, uint16_t *w1,
                             uint16_t *w2, uint16_t *w2t, uint16_t *w3, uint16_t *w3t) {
    const int64_t n1 = (int64_t)h * in, n2 = (int64_t)h * h, n3 = (int64_t)P * h;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n1 + n2 + n3;
         e += (int64_t)gridDim.x * blockDim.x) {
        if (e < n1) {
            w1[e] = tobf(p[e]);
        } else if (e < n1 + n2) {
            const int64_t f = e - n1, i = f / h, j = f % h;
            const uint16_t v = tobf(p[o_w2 + f]);
            w2[f] = v;
            w2t[j * h + i] = v;
        } else {
            const int64_t f = e - n1 - n2, i = f / h, j = f % h;
            const uint16_t v = tobf(p[o_w3 + f]);
            w3[f] = v;
            w3t[j * P + i] = v;
        }
    }
}

__global__ void k_ws_adam(int64_t np, float *p, const float *g, float *m, float *v, float lr, float bc1, float bc2) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < np; e += (int64_t)gridDim.x * blockDim.x) {
        const float ge = g[e];
        const float me = 0.9f * m[e] + 0.1f * ge;
        const float ve = 0.999f * v[e] + 0.001f * ge * ge;
        m[e] = me;
        v[e] = ve;
        p[e] -= lr * (me / bc1) / (sqrtf(ve / bc2) + 1e-8f);
    }
}

// X[b][f] = bf16(A_idx(b)[f]) (column-major vec of the matrix).  Grid: x over
// 8-element vectors of a matrix, y over matrices (in slices of 65535); one
// thread converts 8 values with two 16-byte loads and one 16-byte store when
// the matrix is 16-byte aligned (nn is a multiple of 8).
__global__ void k_ws_pack(int nn, const float *__restrict__ A, int64_t sA, const int *__restrict__ idx, int b0,
                          int batch, uint16_t *__restrict__ X) {
    const int b = b0 + blockIdx.y;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch || 8 * v >= nn) return;
    const int64_t src = idx ? idx[b] : b;
    const float *a = A + src * sA + 8 * v;
    uint16_t *x = X + (int64_t)b * nn + 8 * v;
    if ((reinterpret_cast<uintptr_t>(a) & 15) == 0) {
        const float4 p = reinterpret_cast<const float4 *>(a)[0], q = reinterpret_cast<const float4 *>(a)[1];
        uint4 u;
        u.x = (uint32_t)tobf(p.x) | ((uint32_t)tobf(p.y) << 16);
        u.y = (uint32_t)tobf(p.z) | ((uint32_t)tobf(p.w) << 16);
        u.z = (uint32_t)tobf(q.x) | ((uint32_t)tobf(q.y) << 16);
        u.w = (uint32_t)tobf(q.z) | ((uint32_t)tobf(q.w) << 16);
        *reinterpret_cast<uint4 *>(x) = u;
    } else {
#pragma unroll
        for (int e = 0; e < 8; e++) x[e] = tobf(a[e]);
    }
}

// dst[c][r] = src[r][c] for a rows x cols BF16 matrix (32 x 32 tiles)
__global__ void k_transpose_bf16(int rows, int cols, const uint16_t *src, int64_t lds, uint16_t *dst, int64_t ldd) {
    __shared__ uint16_t tile[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[k][threadIdx.x] = src[(int64_t)r * lds + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int c = c0 + k, r = r0 + threadIdx.x;
        if (r < rows && c < cols) dst[(int64_t)c * ldd + r] = tile[threadIdx.x][k];
    }
}

// dst[r] = sum_c src[r][c] (one warp per row, fixed order)
__global__ void k_rowsum_bf16(int rows, int cols, const uint16_t *src, int64_t lds, float *dst) {
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (r >= rows) return;
    float s = 0.0f;
    for (int c = lane; c < cols; c += 32) s += bf(src[(int64_t)r * lds + c]);
    s = warp_sum(s);
    if (lane == 0) dst[r] = s;
}

// out = scale * sum of v[0..len) (one block, fixed order)
__global__ void k_ws_sum(int len, const float *v, float scale, float *out) {
    __shared__ float part[32];
    float s = 0.0f;
    for (int i = threadIdx.x; i < len; i += blockDim.x) s += v[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
        *out = t * scale;
    }
}

// ------------------------------------------------- per-matrix shared-memory algebra
// All matrices n x n (n <= 64), column-major with stride WS_LD.

// D = alpha * A * B; thread t owns the 4 x 4 block at rows 4(t%16), cols 4(t/16).
// D must not alias A or B.
__device__ void sm_mm(int n, const float *A, const float *B, float *D, float alpha) {
    const int t = threadIdx.x, i0 = (t & 15) * 4, j0 = (t >> 4) * 4;
    float acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = 0.0f;
    if (i0 < n && j0 < n) {
        for (int k = 0; k < n; k++) {
            const float4 av = *reinterpret_cast<const float4 *>(A + k * WS_LD + i0);
            float bv[4];
#pragma unroll
            for (int b = 0; b < 4; b++) bv[b] = B[(j0 + b) * WS_LD + k];
#pragma unroll
            for (int b = 0; b < 4; b++) {
                acc[0][b] = fmaf(av.x, bv[b], acc[0][b]);
                acc[1][b] = fmaf(av.y, bv[b], acc[1][b]);
                acc[2][b] = fmaf(av.z, bv[b], acc[2][b]);
                acc[3][b] = fmaf(av.w, bv[b], acc[3][b]);
            }
        }
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int a = 0; a < 4; a++)
                if (i0 + a < n && j0 + b < n) D[(j0 + b) * WS_LD + i0 + a] = alpha * acc[a][b];
    }
    __syncthreads();
}

__device__ void sm_transpose(int n, const float *A, float *D) {
    for (int e = threadIdx.x; e < n * n; e += WS_T) {
        const int i = e % n, j = e / n;
        D[j * WS_LD + i] = A[i * WS_LD + j];
    }
    __syncthreads();
}

// X = (I - S)^{-1} by Gauss-Jordan without pivoting on [I - S | I].  The
// symmetric part of I - S is I, and so is that of every Schur complement, so
// every pivot has modulus >= 1 and no pivoting is needed.  The 64 x 128
// augmented matrix lives in registers: thread t owns rows 4 (t % 16) .. +3 and
// columns 8 (t / 16) .. +7 (columns 64.. are the X half; rows and columns past
// n are identity padding).  Step k: the owners of column k publish it, the
// owners of row k scale it by the pivot and publish it, every thread updates
// its block.  pcol / prow are double-buffered by the parity of k, so two
// barriers per step suffice.  X is left in shared memory (stride WS_LD).
struct GJBuf {
    float pcol[2][64];
    float prow[2][128];
};

__device__ void sm_cayley_inverse(int n, const float *o, float *X, GJBuf &gb) {
    const int t = threadIdx.x, r0 = (t & 15) * 4, c0 = (t >> 4) * 8;
    float m[4][8];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const int r = r0 + a, c = c0 + b;
            float v;
            if (c < 64) {
                v = r == c ? 1.0f : 0.0f;
                if (r < n && c < n && r != c) v = r < c ? -o[upper_index(r, c, n)] : o[upper_index(c, r, n)];
            } else {
                v = r == c - 64 ? 1.0f : 0.0f;
            }
            m[a][b] = v;
        }
    for (int kk = 0; kk < n; kk += 8) {
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const int k = kk + b;
            if (k >= n) break;
            const int par = k & 1;
            if (c0 == kk) {
#pragma unroll
                for (int a = 0; a < 4; a++) gb.pcol[par][r0 + a] = m[a][b];
            }
            __syncthreads();
            if (r0 == (k & ~3)) {
                const float inv = 1.0f / gb.pcol[par][k];
#pragma unroll
                for (int bb = 0; bb < 8; bb++) {
                    m[b & 3][bb] *= inv;
                    gb.prow[par][c0 + bb] = m[b & 3][bb];
                }
            }
            __syncthreads();
            float pr[8];
#pragma unroll
            for (int bb = 0; bb < 8; bb++) pr[bb] = gb.prow[par][c0 + bb];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                if (r0 + a == k) continue;
                const float f = gb.pcol[par][r0 + a];
#pragma unroll
                for (int bb = 0; bb < 8; bb++) m[a][bb] = fmaf(-f, pr[bb], m[a][bb]);
            }
        }
    }
    if (c0 >= 64) {
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 8; b++) X[(c0 - 64 + b) * WS_LD + r0 + a] = m[a][b];
    }
    __syncthreads();
}

// V0 = Vb (2 X - I) = 2 Vb X - Vb
__device__ void sm_frame(int n, const float *Vb, const float *X, float *V0) {
    sm_mm(n, Vb, X, V0, 2.0f);
    for (int e = threadIdx.x; e < n * n; e += WS_T) {
        const int i = e % n, j = e / n;
        V0[j * WS_LD + i] -= Vb[j * WS_LD + i];
    }
    __syncthreads();
}

// Greedy matching on C (rows: predicted columns, cols: true columns): take the
// largest |C(i, j)| over unmatched rows and columns (ties: smallest i n + j),
// n times.  When every row's best column has that row as its own best row the
// greedy result is exactly that mutual-best matching, found in one pass.
__device__ void sm_assign(int n, const float *C, int *perm, float *sgn, int *rbest, int *cbest, int *rdone,
                          int *cdone, float *wv, int *wi) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < n) {
        float bv = -1.0f;
        int bj = 0;
        for (int j = 0; j < n; j++) {
            const float a = fabsf(C[j * WS_LD + tid]);
            if (a > bv) { bv = a; bj = j; }
        }
        rbest[tid] = bj;
    } else if (tid >= 64 && tid < 64 + n) {
        const int j = tid - 64;
        float bv = -1.0f;
        int bi = 0;
        for (int i = 0; i < n; i++) {
            const float a = fabsf(C[j * WS_LD + i]);
            if (a > bv) { bv = a; bi = i; }
        }
        cbest[j] = bi;
    }
    __syncthreads();
    const int mutual = tid < n ? (cbest[rbest[tid]] == tid) : 1;
    if (__syncthreads_and(mutual)) {
        if (tid < n) {
            perm[tid] = rbest[tid];
            sgn[tid] = C[rbest[tid] * WS_LD + tid] < 0.0f ? -1.0f : 1.0f;
        }
        __syncthreads();
        return;
    }
    if (tid < n) { rdone[tid] = 0; cdone[tid] = 0; }
    __syncthreads();
    for (int it = 0; it < n; it++) {
        float bv = -1.0f;
        int bk = 0x7fffffff;
        for (int e = tid; e < n * n; e += WS_T) {  // e = i n + j (row-major key)
            const int i = e / n, j = e % n;
            if (rdone[i] || cdone[j]) continue;
            const float a = fabsf(C[j * WS_LD + i]);
            if (a > bv || (a == bv && e < bk)) { bv = a; bk = e; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(FULL, bv, o);
            const int ok = __shfl_xor_sync(FULL, bk, o);
            if (ov > bv || (ov == bv && ok < bk)) { bv = ov; bk = ok; }
        }
        if (lane == 0) { wv[warp] = bv; wi[warp] = bk; }
        __syncthreads();
        if (tid == 0) {
            float v = wv[0];
            int k = wi[0];
            for (int w = 1; w < WS_T / 32; w++)
                if (wv[w] > v || (wv[w] == v && wi[w] < k)) { v = wv[w]; k = wi[w]; }
            const int i = k / n, j = k % n;
            perm[i] = j;
            sgn[i] = C[j * WS_LD + i] < 0.0f ? -1.0f : 1.0f;
            rdone[i] = 1;
            cdone[j] = 1;
        }
        __syncthreads();
    }
}

struct LossSmem {
    int perm[64], rbest[64], cbest[64], rdone[64], cdone[64], wi[8];
    float sgn[64], wv[8], red[8];
    GJBuf gj;
};

// Loss + gradient w.r.t. the network outputs for one matrix per block.
// dout[b][p] (BF16) = dL/do_p with L = (1/batch) sum_b loss_b.
__global__ void __launch_bounds__(WS_T)
    k_ws_loss(int n, int P, const float *__restrict__ out, const float *__restrict__ Vbase,
              const float *__restrict__ V, int64_t sV, const int *__restrict__ idx, int batch, float scale,
              uint16_t *__restrict__ dout, float *__restrict__ loss_mat, int *__restrict__ assign) {
    extern __shared__ __align__(16) float wsm[];
    float *L = wsm, *X = L + WS_MAT, *Vb = X + WS_MAT, *VbT = Vb + WS_MAT, *Vt = VbT + WS_MAT, *V0 = Vt + WS_MAT,
          *T1 = V0 + WS_MAT;
    __shared__ LossSmem ls;
    const int b = blockIdx.x, tid = threadIdx.x;
    if (b >= batch) return;
    const int64_t src = idx ? idx[b] : b;
    for (int e = tid; e < n * n; e += WS_T) {
        const int i = e % n, j = e / n;
        Vb[j * WS_LD + i] = Vbase[e];
        Vt[j * WS_LD + i] = V[src * sV + e];
    }
    __syncthreads();
    sm_transpose(n, Vb, VbT);
    sm_cayley_inverse(n, out + (int64_t)b * P, X, ls.gj);
    sm_frame(n, Vb, X, V0);
    sm_transpose(n, V0, T1);
    sm_mm(n, T1, Vt, L, 1.0f);  // C = V0^T V
    sm_assign(n, L, ls.perm, ls.sgn, ls.rbest, ls.cbest, ls.rdone, ls.cdone, ls.wv, ls.wi);
    // R = V0 - V Pi D (into T1), loss = |R|^2
    float part = 0.0f;
    for (int e = tid; e < n * n; e += WS_T) {
        const int i = e % n, j = e / n;
        const float r = V0[j * WS_LD + i] - ls.sgn[j] * Vt[ls.perm[j] * WS_LD + i];
        T1[j * WS_LD + i] = r;
        part = fmaf(r, r, part);
    }
    part = warp_sum(part);
    if ((tid & 31) == 0) ls.red[tid >> 5] = part;
    __syncthreads();
    if (tid == 0) {
        float t = 0.0f;
        for (int w = 0; w < WS_T / 32; w++) t += ls.red[w];
        loss_mat[b] = t;
    }
    if (assign && tid < n) assign[(int64_t)b * n + tid] = (int)ls.sgn[tid] * (ls.perm[tid] + 1);
    sm_mm(n, VbT, T1, L, 2.0f * scale);  // dL/dCay = Vb^T dL/dV0, dL/dV0 = 2 scale R
    sm_transpose(n, X, T1);              // X^T
    sm_mm(n, T1, L, V0, 2.0f);           // 2 X^T dCay
    sm_mm(n, V0, T1, L, 1.0f);           // dS = 2 X^T dCay X^T
    uint16_t *d = dout + (int64_t)b * P;
    for (int p = tid; p < P; p += WS_T) {
        // invert p -> (i, j): row i holds n - 1 - i entries
        int i = 0, base = 0;
        while (base + (n - 1 - i) <= p) { base += n - 1 - i; i++; }
        const int j = i + 1 + (p - base);
        d[p] = tobf(L[j * WS_LD + i] - L[i * WS_LD + j]);
    }
}

// V0 for a batch, without forming the inverse: V0 = Vb (2 (I - S)^{-1} - I),
// so V0^T = 2 (I + S)^{-1} Vb^T - Vb^T: a Gauss-Jordan elimination of
// [I + S | Vb^T] (64 x 128 in registers; I + S has symmetric part I, so no
// pivoting) leaves D Y in the right half, D the diagonal the left half ends
// as and Y = (I + S)^{-1} Vb^T.  Thread t holds rows 4 (t >> 4) + a and
// columns 8 (t & 15) + q, so warp w holds rows 8w .. 8w + 7 across all 128
// columns.  The elimination runs in eight blocks of eight pivots: warp b
// eliminates within its own rows (pivot row and column by shuffle, no block
// barrier), publishes its rows and every row's entries in its pivot columns,
// and after one block barrier every other warp applies the rank-8 update
// (row i loses sum_p (m_{i,8b+p} / d_p) R_p: the block's rows R_p are zero in
// each other's pivot columns).  Pivot rows are never scaled; D is divided
// out at the end.  The network outputs are staged through shared memory so
// that their global reads are coalesced.  Thread (row r, column c of Y)
// writes V0[r n + c] = V0(c, r) = 2 Y(r, c) - Vb(c, r), contiguous in c.
struct FrameBuf {
    float o[64 * 63 / 2];    // the network outputs of the matrix (strict upper triangle of S)
    float prow[2][8][128];   // the pivot block's rows, double-buffered by block parity
    float pcol[2][64][8];    // every row's entries in the block's pivot columns
    float dinv[64];          // 1 / d_k
};

__global__ void __launch_bounds__(WS_T, 3)
    k_ws_frame(int n, int P, const float *__restrict__ out, const float *__restrict__ Vbase, float *__restrict__ V0g,
               int64_t sV0, int batch) {
    __shared__ __align__(16) FrameBuf fb;
    const int t = threadIdx.x, rg = t >> 4, cg = t & 15, r0 = 4 * rg, c0 = 8 * cg;
    const int warp = t >> 5, lane = t & 31;
    const int nblk = (n + 7) >> 3;
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        const float *o = out + (int64_t)b * P;
        __syncthreads();  // the previous matrix is done with the buffers
        for (int e = t; e < P; e += WS_T) fb.o[e] = o[e];
        __syncthreads();
        float m[4][8];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int r = r0 + a, c = c0 + q;
                float v;
                if (c < 64) {
                    v = r == c ? 1.0f : 0.0f;
                    if (r < n && c < n && r != c) v = r < c ? fb.o[upper_index(r, c, n)] : -fb.o[upper_index(c, r, n)];
                } else {
                    // Vb^T(r, c - 64) = Vb(c - 64, r), column-major Vb
                    v = (r < n && c - 64 < n) ? Vbase[r * n + (c - 64)] : 0.0f;
                }
                m[a][q] = v;
            }
        for (int blk = 0; blk < nblk; blk++) {
            const int par = blk & 1;
            if (warp == blk) {
                // eliminate within rows 8 blk .. 8 blk + 7: pivot k = 8 blk + p sits in
                // lane 16 (p >> 2) + cg (row slot p & 3), its column in column group blk
#pragma unroll
                for (int p = 0; p < 8; p++) {
                    const int src_row = 16 * (p >> 2);
                    float pr[8];
#pragma unroll
                    for (int q = 0; q < 8; q++) pr[q] = shfl(m[p & 3][q], src_row + cg);
                    const float piv = shfl(m[p & 3][p], src_row + blk);
                    float f[4];
#pragma unroll
                    for (int a = 0; a < 4; a++) f[a] = shfl(m[a][p], (lane & 16) + blk);
                    const float ip = 1.0f / piv;
#pragma unroll
                    for (int a = 0; a < 4; a++) {
                        if ((lane >> 4) == (p >> 2) && a == (p & 3)) continue;  // the pivot row itself
                        const float fa = f[a] * ip;
#pragma unroll
                        for (int q = 0; q < 8; q++) m[a][q] = fmaf(-fa, pr[q], m[a][q]);
                    }
                    if (lane == 0) fb.dinv[8 * blk + p] = ip;
                }
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int q = 0; q < 8; q++) fb.prow[par][4 * (lane >> 4) + a][c0 + q] = m[a][q];
            }
            if (cg == blk && warp != blk) {
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int q = 0; q < 8; q++) fb.pcol[par][r0 + a][q] = m[a][q];
            }
            __syncthreads();
            if (warp != blk) {
                float di[8];
#pragma unroll
                for (int p = 0; p < 8; p++) di[p] = fb.dinv[8 * blk + p];
#pragma unroll
                for (int p = 0; p < 8; p++) {
                    float pr[8];
#pragma unroll
                    for (int q = 0; q < 8; q++) pr[q] = fb.prow[par][p][c0 + q];
#pragma unroll
                    for (int a = 0; a < 4; a++) {
                        const float fa = fb.pcol[par][r0 + a][p] * di[p];
#pragma unroll
                        for (int q = 0; q < 8; q++) m[a][q] = fmaf(-fa, pr[q], m[a][q]);
                    }
                }
            }
        }
        __syncthreads();  // every 1 / d_k is published
        if (c0 >= 64) {
            float *dst = V0g + (int64_t)b * sV0;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int r = r0 + a;
                if (r >= n) continue;
                const float inv = fb.dinv[r];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int c = c0 - 64 + q;
                    if (c < n) dst[r * n + c] = 2.0f * (m[a][q] * inv) - Vbase[r * n + c];
                }
            }
        }
    }
}

constexpr size_t LOSS_SMEM = 7 * WS_MAT * sizeof(float);
constexpr size_t FRAME_SMEM = 0;

unsigned grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * 16;
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

gbla_bf16_epilogue epilogue() {
    gbla_bf16_epilogue e;
    e.alpha = 1.0f;
    e.bias = nullptr;
    e.relu = 0;
    e.mask = nullptr;
    e.ld_mask = 0;
    e.out_f32 = nullptr;
    e.ld_f32 = 0;
    e.out_bf16 = nullptr;
    e.ld_bf16 = 0;
    e.out_bf16_t = nullptr;
    e.ld_bf16_t = 0;
    return e;
}

#define WS_TRY(x)                                   \
    do {                                            \
        gbla_status s_ = (x);                       \
        if (s_ != GBLA_SUCCESS) return s_;          \
    } while (0)

gbla_status transpose(int rows, int cols, const uint16_t *src, int64_t lds, uint16_t *dst, int64_t ldd,
                      cudaStream_t st) {
    dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32)), block(32, 8);
    k_transpose_bf16<<<grid, block, 0, st>>>(rows, cols, src, lds, dst, ldd);
    return launch_status();
}

gbla_status rowsum(int rows, int cols, const uint16_t *src, int64_t lds, float *dst, cudaStream_t st) {
    k_rowsum_bf16<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, st>>>(rows, cols, src, lds, dst);
    return launch_status();
}

// Forward pass for `batch` matrices; with `train` the transposed activations
// the backward pass needs are written too.
gbla_status forward(gbla_wsnet *w, const float *A, int64_t sA, const int *idx, int batch, bool train,
                    cudaStream_t st) {
    for (int b0 = 0; b0 < batch; b0 += 65535) {
        const int nbat = batch - b0 < 65535 ? batch - b0 : 65535;
        dim3 pg((unsigned)((w->in / 8 + 255) / 256), (unsigned)nbat);
        k_ws_pack<<<pg, 256, 0, st>>>(w->in, A, sA, idx, b0, batch, w->x);
        WS_TRY(launch_status());
    }
    if (train) WS_TRY(transpose(batch, w->in, w->x, w->in, w->xt, w->ldb, st));
    gbla_bf16_epilogue e = epilogue();
    e.bias = w->param + w->o_b1;
    e.relu = 1;
    e.out_bf16 = w->h1;
    e.ld_bf16 = w->h;
    if (train) { e.out_bf16_t = w->h1t; e.ld_bf16_t = w->ldb; }
    WS_TRY(gemm_bf16_tn(batch, w->h, w->in, w->x, w->in, w->w1, w->in, e, st));
    e.bias = w->param + w->o_b2;
    e.out_bf16 = w->h2;
    if (train) e.out_bf16_t = w->h2t;
    WS_TRY(gemm_bf16_tn(batch, w->h, w->h, w->h1, w->h, w->w2, w->h, e, st));
    e = epilogue();
    e.bias = w->param + w->o_b3;
    e.out_f32 = w->out;
    e.ld_f32 = w->P;
    return gemm_bf16_tn(batch, w->P, w->h, w->h2, w->h, w->w3, w->h, e, st);
}

// Loss and gradients into w->grad (after forward(..., train = true)).
gbla_status backward(gbla_wsnet *w, const float *V, int64_t sV, const int *idx, int batch, float *loss, int *assign,
                     cudaStream_t st) {
    const int n = w->n, h = w->h, P = w->P, B = batch;
    k_ws_loss<<<(unsigned)B, WS_T, LOSS_SMEM, st>>>(n, P, w->out, w->vbase, V, sV, idx, B, 1.0f / B, w->dout,
                                                    w->loss_mat, assign);
    WS_TRY(launch_status());
    if (loss) {
        k_ws_sum<<<1, 256, 0, st>>>(B, w->loss_mat, 1.0f / B, loss);
        WS_TRY(launch_status());
    }
    WS_TRY(transpose(B, P, w->dout, P, w->doutt, w->ldb, st));
    gbla_bf16_epilogue e = epilogue();
    // dW3 = dO^T H2, db3 = column sums of dO
    e.out_f32 = w->grad + w->o_w3;
    e.ld_f32 = h;
    WS_TRY(gemm_bf16_tn(P, h, B, w->doutt, w->ldb, w->h2t, w->ldb, e, st));
    WS_TRY(rowsum(P, B, w->doutt, w->ldb, w->grad + w->o_b3, st));
    // dH2 = (dO W3) * [H2 > 0]
    e = epilogue();
    e.mask = w->h2;
    e.ld_mask = h;
    e.out_bf16 = w->dh2;
    e.ld_bf16 = h;
    e.out_bf16_t = w->dh2t;
    e.ld_bf16_t = w->ldb;
    WS_TRY(gemm_bf16_tn(B, h, P, w->dout, P, w->w3t, P, e, st));
    // dW2 = dH2^T H1, db2
    e = epilogue();
    e.out_f32 = w->grad + w->o_w2;
    e.ld_f32 = h;
    WS_TRY(gemm_bf16_tn(h, h, B, w->dh2t, w->ldb, w->h1t, w->ldb, e, st));
    WS_TRY(rowsum(h, B, w->dh2t, w->ldb, w->grad + w->o_b2, st));
    // dH1 = (dH2 W2) * [H1 > 0], kept transposed only
    e = epilogue();
    e.mask = w->h1;
    e.ld_mask = h;
    e.out_bf16_t = w->dh1t;
    e.ld_bf16_t = w->ldb;
    WS_TRY(gemm_bf16_tn(B, h, h, w->dh2, h, w->w2t, h, e, st));
    // dW1 = dH1^T X, db1
    e = epilogue();
    e.out_f32 = w->grad + w->o_w1;
    e.ld_f32 = w->in;
    WS_TRY(gemm_bf16_tn(h, w->in, B, w->dh1t, w->ldb, w->xt, w->ldb, e, st));
    return rowsum(h, B, w->dh1t, w->ldb, w->grad + w->o_b1, st);
}

gbla_status refresh(gbla_wsnet *w, cudaStream_t st) {
    const int64_t tot = (int64_t)w->h * w->in + (int64_t)w->h * w->h + (int64_t)w->P * w->h;
    k_ws_refresh<<<grid_for(tot, 256), 256, 0, st>>>(w->param, w->o_w2, w->o_w3, w->in, w->h, w->P, w->w1, w->w2,
                                                     w->w2t, w->w3, w->w3t);
    return launch_status();
}

bool smem_attrs() {
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return false;
    if (!done[dev]) {
        if (cudaFuncSetAttribute(k_ws_loss, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LOSS_SMEM) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_ws_frame, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FRAME_SMEM) !=
                cudaSuccess)
            return false;
        done[dev] = true;
    }
    return true;
}

bool batch_ok(const gbla_wsnet *w, const float *A, int64_t sA, int batch) {
    return w && A && batch >= 1 && batch <= w->maxb && sA >= (int64_t)w->n * w->n;
}

}  // namespace
}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_wsnet_create(int n, int hidden, int max_batch, uint64_t seed, gbla_wsnet **net) {
    if (!net) return GBLA_INVALID_VALUE;
    *net = nullptr;
    const int P = n * (n - 1) / 2;
    if (n < 2 || n > 64 || (n * n) % 8 || P % 8 || hidden < 64 || hidden % 64 || max_batch < 1)
        return GBLA_INVALID_VALUE;
    gbla_wsnet *w = new (std::nothrow) gbla_wsnet();
    if (!w) return GBLA_CUDA_ERROR;
    w->n = n;
    w->h = hidden;
    w->P = P;
    w->in = n * n;
    w->maxb = max_batch;
    w->ldb = (int)round_up(max_batch, 8);
    w->o_w1 = 0;
    w->o_b1 = (int64_t)hidden * w->in;
    w->o_w2 = w->o_b1 + hidden;
    w->o_b2 = w->o_w2 + (int64_t)hidden * hidden;
    w->o_w3 = w->o_b2 + hidden;
    w->o_b3 = w->o_w3 + (int64_t)P * hidden;
    w->np = w->o_b3 + P;
    const int64_t B = max_batch, L = w->ldb, h = hidden;
    bool ok = true;
    auto alloc = [&](auto **p, int64_t count) {
        if (!ok) return;
        void *q = nullptr;
        if (cudaMalloc(&q, (size_t)count * sizeof(**p)) != cudaSuccess) ok = false;
        *p = static_cast<std::remove_reference_t<decltype(*p)>>(q);
    };
    alloc(&w->param, w->np);
    alloc(&w->grad, w->np);
    alloc(&w->adam_m, w->np);
    alloc(&w->adam_v, w->np);
    alloc(&w->vbase, (int64_t)n * n);
    alloc(&w->out, B * P);
    alloc(&w->loss_mat, B);
    alloc(&w->w1, h * w->in);
    alloc(&w->w2, h * h);
    alloc(&w->w2t, h * h);
    alloc(&w->w3, (int64_t)P * h);
    alloc(&w->w3t, (int64_t)P * h);
    alloc(&w->x, B * w->in);
    alloc(&w->xt, (int64_t)w->in * L);
    alloc(&w->h1, B * h);
    alloc(&w->h1t, h * L);
    alloc(&w->h2, B * h);
    alloc(&w->h2t, h * L);
    alloc(&w->dout, B * P);
    alloc(&w->doutt, (int64_t)P * L);
    alloc(&w->dh2, B * h);
    alloc(&w->dh2t, h * L);
    alloc(&w->dh1t, h * L);
    if (!ok) {
        gbla_wsnet_destroy(w);
        return from_cuda(cudaErrorMemoryAllocation);
    }
    // transposed activations: the columns past the batch are read as K tail
    cudaMemset(w->xt, 0, (size_t)w->in * L * 2);
    k_ws_init<<<grid_for(w->np, 256), 256>>>(w->param, w->np, w->o_b1, w->o_w2, w->o_b2, w->in, hidden, seed);
    gbla_status s = launch_status();
    if (s == GBLA_SUCCESS) s = refresh(w, 0);
    if (s == GBLA_SUCCESS) s = from_cuda(cudaMemset(w->adam_m, 0, (size_t)w->np * 4));
    if (s == GBLA_SUCCESS) s = from_cuda(cudaMemset(w->adam_v, 0, (size_t)w->np * 4));
    if (s == GBLA_SUCCESS) {
        float *eye = new (std::nothrow) float[(size_t)n * n];
        if (!eye) s = GBLA_CUDA_ERROR;
        else {
            for (int e = 0; e < n * n; e++) eye[e] = (e % n == e / n) ? 1.0f : 0.0f;
            s = from_cuda(cudaMemcpy(w->vbase, eye, (size_t)n * n * 4, cudaMemcpyHostToDevice));
            delete[] eye;
        }
    }
    if (s == GBLA_SUCCESS) s = from_cuda(cudaDeviceSynchronize());
    if (s != GBLA_SUCCESS || !smem_attrs()) {
        gbla_wsnet_destroy(w);
        return s != GBLA_SUCCESS ? s : GBLA_CUDA_ERROR;
    }
    *net = w;
    return GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_wsnet_destroy(gbla_wsnet *w) {
    if (!w) return GBLA_SUCCESS;
    void *bufs[] = {w->param, w->grad, w->adam_m, w->adam_v, w->vbase, w->out, w->loss_mat, w->w1, w->w2, w->w2t,
                    w->w3, w->w3t, w->x, w->xt, w->h1, w->h1t, w->h2, w->h2t, w->dout, w->doutt, w->dh2, w->dh2t,
                    w->dh1t};
    for (void *p : bufs)
        if (p) cudaFree(p);
    delete w;
    return GBLA_SUCCESS;
}

GBLA_API int64_t gbla_wsnet_param_count(const gbla_wsnet *w) { return w ? w->np : -1; }

GBLA_API gbla_status gbla_wsnet_get_params(const gbla_wsnet *w, float *params, cudaStream_t st) {
    if (!w || !params) return GBLA_INVALID_VALUE;
    return from_cuda(cudaMemcpyAsync(params, w->param, (size_t)w->np * 4, cudaMemcpyDeviceToDevice, st));
}

GBLA_API gbla_status gbla_wsnet_set_params(gbla_wsnet *w, const float *params, cudaStream_t st) {
    if (!w || !params) return GBLA_INVALID_VALUE;
    WS_TRY(from_cuda(cudaMemcpyAsync(w->param, params, (size_t)w->np * 4, cudaMemcpyDeviceToDevice, st)));
    WS_TRY(from_cuda(cudaMemsetAsync(w->adam_m, 0, (size_t)w->np * 4, st)));
    WS_TRY(from_cuda(cudaMemsetAsync(w->adam_v, 0, (size_t)w->np * 4, st)));
    w->step = 0;
    return refresh(w, st);
}

GBLA_API gbla_status gbla_wsnet_get_base(const gbla_wsnet *w, float *Vb, cudaStream_t st) {
    if (!w || !Vb) return GBLA_INVALID_VALUE;
    return from_cuda(cudaMemcpyAsync(Vb, w->vbase, (size_t)w->n * w->n * 4, cudaMemcpyDeviceToDevice, st));
}

GBLA_API gbla_status gbla_wsnet_set_base(gbla_wsnet *w, const float *Vb, cudaStream_t st) {
    if (!w || !Vb) return GBLA_INVALID_VALUE;
    return from_cuda(cudaMemcpyAsync(w->vbase, Vb, (size_t)w->n * w->n * 4, cudaMemcpyDeviceToDevice, st));
}

GBLA_API gbla_status gbla_wsnet_gradients(gbla_wsnet *w, const float *A, int64_t sA, const float *V, int64_t sV,
                                          const int *idx, int batch, float *grad, float *loss, int *assign,
                                          cudaStream_t st) {
    if (!batch_ok(w, A, sA, batch) || !V || sV < (int64_t)w->n * w->n || !grad || !smem_attrs())
        return GBLA_INVALID_VALUE;
    WS_TRY(forward(w, A, sA, idx, batch, true, st));
    WS_TRY(backward(w, V, sV, idx, batch, loss, assign, st));
    return from_cuda(cudaMemcpyAsync(grad, w->grad, (size_t)w->np * 4, cudaMemcpyDeviceToDevice, st));
}

GBLA_API gbla_status gbla_wsnet_train_step(gbla_wsnet *w, const float *A, int64_t sA, const float *V, int64_t sV,
                                           const int *idx, int batch, float lr, float *loss, cudaStream_t st) {
    if (!batch_ok(w, A, sA, batch) || !V || sV < (int64_t)w->n * w->n || !(lr > 0.0f) || !smem_attrs())
        return GBLA_INVALID_VALUE;
    WS_TRY(forward(w, A, sA, idx, batch, true, st));
    WS_TRY(backward(w, V, sV, idx, batch, loss, nullptr, st));
    w->step++;
    const float bc1 = 1.0f - powf(0.9f, (float)w->step), bc2 = 1.0f - powf(0.999f, (float)w->step);
    k_ws_adam<<<grid_for(w->np, 256), 256, 0, st>>>(w->np, w->param, w->grad, w->adam_m, w->adam_v, lr, bc1, bc2);
    WS_TRY(launch_status());
    return refresh(w, st);
}

GBLA_API gbla_status gbla_wsnet_predict(gbla_wsnet *w, const float *A, int64_t sA, float *V0, int64_t sV0, int batch,
                                        cudaStream_t st) {
    if (!w || batch < 0) return GBLA_INVALID_VALUE;
    if (batch == 0) return GBLA_SUCCESS;
    if (!A || !V0 || sA < (int64_t)w->n * w->n || sV0 < (int64_t)w->n * w->n || !smem_attrs())
        return GBLA_INVALID_VALUE;
    for (int b0 = 0; b0 < batch; b0 += w->maxb) {
        const int nb = batch - b0 < w->maxb ? batch - b0 : w->maxb;
        WS_TRY(forward(w, A + (int64_t)b0 * sA, sA, nullptr, nb, false, st));
        // persistent blocks: exactly the resident count, so no block waits for
        // another's whole loop to finish
        const int grid = (int)persistent_grid(reinterpret_cast<const void *>(k_ws_frame), WS_T, FRAME_SMEM, nb);
        k_ws_frame<<<(unsigned)grid, WS_T, FRAME_SMEM, st>>>(w->n, w->P, w->out, w->vbase, V0 + (int64_t)b0 * sV0, sV0,
                                                           nb);
        WS_TRY(launch_status());
    }
    return GBLA_SUCCESS;
}
