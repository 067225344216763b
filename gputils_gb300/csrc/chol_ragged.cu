// chol_ragged.cu -- one call that factors and solves a ragged batch of SPD
// systems of mixed sizes (1 <= n <= 128, any nrhs), with iterative refinement.
//
// The reference has no ragged API: a mixed batch is one
// CholeskyBatchFactoriser per size and one potrs per right-hand-side column
// (include/tensor.cuh:2100-2197).  Here a host-built plan sorts the systems
// and cuts them into tasks, and a call is ONE persistent kernel launch whose
// blocks pull tasks from a device queue (an atomic counter; a block that finds
// the queue empty leaves, and the last block to leave resets the counter for
// the next call, so a call needs no memset and replays in a CUDA graph):
//   * n > 32   : a task is a group of 1..systems_per_block systems of similar
//                size (largest first), each worked on by threads/32/count
//                warps in its own shared-memory slot: blocked factorisation
//                (one warp factors an 8-column panel while the others apply
//                the previous panel's update; a named barrier per system), one
//                warp per right-hand side for the solves and refinement.
//   * n <= 32  : three size classes (n <= 8, 16, 32) run the lane-row method
//                (NB lanes per system, rows in registers, shuffles only); a
//                task is one class's systems for every warp of the block.
//                Within a warp the loop bounds are the warp's largest n /
//                nrhs; smaller systems are padded with the identity, which
//                leaves their factor and solution unchanged.
// Tasks are queued largest first (LPT), so the queue balances the n^3 spread
// of the work across the persistent blocks.  The launch configuration --
// threads per block and the most large systems a block takes at once (which
// sets its shared memory and with it the blocks per SM) -- is a plan
// property; gbla_{s,d}ragged_autotune times every candidate on the caller's
// batch and keeps the fastest.  Every configuration gives bit-identical
// results: each element of each system receives its updates in the same
// order whatever the grouping.
//
// Precision: the factorisation and the triangular solves run in FP32; each
// refinement step recomputes r = b - A x from the original, full symmetric A
// (lower and upper triangles) in extended precision -- double-FP32 for float
// data, FP64 for double data -- and adds the FP32 correction.
#include <algorithm>
#include <new>
#include <vector>
#include "chol_common.cuh"
#include "xprec.cuh"

struct RaggedSys {
    int64_t a_off, b_off;
    int n, nrhs, orig, pad;
};

// A task of the persistent launch: `count` systems from sys[first] on, either
// a group of large systems (nb == 0; `warps` warps and one shared-memory slot
// sized for nmax each) or a chunk of one small class (nb = lanes per system).
struct RaggedTask {
    int first, count, nb, warps, nmax, pad;
};

struct gbla_ragged_plan {
    int device = -1;
    int count = 0;
    int first[4] = {0, 0, 0, 0};   // classes: NB 8, NB 16, NB 32, large
    int num[4] = {0, 0, 0, 0};
    int max_n_large = 0;
    gbla_ragged_config cfg = {256, 2};
    int ntasks = 0;
    size_t smem = 0;                     // dynamic shared memory per block for cfg
    int64_t a_extent = 0, b_extent = 0;  // arena sizes in elements
    std::vector<int> large_n;            // n of the large class, in plan order
    RaggedSys *d_sys = nullptr;
    RaggedTask *d_tasks = nullptr;       // capacity: count tasks
    int *d_ctr = nullptr;                // queue head, blocks finished
};

namespace gbla {


// ------------------------------------------------------------ small systems
// One warp's share of a small-class task: systems first + warp * GPW + g.
template <typename T, int NB>
__device__ __forceinline__ void small_systems(const RaggedSys *__restrict__ sys, int first, int count, int warp,
                                              int lane, const T *__restrict__ A_in, T *__restrict__ A,
                                              T *__restrict__ B, int *__restrict__ info, int refine) {
    constexpr int GPW = 32 / NB;
    const int g = lane / NB, r = lane % NB;
    const int local = warp * GPW + g;
    const bool act = local < count;
    RaggedSys s = {0, 0, 0, 0, 0, 0};
    if (act) s = sys[first + local];
    const int n = s.n, nrhs = s.nrhs;
    int nw = n, rw = nrhs;  // warp-uniform loop bounds
#pragma unroll
    for (int o = NB; o < 32; o <<= 1) {
        nw = max(nw, shfl_xor(nw, o));
        rw = max(rw, shfl_xor(rw, o));
    }
    const bool rowok = act && r < n;
    const T *ag = A_in + s.a_off;
    float a[NB];
#pragma unroll
    for (int j = 0; j < NB; j++) {
        bool ld = rowok && j < n && j <= r;
        a[j] = ld ? (float)ag[(int64_t)j * n + r] : (r == j ? 1.f : 0.f);
    }
    float dinv = 1.f;
    int fail = 0;
    lr_factor<float, NB>(a, dinv, fail, nw, r);
    if (act && r == 0 && info) info[s.orig] = fail;
    T *bg = B + s.b_off;
    for (int c = 0; c < rw; c++) {
        const bool has = rowok && c < nrhs;
        const T b = has ? bg[(int64_t)c * n + r] : T(0);
        float x = lr_solve<float, NB>(a, dinv, (float)b, nw, r);
        T xo;
        if constexpr (sizeof(T) == 4) {
            float xh = x, xl = 0.f;
            for (int it = 0; it < refine; it++) {
                ff f = {(float)b, 0.f};
                for (int j = 0; j < nw; j++) {
                    const float xjh = shfl(xh, j, NB), xjl = shfl(xl, j, NB);
                    const float aij = (rowok && j < n) ? (float)ag[(int64_t)j * n + r] : 0.f;
                    ff_fma(f, -aij, xjh, xjl);
                }
                const float d = lr_solve<float, NB>(a, dinv, has ? f.h + f.l : 0.f, nw, r);
                float sum, e;
                two_sum(xh, d, sum, e);
                const float l = xl + e;
                xh = sum + l;
                xl = l - (xh - sum);
            }
            xo = (T)(xh + xl);
        } else {
            double xd = (double)x;
            for (int it = 0; it < refine; it++) {
                double acc = (double)b;
                for (int j = 0; j < nw; j++) {
                    const double xj = shfl(xd, j, NB);
                    const double aij = (rowok && j < n) ? (double)ag[(int64_t)j * n + r] : 0.0;
                    acc = fma(-aij, xj, acc);
                }
                const float d = lr_solve<float, NB>(a, dinv, has ? (float)acc : 0.f, nw, r);
                xd += (double)d;
            }
            xo = (T)xd;
        }
        if (has) bg[(int64_t)c * n + r] = xo;
    }
    if (rowok) {
        T *aw = A + s.a_off;
#pragma unroll
        for (int j = 0; j < NB; j++)
            if (j < n && j <= r) aw[(int64_t)j * n + r] = (T)a[j];
    }
}

// ------------------------------------------------------------ large systems
// Shared-memory slot of one large system: two panel-row buffers (n x 8 each),
// the FP32 factor (n x ld), 1 / L_kk (n) and the failure flag; a multiple of
// 16 bytes so that consecutive slots stay 16-byte aligned.
__host__ __device__ inline size_t ragged_slot_bytes(int nmax) {
    const int ld = cta_ld(nmax);
    return (sizeof(float) * ((size_t)nmax * 16 + (size_t)nmax * ld + (size_t)nmax) + 16 + 15) & ~(size_t)15;
}

// Solve L L^T x = b for one column held in registers (element lane + 32 t in
// x[t], n <= 128): the pivot value travels by shuffle, L is read from shared
// memory (column-major, odd stride, so row and column walks are both
// conflict-free).  The step loop runs over (register chunk tk, lane lk) with
// tk known at compile time, so the pivot register needs no select and only
// the pivot's own chunk needs a row comparison.  Per element the updates run
// in the same order as a column-oriented shared-memory solve.
__device__ __forceinline__ void reg_solve(const float *__restrict__ a, int ld, const float *__restrict__ dinv,
                                          float (&x)[4], int n, int lane) {
    const int nt = (n + 31) >> 5;
#pragma unroll
    for (int tk = 0; tk < 4; tk++) {
        if (tk >= nt) break;
        const int kmax = n - 32 * tk < 32 ? n - 32 * tk : 32;
        for (int lk = 0; lk < kmax; lk++) {
            const int k = 32 * tk + lk;
            const float yk = shfl(x[tk], lk) * dinv[k];
            if (lane == lk) x[tk] = yk;
            const float *col = a + k * ld + lane;
            if (lane > lk) x[tk] = fmaf(-col[32 * tk], yk, x[tk]);
#pragma unroll
            for (int t = tk + 1; t < 4; t++)
                if (t < nt) x[t] = fmaf(-col[32 * t], yk, x[t]);
        }
    }
#pragma unroll
    for (int tk = 3; tk >= 0; tk--) {
        if (tk >= nt) continue;
        const int kmax = n - 32 * tk < 32 ? n - 32 * tk : 32;
        for (int lk = kmax - 1; lk >= 0; lk--) {
            const int k = 32 * tk + lk;
            const float zk = shfl(x[tk], lk) * dinv[k];
            if (lane == lk) x[tk] = zk;
            const float *row = a + lane * ld + k;  // L(k, i) for i = lane + 32 t
            if (lane < lk) x[tk] = fmaf(-row[32 * tk * ld], zk, x[tk]);
#pragma unroll
            for (int t = 0; t < tk; t++) x[t] = fmaf(-row[32 * t * ld], zk, x[t]);
        }
    }
}

constexpr int RG_PANEL = 8;

// Warp 0: factor the panel of columns [k0, k0 + pw) (rows k0 .. n-1, held in
// registers as rows k0 + lane + 32 t), write it back into the factor and,
// row-major, into pbuf for the rank-8 updates.
__device__ __forceinline__ void panel_factor(float *__restrict__ a, int ld, int n, int k0, int pw,
                                             float *__restrict__ pbuf, float *__restrict__ dinv, int *s_fail,
                                             int lane) {
    float pv[4][RG_PANEL];
#pragma unroll
    for (int t = 0; t < 4; t++)
#pragma unroll
        for (int c = 0; c < RG_PANEL; c++) {
            const int r = k0 + lane + 32 * t;
            pv[t][c] = (c < pw && r < n) ? a[(k0 + c) * ld + r] : 0.f;
        }
#pragma unroll
    for (int c = 0; c < RG_PANEL; c++) {
        if (c >= pw) break;
        const int k = k0 + c;
        const float d = shfl(pv[0][c], c);  // row k sits in lane c, t = 0
        if (!(d > 0.f) && lane == 0 && *s_fail == 0) *s_fail = k + 1;
        const float l = sqrtf(d), il = 1.f / l;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int r = k0 + lane + 32 * t;
            if (r > k) pv[t][c] *= il;
        }
        if (lane == c) pv[0][c] = l;
        if (lane == 0) dinv[k] = il;
#pragma unroll
        for (int c2 = c + 1; c2 < RG_PANEL; c2++) {
            if (c2 >= pw) break;
            const float ljk = shfl(pv[0][c], c2);  // L(k0 + c2, k)
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int r = k0 + lane + 32 * t;
                if (r >= k0 + c2) pv[t][c2] = fmaf(-pv[t][c], ljk, pv[t][c2]);
            }
        }
    }
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const int r = k0 + lane + 32 * t;
        if (r >= n) continue;
#pragma unroll
        for (int c = 0; c < RG_PANEL; c++)
            if (c < pw && r >= k0 + c) a[(k0 + c) * ld + r] = pv[t][c];
        // the panel's rows for the rank-8 updates, row-major (zero past pw)
        float4 *pr = reinterpret_cast<float4 *>(pbuf + 8 * r);
        pr[0] = make_float4(pv[t][0], pw > 1 ? pv[t][1] : 0.f, pw > 2 ? pv[t][2] : 0.f, pw > 3 ? pv[t][3] : 0.f);
        pr[1] = make_float4(pw > 4 ? pv[t][4] : 0.f, pw > 5 ? pv[t][5] : 0.f, pw > 6 ? pv[t][6] : 0.f,
                            pw > 7 ? pv[t][7] : 0.f);
    }
}

// Rank-8 update of the lower-triangle columns j = j_lo + wi, + ws, ... < j_hi
// (rows j .. n-1) with the panel rows in pbuf: increasing k, one fma each
// (zeros past the panel width leave the value unchanged).
__device__ __forceinline__ void panel_update(float *__restrict__ a, int ld, int n, const float *__restrict__ pbuf,
                                             int j_lo, int j_hi, int wi, int ws, int lane) {
    for (int j = j_lo + wi; j < j_hi; j += ws) {
        const float4 lj0 = reinterpret_cast<const float4 *>(pbuf + 8 * j)[0];
        const float4 lj1 = reinterpret_cast<const float4 *>(pbuf + 8 * j)[1];
        float *colj = a + j * ld;
        for (int i = j + lane; i < n; i += 32) {
            const float4 li0 = reinterpret_cast<const float4 *>(pbuf + 8 * i)[0];
            const float4 li1 = reinterpret_cast<const float4 *>(pbuf + 8 * i)[1];
            float acc = colj[i];
            acc = fmaf(-li0.x, lj0.x, acc);
            acc = fmaf(-li0.y, lj0.y, acc);
            acc = fmaf(-li0.z, lj0.z, acc);
            acc = fmaf(-li0.w, lj0.w, acc);
            acc = fmaf(-li1.x, lj1.x, acc);
            acc = fmaf(-li1.y, lj1.y, acc);
            acc = fmaf(-li1.z, lj1.z, acc);
            acc = fmaf(-li1.w, lj1.w, acc);
            colj[i] = acc;
        }
    }
}

// x_j of a right-hand side held in registers (row lane + 32 t in x[t]), for
// j = 32 tk + lk with tk known at compile time
template <typename T>
__device__ __forceinline__ T xget(const T (&x)[4], int tk, int lk) {
    return shfl(tk == 0 ? x[0] : tk == 1 ? x[1] : tk == 2 ? x[2] : x[3], lk);
}

// Barrier of the `nthreads` threads (whole warps) of one system's group.
__device__ __forceinline__ void group_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// One large system on the `gwarps` warps of its group (warp index gw, named
// barrier bar) in its shared-memory slot sized for nmax.
template <typename T>
__device__ __forceinline__ void large_system(const RaggedSys &s, int nmax, unsigned char *slot, int gw, int gwarps,
                                             int bar, const T *__restrict__ A_in, T *__restrict__ A,
                                             T *__restrict__ B, int *__restrict__ info, int refine, int lane) {
    const int RG_LARGE_WARPS = gwarps, warp = gw, nthr = 32 * gwarps;
    const int n = s.n, nrhs = s.nrhs, ld = cta_ld(n);
    const int ldmax = cta_ld(nmax);
    float *pbuf0 = reinterpret_cast<float *>(slot);  // panel row r at pbuf[8 r .. 8 r + 7]
    float *pbuf1 = pbuf0 + (size_t)nmax * 8;
    float *a = pbuf1 + (size_t)nmax * 8;
    float *dinv = a + (size_t)nmax * ldmax;
    int *s_fail = reinterpret_cast<int *>(dinv + nmax);
    const T *ag = A_in + s.a_off;

    for (int j = warp; j < n; j += RG_LARGE_WARPS)
        for (int i = j + lane; i < n; i += 32) a[j * ld + i] = (float)ag[(int64_t)j * n + i];
    if (gw == 0 && lane == 0) *s_fail = 0;
    group_sync(bar, nthr);
    // Blocked right-looking factorisation with look-ahead: while warps 1..W-1
    // apply panel p's rank-8 update to the columns past panel p + 1, warp 0
    // applies it to panel p + 1's columns and factors panel p + 1 (into the
    // other panel buffer).  Each element still receives its updates in
    // increasing k with one fma each, as in the column-by-column algorithm.
    // One barrier per panel.
    if (warp == 0) panel_factor(a, ld, n, 0, n < RG_PANEL ? n : RG_PANEL, pbuf0, dinv, s_fail, lane);
    group_sync(bar, nthr);
    for (int k0 = 0, p = 0; k0 < n; k0 += RG_PANEL, p++) {
        const int pw = n - k0 < RG_PANEL ? n - k0 : RG_PANEL;
        const int kn = k0 + pw, pwn = n - kn < RG_PANEL ? n - kn : RG_PANEL;  // next panel
        const float *pb = (p & 1) ? pbuf1 : pbuf0;
        float *pnext = (p & 1) ? pbuf0 : pbuf1;
        if (warp == 0) {
            if (pwn > 0) {
                panel_update(a, ld, n, pb, kn, kn + pwn, 0, 1, lane);
                __syncwarp();
                panel_factor(a, ld, n, kn, pwn, pnext, dinv, s_fail, lane);
            }
        } else {
            panel_update(a, ld, n, pb, kn + pwn, n, warp - 1, RG_LARGE_WARPS - 1, lane);
        }
        group_sync(bar, nthr);
    }
    if (gw == 0 && lane == 0 && info) info[s.orig] = *s_fail;

    T *bg = B + s.b_off;
    const int nt = (n + 31) >> 5;
    for (int c = warp; c < nrhs; c += RG_LARGE_WARPS) {
        const T *bc = bg + (int64_t)c * n;
        float w[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int i = lane + 32 * t;
            w[t] = i < n ? (float)bc[i] : 0.f;
        }
        reg_solve(a, ld, dinv, w, n, lane);
        T x[4];  // the solution, rows lane + 32 t, in the precision of the data
#pragma unroll
        for (int t = 0; t < 4; t++) x[t] = (T)w[t];
        for (int it = 0; it < refine; it++) {
            // r = b - A x with the full symmetric A; rows lane + 32 t; A's
            // columns four at a time, x_j by shuffle
            if constexpr (sizeof(T) == 4) {
                ff acc[4];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int i = lane + 32 * t;
                    acc[t].h = i < n ? (float)bc[i] : 0.f;
                    acc[t].l = 0.f;
                }
#pragma unroll
                for (int tk = 0; tk < 4; tk++) {
                    if (tk >= nt) break;
                    const int kmax = n - 32 * tk < 32 ? n - 32 * tk : 32;
                    int lk = 0;
                    for (; lk + 4 <= kmax; lk += 4) {
                        const int j = 32 * tk + lk;
                        float av[4][4];
#pragma unroll
                        for (int q = 0; q < 4; q++)
#pragma unroll
                            for (int t = 0; t < 4; t++) {
                                const int i = lane + 32 * t;
                                av[q][t] = (t < nt && i < n) ? (float)ag[(int64_t)(j + q) * n + i] : 0.f;
                            }
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const float xj = (float)xget(x, tk, lk + q);
#pragma unroll
                            for (int t = 0; t < 4; t++)
                                if (t < nt) ff_fma(acc[t], -av[q][t], xj, 0.f);
                        }
                    }
                    for (; lk < kmax; lk++) {
                        const int j = 32 * tk + lk;
                        const float xj = (float)xget(x, tk, lk);
#pragma unroll
                        for (int t = 0; t < 4; t++) {
                            const int i = lane + 32 * t;
                            if (t < nt && i < n) ff_fma(acc[t], -(float)ag[(int64_t)j * n + i], xj, 0.f);
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < 4; t++) w[t] = acc[t].h + acc[t].l;
            } else {
                double acc[4];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int i = lane + 32 * t;
                    acc[t] = i < n ? (double)bc[i] : 0.0;
                }
#pragma unroll
                for (int tk = 0; tk < 4; tk++) {
                    if (tk >= nt) break;
                    const int kmax = n - 32 * tk < 32 ? n - 32 * tk : 32;
                    int lk = 0;
                    for (; lk + 4 <= kmax; lk += 4) {
                        const int j = 32 * tk + lk;
                        double av[4][4];
#pragma unroll
                        for (int q = 0; q < 4; q++)
#pragma unroll
                            for (int t = 0; t < 4; t++) {
                                const int i = lane + 32 * t;
                                av[q][t] = (t < nt && i < n) ? (double)ag[(int64_t)(j + q) * n + i] : 0.0;
                            }
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const double xj = (double)xget(x, tk, lk + q);
#pragma unroll
                            for (int t = 0; t < 4; t++)
                                if (t < nt) acc[t] = fma(-av[q][t], xj, acc[t]);
                        }
                    }
                    for (; lk < kmax; lk++) {
                        const int j = 32 * tk + lk;
                        const double xj = (double)xget(x, tk, lk);
#pragma unroll
                        for (int t = 0; t < 4; t++) {
                            const int i = lane + 32 * t;
                            if (t < nt && i < n) acc[t] = fma(-(double)ag[(int64_t)j * n + i], xj, acc[t]);
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < 4; t++) w[t] = (float)acc[t];
            }
            reg_solve(a, ld, dinv, w, n, lane);
#pragma unroll
            for (int t = 0; t < 4; t++) x[t] = x[t] + (T)w[t];
        }
        T *bo = bg + (int64_t)c * n;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int i = lane + 32 * t;
            if (i < n) bo[i] = x[t];
        }
    }
    // L (lower triangle, FP32 factor) back in place, once every warp has
    // finished reading the original A for its residuals
    group_sync(bar, nthr);
    T *aw = A + s.a_off;
    for (int j = warp; j < n; j += RG_LARGE_WARPS)
        for (int i = j + lane; i < n; i += 32) aw[(int64_t)j * n + i] = (T)a[j * ld + i];
}

// ------------------------------------------------------------ persistent launch
// Blocks pull tasks from the queue head ctr[0] until it passes ntasks; the
// last block to finish (ctr[1]) resets both counters for the next call.  No
// block waits on another: a block that finds the queue empty simply leaves.
// 128 registers per thread up to 512 threads (the lane-row path keeps a
// 32-wide row and its refinement state in registers); 768 threads trade
// registers (80 a thread) for 24 warps per SM
template <typename T, int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS > 512 ? 1 : 512 / THREADS)
    k_ragged_persistent(const RaggedTask *__restrict__ tasks, int ntasks, const RaggedSys *__restrict__ sys,
                        int *__restrict__ ctr, T *__restrict__ A, T *__restrict__ B, int *__restrict__ info,
                        int refine) {
    extern __shared__ __align__(16) unsigned char rsm[];
    __shared__ int s_task;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (;;) {
        if (threadIdx.x == 0) s_task = atomicAdd(ctr, 1);
        __syncthreads();
        const int t = s_task;
        __syncthreads();  // every thread has read s_task before the next fetch
        if (t >= ntasks) break;
        const RaggedTask tk = tasks[t];
        if (tk.nb == 0) {
            // a launch captured before the plan's configuration changed may have
            // less shared memory than the new task table needs: flag, never overrun
            unsigned dyn;
            asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
            if ((size_t)tk.count * ragged_slot_bytes(tk.nmax) > dyn) {
                if (threadIdx.x < tk.count && info) info[sys[tk.first + threadIdx.x].orig] = -1;
                __syncthreads();
                continue;
            }
            const int grp = warp / tk.warps;  // system of the group this warp works on
            if (grp < tk.count)
                large_system<T>(sys[tk.first + grp], tk.nmax, rsm + (size_t)grp * ragged_slot_bytes(tk.nmax),
                                warp % tk.warps, tk.warps, 1 + grp, A, A, B, info, refine, lane);
        } else if (tk.nb == 8) {
            small_systems<T, 8>(sys, tk.first, tk.count, warp, lane, A, A, B, info, refine);
        } else if (tk.nb == 16) {
            small_systems<T, 16>(sys, tk.first, tk.count, warp, lane, A, A, B, info, refine);
        } else {
            small_systems<T, 32>(sys, tk.first, tk.count, warp, lane, A, A, B, info, refine);
        }
        __syncthreads();  // the slots are reused by the next task
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(ctr + 1, 1) == (int)gridDim.x - 1) {
            ctr[0] = 0;
            ctr[1] = 0;
            __threadfence();
        }
    }
}

static bool config_valid(const gbla_ragged_config &c) {
    const bool t = c.threads == 128 || c.threads == 256 || c.threads == 512 || c.threads == 768;
    const bool g = c.systems_per_block == 1 || c.systems_per_block == 2 || c.systems_per_block == 4 ||
                   c.systems_per_block == 8;
    return t && g && c.systems_per_block * 64 <= c.threads;  // at least two warps per system
}

constexpr size_t RG_SMEM_MAX = 226 * 1024;

// Cut the plan's systems into tasks for p->cfg (host), upload them (set-up
// time: synchronous copy) and size the block's shared memory.
static gbla_status ragged_build_tasks(gbla_ragged_plan *p, std::vector<RaggedTask> *out = nullptr) {
    std::vector<RaggedTask> t;
    const int W = p->cfg.threads / 32;
    const size_t top = p->num[3] > 0 ? ragged_slot_bytes(p->max_n_large) : 0;
    size_t cap = top * (size_t)p->cfg.systems_per_block;
    if (cap > RG_SMEM_MAX) cap = top > RG_SMEM_MAX ? top : (RG_SMEM_MAX / top) * top;
    for (int i = p->first[3]; i < p->count;) {
        const int nmax = p->large_n[i - p->first[3]];
        const size_t slot = ragged_slot_bytes(nmax);
        int cnt = (int)(cap / slot);
        cnt = cnt < p->cfg.systems_per_block ? cnt : p->cfg.systems_per_block;
        cnt = cnt < W / 2 ? cnt : W / 2;
        cnt = cnt < p->count - i ? cnt : p->count - i;
        if (cnt < 1) cnt = 1;
        t.push_back({i, cnt, 0, W / cnt, nmax, 0});
        i += cnt;
    }
    // small classes after the large ones, larger class first
    const int nbs[3] = {8, 16, 32};
    for (int c = 2; c >= 0; c--) {
        const int per = W * (32 / nbs[c]);
        for (int i = 0; i < p->num[c]; i += per)
            t.push_back({p->first[c] + i, p->num[c] - i < per ? p->num[c] - i : per, nbs[c], 1, 0, 0});
    }
    p->ntasks = (int)t.size();
    p->smem = cap;
    if (out) *out = t;
    if (t.empty()) return GBLA_SUCCESS;
    // a set-up step: no call of the plan may still be reading the old table
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return from_cuda(e);
    return from_cuda(cudaMemcpy(p->d_tasks, t.data(), sizeof(RaggedTask) * t.size(), cudaMemcpyHostToDevice));
}

template <typename T, int THREADS>
static gbla_status launch_persistent(const gbla_ragged_plan *p, T *A, T *B, int *info, int refine, cudaStream_t st) {
    auto kern = k_ragged_persistent<T, THREADS>;
    if (p->smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem);
        if (e != cudaSuccess) return from_cuda(e);
    }
    const int64_t grid = persistent_grid(reinterpret_cast<const void *>(kern), THREADS, p->smem, p->ntasks);
    kern<<<(unsigned)grid, THREADS, p->smem, st>>>(p->d_tasks, p->ntasks, p->d_sys, p->d_ctr, A, B, info, refine);
    return launch_status();
}

template <typename T>
static gbla_status ragged_launch(const gbla_ragged_plan *p, T *A, T *B, int *info, int refine, cudaStream_t st) {
    if (!p || refine < 0) return GBLA_INVALID_VALUE;
    if (p->count == 0) return GBLA_SUCCESS;
    if (!A || !B) return GBLA_INVALID_VALUE;
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != p->device) return GBLA_INVALID_VALUE;
    if (p->cfg.threads == 128) return launch_persistent<T, 128>(p, A, B, info, refine, st);
    if (p->cfg.threads == 512) return launch_persistent<T, 512>(p, A, B, info, refine, st);
    if (p->cfg.threads == 768) return launch_persistent<T, 768>(p, A, B, info, refine, st);
    return launch_persistent<T, 256>(p, A, B, info, refine, st);
}

// Time every candidate configuration on the caller's batch.  A and B are
// copied to scratch arenas; every trial runs on fresh copies and the
// caller's arrays are left as they were.
template <typename T>
static gbla_status ragged_autotune(gbla_ragged_plan *p, const T *A, const T *B, int refine, int reps,
                                   gbla_ragged_config *best_out, float *best_ms, cudaStream_t st) {
    if (!p || refine < 0 || reps < 1) return GBLA_INVALID_VALUE;
    if (p->count == 0) {
        if (best_out) *best_out = p->cfg;
        if (best_ms) *best_ms = 0.f;
        return GBLA_SUCCESS;
    }
    if (!A || !B) return GBLA_INVALID_VALUE;
    T *sa = nullptr, *sb = nullptr, *wa = nullptr, *wb = nullptr;
    int *sinfo = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const size_t abytes = sizeof(T) * (size_t)(p->a_extent > 0 ? p->a_extent : 1);
    const size_t bbytes = sizeof(T) * (size_t)(p->b_extent > 0 ? p->b_extent : 1);
    cudaError_t e = cudaMalloc(&sa, abytes);
    if (e == cudaSuccess) e = cudaMalloc(&sb, bbytes);
    if (e == cudaSuccess) e = cudaMalloc(&wa, abytes);
    if (e == cudaSuccess) e = cudaMalloc(&wb, bbytes);
    if (e == cudaSuccess) e = cudaMalloc(&sinfo, sizeof(int) * (size_t)p->count);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sa, A, abytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sb, B, bbytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    gbla_status status = from_cuda(e);
    const gbla_ragged_config saved = p->cfg;
    gbla_ragged_config best = saved;
    float best_t = 3.4e38f;
    const int threads[4] = {128, 256, 512, 768}, groups[4] = {1, 2, 4, 8};
    for (int ti = 0; ti < 4 && status == GBLA_SUCCESS; ti++)
        for (int gi = 0; gi < 4 && status == GBLA_SUCCESS; gi++) {
            const gbla_ragged_config c = {threads[ti], groups[gi]};
            if (!config_valid(c)) continue;
            p->cfg = c;
            status = ragged_build_tasks(p);
            float t_min = 3.4e38f;
            for (int r = 0; r <= reps && status == GBLA_SUCCESS; r++) {  // r = 0: warm-up
                e = cudaMemcpyAsync(wa, sa, abytes, cudaMemcpyDeviceToDevice, st);
                if (e == cudaSuccess) e = cudaMemcpyAsync(wb, sb, bbytes, cudaMemcpyDeviceToDevice, st);
                if (e == cudaSuccess) e = cudaEventRecord(e0, st);
                if (e != cudaSuccess) { status = from_cuda(e); break; }
                status = ragged_launch<T>(p, wa, wb, sinfo, refine, st);
                if (status != GBLA_SUCCESS) break;
                e = cudaEventRecord(e1, st);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess) { status = from_cuda(e); break; }
                if (r > 0 && ms < t_min) t_min = ms;
            }
            if (status == GBLA_SUCCESS && t_min < best_t) {
                best_t = t_min;
                best = c;
            }
        }
    p->cfg = status == GBLA_SUCCESS ? best : saved;
    gbla_status s2 = ragged_build_tasks(p);
    if (status == GBLA_SUCCESS) status = s2;
    cudaStreamSynchronize(st);
    if (sa) cudaFree(sa);
    if (sb) cudaFree(sb);
    if (wa) cudaFree(wa);
    if (wb) cudaFree(wb);
    if (sinfo) cudaFree(sinfo);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (status == GBLA_SUCCESS) {
        if (best_out) *best_out = best;
        if (best_ms) *best_ms = best_t;
    }
    return status;
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_ragged_plan_create(const int64_t *a_offsets, const int64_t *b_offsets, const int *n,
                                             const int *nrhs, int count, gbla_ragged_plan **plan) {
    if (!plan || count < 0) return GBLA_INVALID_VALUE;
    *plan = nullptr;
    if (count > 0 && (!a_offsets || !b_offsets || !n || !nrhs)) return GBLA_INVALID_VALUE;
    std::vector<RaggedSys> v((size_t)count);
    for (int i = 0; i < count; i++) {
        if (n[i] < 1 || n[i] > 128 || nrhs[i] < 0 || a_offsets[i] < 0 || b_offsets[i] < 0) return GBLA_INVALID_VALUE;
        v[i] = {a_offsets[i], b_offsets[i], n[i], nrhs[i], i, 0};
    }
    auto cls = [](int nn) { return nn <= 8 ? 0 : nn <= 16 ? 1 : nn <= 32 ? 2 : 3; };
    // class, then largest first (LPT), then most right-hand sides, then input order
    std::stable_sort(v.begin(), v.end(), [&](const RaggedSys &x, const RaggedSys &y) {
        int cx = cls(x.n), cy = cls(y.n);
        if (cx != cy) return cx < cy;
        if (x.n != y.n) return x.n > y.n;
        return x.nrhs > y.nrhs;
    });
    auto *p = new (std::nothrow) gbla_ragged_plan();
    if (!p) return GBLA_CUDA_ERROR;
    p->count = count;
    for (int i = 0; i < count; i++) {
        p->num[cls(v[i].n)]++;
        p->a_extent = std::max(p->a_extent, v[i].a_off + (int64_t)v[i].n * v[i].n);
        p->b_extent = std::max(p->b_extent, v[i].b_off + (int64_t)v[i].n * v[i].nrhs);
    }
    p->first[0] = 0;
    for (int c = 1; c < 4; c++) p->first[c] = p->first[c - 1] + p->num[c - 1];
    p->max_n_large = p->num[3] > 0 ? v[p->first[3]].n : 0;
    for (int i = p->first[3]; i < count; i++) p->large_n.push_back(v[i].n);
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess && count > 0) e = cudaMalloc(&p->d_sys, sizeof(RaggedSys) * (size_t)count);
    if (e == cudaSuccess && count > 0)
        e = cudaMemcpy(p->d_sys, v.data(), sizeof(RaggedSys) * (size_t)count, cudaMemcpyHostToDevice);
    // at most one task per system
    if (e == cudaSuccess && count > 0) e = cudaMalloc(&p->d_tasks, sizeof(RaggedTask) * (size_t)count);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_ctr, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->d_ctr, 0, 2 * sizeof(int));
    gbla_status s = from_cuda(e);
    if (s == GBLA_SUCCESS && count > 0) s = ragged_build_tasks(p);
    if (s != GBLA_SUCCESS) {
        gbla_ragged_plan_destroy(p);
        return s;
    }
    *plan = p;
    return GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_ragged_plan_destroy(gbla_ragged_plan *p) {
    if (!p) return GBLA_SUCCESS;
    cudaError_t e = cudaSuccess;
    if (p->d_sys) e = cudaFree(p->d_sys);
    if (p->d_tasks) {
        cudaError_t e2 = cudaFree(p->d_tasks);
        if (e == cudaSuccess) e = e2;
    }
    if (p->d_ctr) {
        cudaError_t e2 = cudaFree(p->d_ctr);
        if (e == cudaSuccess) e = e2;
    }
    delete p;
    return from_cuda(e);
}

GBLA_API gbla_status gbla_ragged_plan_get_config(const gbla_ragged_plan *p, gbla_ragged_config *cfg) {
    if (!p || !cfg) return GBLA_INVALID_VALUE;
    *cfg = p->cfg;
    return GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_ragged_plan_set_config(gbla_ragged_plan *p, const gbla_ragged_config *cfg) {
    if (!p || !cfg || !config_valid(*cfg)) return GBLA_INVALID_VALUE;
    p->cfg = *cfg;
    return p->count > 0 ? ragged_build_tasks(p) : GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_ragged_plan_tasks(const gbla_ragged_plan *p, int *ntasks, size_t *smem_bytes) {
    if (!p) return GBLA_INVALID_VALUE;
    if (ntasks) *ntasks = p->ntasks;
    if (smem_bytes) *smem_bytes = p->smem;
    return GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_sragged_autotune(gbla_ragged_plan *p, const float *A, const float *B, int refine_iters,
                                           int reps, gbla_ragged_config *best, float *best_ms, cudaStream_t st) {
    return ragged_autotune<float>(p, A, B, refine_iters, reps, best, best_ms, st);
}

GBLA_API gbla_status gbla_dragged_autotune(gbla_ragged_plan *p, const double *A, const double *B, int refine_iters,
                                           int reps, gbla_ragged_config *best, float *best_ms, cudaStream_t st) {
    return ragged_autotune<double>(p, A, B, refine_iters, reps, best, best_ms, st);
}

GBLA_API gbla_status gbla_sposv_ragged(const gbla_ragged_plan *plan, float *A, float *B, int *info, int refine_iters,
                                       cudaStream_t st) {
    return ragged_launch<float>(plan, A, B, info, refine_iters, st);
}

GBLA_API gbla_status gbla_dposv_ragged(const gbla_ragged_plan *plan, double *A, double *B, int *info,
                                       int refine_iters, cudaStream_t st) {
    return ragged_launch<double>(plan, A, B, info, refine_iters, st);
}
