// qr_common.cuh -- batched Householder QR, Q^T / Q application,
// upper-triangular solve, and least squares with extended-precision
// iterative refinement: the device code and launchers shared by qr.cu (FP32
// warp kernels, the two-kernel least squares), qr_f64.cu (FP64) and gels.cu
// (the fused FP32 least-squares kernel).  Each kernel instantiation is used
// by one translation unit only.
//
// Warp kernels (k_qr_warp, k_ormqr_warp): one warp per matrix (m <= 128,
// n <= 32).  Lane l owns rows
// l + 32 t (t < R = ceil(m/32)) of A in registers; the Householder vector of
// step k lives in column k below the diagonal (LAPACK dgeqr2/dlarfg
// convention: beta = -sign(alpha) ||x||, tau = (beta - alpha) / beta).  The
// 32 column dot products of one step are reduced with a butterfly
// reduce-scatter (31 shuffles for all columns) and broadcast back.
//
// Least squares refinement (augmented system of Bjorck): with x and the
// residual r carried as FP32 pairs (hi + lo), each step computes
//   f = b - r - A x,   g = -A^T r
// with error-free products and compensated sums (double-FP32 arithmetic,
// about 48 significant bits; the device's FP64 rate is ~1/74 of FP32), then
// solves the correction with the FP32 factors:
//   h = R^-T g,  d = Q^T f,  dx = R^-1 (d_1 - h),  dr = Q [h; d_2].
// The original A is kept in shared memory for the residuals.
#pragma once
#include "common.cuh"
#include "qr_big.cuh"
#include "xprec.cuh"

namespace gbla {

// ------------------------------------------------------------ butterfly
// On entry p[j] is this lane's partial for slot j (32 slots); on exit the
// return value is the warp-wide total of slot `lane`.
template <typename T>
__device__ __forceinline__ T reduce_scatter32(T (&p)[32], int lane) {
    T q[16];
    const bool b4 = lane & 16;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        T mine = b4 ? p[i + 16] : p[i];
        T other = b4 ? p[i] : p[i + 16];
        q[i] = mine + shfl_xor(other, 16);
    }
    const bool b3 = lane & 8;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        T mine = b3 ? q[i + 8] : q[i];
        T other = b3 ? q[i] : q[i + 8];
        q[i] = mine + shfl_xor(other, 8);
    }
    const bool b2 = lane & 4;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        T mine = b2 ? q[i + 4] : q[i];
        T other = b2 ? q[i] : q[i + 4];
        q[i] = mine + shfl_xor(other, 4);
    }
    const bool b1 = lane & 2;
#pragma unroll
    for (int i = 0; i < 2; i++) {
        T mine = b1 ? q[i + 2] : q[i];
        T other = b1 ? q[i] : q[i + 2];
        q[i] = mine + shfl_xor(other, 2);
    }
    const bool b0 = lane & 1;
    T mine = b0 ? q[1] : q[0];
    T other = b0 ? q[0] : q[1];
    return mine + shfl_xor(other, 1);
}

// Householder coefficients of a column with leading entry alpha and squared
// norm x2 > 0 below it (LAPACK dlarfg convention): beta = -sign(alpha)
// sqrt(alpha^2 + x2), tau = (beta - alpha) / beta, scal = 1 / (alpha - beta).
// FP32: from one Newton-refined reciprocal square root y = 1 / sqrt(alpha^2 +
// x2) (about 1 ulp) -- beta = -sign(alpha) s y, tau = 1 + |alpha| y, scal =
// sign(alpha) / (|alpha| + s y) -- a shorter dependency chain than a square
// root and two divisions on the critical path of every step.  FP64: as LAPACK.
template <typename T>
__device__ __forceinline__ void house_coeffs(T alpha, T x2, T &beta, T &tau, T &scal) {
    if constexpr (sizeof(T) == 4) {
        const float s2 = fmaf(alpha, alpha, x2);
        float y = rsqrtf(s2);
        y = y * fmaf(-0.5f * s2 * y, y, 1.5f);
        const float r = s2 * y;  // sqrt(alpha^2 + x2)
        beta = -copysignf(r, alpha);
        tau = fmaf(fabsf(alpha), y, 1.0f);
        scal = copysignf(__fdividef(1.0f, fabsf(alpha) + r), alpha);
    } else {
        beta = -copysign(dev_sqrt<T>(fma(alpha, alpha, x2)), alpha);
        tau = (beta - alpha) / beta;
        scal = T(1) / (alpha - beta);
    }
}

// --------------------------------------------------------- warp QR core
template <typename T, int R>
struct QrWarp {
    T a[R][32];  // rows lane + 32 t, columns 0..31
    T dinv;      // 1 / R_ll in lane l < n (set by factor)
    int lane;

    __device__ __forceinline__ int row(int t) const { return lane + 32 * t; }

    // Householder QR in registers; tau written to tau_s[k] (shared, per warp).
    __device__ __forceinline__ int factor(int m, int n, T *tau_s) {
        int rank_fail = 0;
        T rdiag = T(0);  // R_ll of this lane (warp-uniform value of step l)
#pragma unroll
        for (int k = 0; k < 32; k++) {
            if (k < n) {
                T x2 = T(0);
#pragma unroll
                for (int t = 0; t < R; t++)
                    if (row(t) > k && row(t) < m) x2 = fma(a[t][k], a[t][k], x2);
                x2 = warp_sum(x2);
                const T alpha = shfl(a[0][k], k);
                T tau = T(0);
                if (lane == k) rdiag = alpha;
                if (x2 > T(0)) {
                    T beta, scal;
                    house_coeffs<T>(alpha, x2, beta, tau, scal);
                    if (lane == k) rdiag = beta;
#pragma unroll
                    for (int t = 0; t < R; t++)
                        if (row(t) > k) a[t][k] *= scal;
                    if (lane == k) a[0][k] = beta;
                    // w_j = v^T a_j for all slots, then a_j -= tau w_j v
                    T p[32];
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        T s = T(0);
                        if (j > k) {
#pragma unroll
                            for (int t = 0; t < R; t++) {
                                T v = row(t) > k ? a[t][k] : (row(t) == k ? T(1) : T(0));
                                s = fma(v, a[t][j], s);
                            }
                        }
                        p[j] = s;
                    }
                    T w = reduce_scatter32(p, lane);
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        if (j > k && j < n) {
                            T twj = tau * shfl(w, j);
#pragma unroll
                            for (int t = 0; t < R; t++) {
                                T v = row(t) > k ? a[t][k] : (row(t) == k ? T(1) : T(0));
                                a[t][j] = fma(-twj, v, a[t][j]);
                            }
                        }
                    }
                }
                if (lane == 0) tau_s[k] = tau;
                if (shfl(a[0][k], k) == T(0) && rank_fail == 0) rank_fail = k + 1;
            }
        }
        // reciprocal of this lane's diagonal entry, once for every triangular solve
        dinv = (lane < n && rdiag != T(0)) ? T(1) / rdiag : T(0);
        __syncwarp();
        return rank_fail;
    }

    // y <- H_k y for one column held as y[t] (rows lane + 32 t)
    __device__ __forceinline__ void apply_h(int k, T tau, T (&y)[R]) const {
        T s = T(0);
#pragma unroll
        for (int t = 0; t < R; t++) {
            T v = row(t) > k ? a[t][k] : (row(t) == k ? T(1) : T(0));
            s = fma(v, y[t], s);
        }
        s = tau * warp_sum(s);
#pragma unroll
        for (int t = 0; t < R; t++) {
            T v = row(t) > k ? a[t][k] : (row(t) == k ? T(1) : T(0));
            y[t] = fma(-s, v, y[t]);
        }
    }

    __device__ __forceinline__ void apply_qt(int n, const T *tau_s, T (&y)[R]) const {
#pragma unroll
        for (int k = 0; k < 32; k++)
            if (k < n) apply_h(k, tau_s[k], y);
    }

    __device__ __forceinline__ void apply_q(int n, const T *tau_s, T (&y)[R]) const {
#pragma unroll
        for (int k = 31; k >= 0; k--)
            if (k < n) apply_h(k, tau_s[k], y);
    }

    // Solve R z = y (y in lane j for j < n); returns z in lane j.
    __device__ __forceinline__ T back_solve(int n, T y) const {
        T z = T(0);
#pragma unroll
        for (int j = 31; j >= 0; j--) {
            if (j < n) {
                T zj = shfl(y * dinv, j);  // lane j holds y_j and 1 / R_jj
                if (lane == j) z = zj;
                if (lane < j) y = fma(-a[0][j], zj, y);
            }
        }
        return z;
    }

    // Solve R^T h = g (g in lane j); returns h in lane j.
    __device__ __forceinline__ T forward_solve_rt(int n, T g) const {
        T h = T(0);
#pragma unroll
        for (int j = 0; j < 32; j++) {
            if (j < n) {
                T part = lane < j ? a[0][j] * h : T(0);  // R_ij h_i, i < j
                T s = warp_sum(part);
                T hj = shfl((g - s) * dinv, j);
                if (lane == j) h = hj;
            }
        }
        return h;
    }
};

// Augmented-system refinement of one right-hand side (FP32 data, double-FP32
// residuals).  A0: the original matrix, column stride lda, rows [m, 32 R)
// zero (every caller stages it zero-padded in shared memory); x0: FP32
// solution in lane j; returns the refined x in lane j.
template <int R, class QF>
__device__ __forceinline__ float refine_ls(const QF &q, const float *A0, int lda, int m, int n,
                                           const float (&b)[R], float x0, const float *tau_s, int refine) {
    const int lane = q.lane;
    float xh = x0, xl = 0.f;
    float rh[R], rl[R];
#pragma unroll
    for (int t = 0; t < R; t++) { rh[t] = 0.f; rl[t] = 0.f; }
    for (int it = 0; it <= refine; it++) {
        // f = b - r - A x (rows).  At it == 1, r is the residual of x adopted
        // at it == 0 and x has not moved, so f vanishes to ~2^-48: skip it
        // (and d = Q^T f with it).
        const bool fzero = it == 1;
        ff f[R];
#pragma unroll
        for (int t = 0; t < R; t++) {
            f[t].h = fzero ? 0.f : b[t];
            f[t].l = 0.f;
            if (!fzero) ff_add(f[t], -rh[t], -rl[t]);
        }
        if (!fzero) {
            for (int j = 0; j < n; j++) {
                float xjh = shfl(xh, j), xjl = shfl(xl, j);
#pragma unroll
                for (int t = 0; t < R; t++) {
                    int r = lane + 32 * t;
                    const float aij = A0[j * lda + r];
                    ff_fma(f[t], -aij, xjh, xjl);
                }
            }
        }
        if (it == 0) {
            // first pass: adopt the accurate residual of the FP32 solution as r
#pragma unroll
            for (int t = 0; t < R; t++) {
                ff fn = ff_norm(f[t]);
                rh[t] = fn.h; rl[t] = fn.l;
            }
            continue;
        }
        // g = -A^T r (lane j keeps column j); eight columns per reduce-scatter
        float gj = 0.f;
        for (int j0 = 0; j0 < n; j0 += 8) {
            ff acc[8];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                acc[c].h = 0.f;
                acc[c].l = 0.f;
                if (j0 + c < n) {
#pragma unroll
                    for (int t = 0; t < R; t++) {
                        int r = lane + 32 * t;
                        const float aij = A0[(j0 + c) * lda + r];
                        ff_fma(acc[c], aij, rh[t], rl[t]);
                    }
                }
            }
            const ff tot = ff_reduce_scatter8(acc, lane);
            const float gs = shfl(tot.h + tot.l, 4 * (lane & 7));
            if ((lane >> 3) == (j0 >> 3)) gj = -gs;
        }
        float h = q.forward_solve_rt(n, gj);
        float fr[R];
#pragma unroll
        for (int t = 0; t < R; t++) fr[t] = fzero ? 0.f : f[t].h + f[t].l;
        if (!fzero) q.apply_qt(n, tau_s, fr);           // d = Q^T f
        float dx = q.back_solve(n, lane < n ? fr[0] - h : 0.f);
        if (it < refine) {
            // dr = Q [h; d2], needed only by a further step
            float z[R];
#pragma unroll
            for (int t = 0; t < R; t++) z[t] = (lane + 32 * t) < n ? h : fr[t];
            q.apply_q(n, tau_s, z);
#pragma unroll
            for (int t = 0; t < R; t++) {
                float s, e;
                two_sum(rh[t], z[t], s, e);
                float l = rl[t] + e;
                rh[t] = s + l; rl[t] = l - (rh[t] - s);
            }
        }
        {
            float s, e;
            two_sum(xh, dx, s, e);
            float l = xl + e;
            xh = s + l; xl = l - (xh - s);
        }
    }
    return xh + xl;
}

// SOLVE = false: factorisation only (the solve of gbla_sgels_batched_ws runs
// in k_ls_solve); F (nullable) receives the factors instead of A.
template <typename T, int R, bool SOLVE = true>
__global__ void __launch_bounds__(128, (SOLVE || sizeof(T) == 8) ? 1 : 3)
    k_qr_warp(int m, int n, int nrhs, T *__restrict__ A, int64_t sA, T *__restrict__ B, int64_t sB,
              T *__restrict__ tau_g, int64_t sTau, int *__restrict__ info, int flags, int batch,
              T *__restrict__ F = nullptr, int64_t sF = 0) {
    __shared__ T tau_all[4 * 32];  // 32 taus per warp
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T *tau_s = tau_all + 32 * warp;
    const int64_t mat = (int64_t)blockIdx.x * 4 + warp;
    if (mat >= batch) return;  // whole warp leaves together; no block barriers below
    QrWarp<T, R> q;
    q.lane = lane;
    T *a_g = A + mat * sA;
#pragma unroll
    for (int j = 0; j < 32; j++)
#pragma unroll
        for (int t = 0; t < R; t++) {
            int r = lane + 32 * t;
            T v = (j < n && r < m) ? a_g[(int64_t)j * m + r] : T(0);
            q.a[t][j] = v;
        }
    int fail = q.factor(m, n, tau_s);
    if (info && lane == 0) info[mat] = fail;

    if (SOLVE && (flags & QR_SOLVE) && nrhs > 0) {
        T *b_g = B + mat * sB;
        for (int c = 0; c < nrhs; c++) {
            T y[R];
#pragma unroll
            for (int t = 0; t < R; t++) {
                int r = lane + 32 * t;
                y[t] = r < m ? b_g[(int64_t)c * m + r] : T(0);
            }
            q.apply_qt(n, tau_s, y);
            const T x = q.back_solve(n, lane < n ? y[0] : T(0));
            // rows < n: solution (row r = this lane when t = 0, since n <= 32);
            // rows >= n: (Q^T b)(n:m), as gels leaves them
#pragma unroll
            for (int t = 0; t < R; t++) {
                int r = lane + 32 * t;
                if (r < m) b_g[(int64_t)c * m + r] = r < n ? x : y[t];
            }
        }
    }
    if (flags & QR_WRITE_FACTORS) {
        T *f_g = F ? F + mat * sF : a_g;
#pragma unroll
        for (int j = 0; j < 32; j++)
#pragma unroll
            for (int t = 0; t < R; t++) {
                int r = lane + 32 * t;
                if (j < n && r < m) f_g[(int64_t)j * m + r] = q.a[t][j];
            }
    }
    if ((flags & QR_WRITE_TAU) && tau_g && lane < n) tau_g[mat * sTau + lane] = tau_s[lane];
}

// ------------------------------------------ solve from stored factors
// The QrWarp interface over factors held in shared memory, column-major with
// column stride LDQ = 32 R + 1: a column (lanes on consecutive rows) and a
// row of R (lane l reading R(j, l)) are both free of bank conflicts.  The
// reflector applications and the back substitution follow QrWarp operation
// for operation; the substitution with R^T runs column by column (a row of R
// per step) instead of with one warp reduction per step.
template <int R>
struct QrSmem {
    static constexpr int LDQ = 32 * R + 1;
    const float *Q;  // Q[j * LDQ + i] = factor element (i, j)
    float dinv;
    int lane;

    __device__ __forceinline__ int row(int t) const { return lane + 32 * t; }
    __device__ __forceinline__ float at(int t, int k) const { return Q[k * LDQ + row(t)]; }
    __device__ __forceinline__ float rt(int j) const { return Q[lane * LDQ + j]; }  // R(j, lane)

    // Reflector k < 32: rows 32 t (t >= 1) are all below the diagonal.
    __device__ __forceinline__ float vk(int t, int k) const {
        return t > 0 ? at(t, k) : (lane > k ? at(0, k) : (lane == k ? 1.f : 0.f));
    }
    __device__ __forceinline__ void apply_h(int k, float tau, float (&y)[R]) const {
        float v[R];
        float s = 0.f;
#pragma unroll
        for (int t = 0; t < R; t++) {
            v[t] = vk(t, k);
            s = fmaf(v[t], y[t], s);
        }
        s = tau * warp_sum(s);
#pragma unroll
        for (int t = 0; t < R; t++) y[t] = fmaf(-s, v[t], y[t]);
    }
    __device__ __forceinline__ void apply_qt(int n, const float *tau_s, float (&y)[R]) const {
        for (int k = 0; k < n; k++) apply_h(k, tau_s[k], y);
    }
    __device__ __forceinline__ void apply_q(int n, const float *tau_s, float (&y)[R]) const {
        for (int k = n - 1; k >= 0; k--) apply_h(k, tau_s[k], y);
    }
    __device__ __forceinline__ float back_solve(int n, float y) const {
        float z = 0.f;
        for (int j = n - 1; j >= 0; j--) {
            float zj = shfl(y * dinv, j);
            if (lane == j) z = zj;
            if (lane < j) y = fmaf(-at(0, j), zj, y);
        }
        return z;
    }
    // Solve R^T h = g (g in lane j); returns h in lane j.  After h_j is known
    // every later row l subtracts R(j, l) h_j from its g_l.
    __device__ __forceinline__ float forward_solve_rt(int n, float g) const {
        float h = 0.f;
        const bool live = lane < n;
        for (int j = 0; j < n; j++) {
            const float hj = shfl(g * dinv, j);
            if (lane == j) h = hj;
            if (live && lane > j) g = fmaf(-rt(j), hj, g);
        }
        return h;
    }
};

// 4-byte asynchronous global -> shared copy (zero-filled when `valid` is false;
// the source address is then not read).
__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Solve phase shared by k_ls_solve and k_gels_cta: factors (Q, column-major,
// column stride 32 R + 1), taus and the original A (A0, refinement only,
// column stride 32 R, zero-padded rows) are in shared memory; one warp per right-hand side solves in FP32 and refines with
// double-FP32 residuals, then the block copies the factors into A.
template <int R>
__device__ __forceinline__ void ls_solve_block(int m, int n, int nrhs, const float *Q, const float *A0,
                                               const float *taus, float *a_g, float *b_g, int refine, int warp,
                                               int lane) {
    constexpr int LDM = 32 * R, LDQ = QrSmem<R>::LDQ;
    QrSmem<R> q;
    q.Q = Q;
    q.lane = lane;
    {
        const float d = lane < n ? Q[lane * LDQ + lane] : 0.f;
        q.dinv = (lane < n && d != 0.f) ? 1.f / d : 0.f;
    }
    for (int c = warp; c < nrhs; c += 4) {
        float y[R], b[R];
#pragma unroll
        for (int t = 0; t < R; t++) {
            int r = lane + 32 * t;
            b[t] = r < m ? b_g[(int64_t)c * m + r] : 0.f;
            y[t] = b[t];
        }
        q.apply_qt(n, taus, y);
        float x = q.back_solve(n, lane < n ? y[0] : 0.f);
        if (refine > 0) x = refine_ls<R>(q, A0, LDM, m, n, b, x, taus, refine);
#pragma unroll
        for (int t = 0; t < R; t++) {
            int r = lane + 32 * t;
            if (r < m) b_g[(int64_t)c * m + r] = r < n ? x : y[t];
        }
    }
    // the factors into A (the original A is no longer read from global memory)
    for (int j = warp; j < n; j += 4) {
#pragma unroll
        for (int t = 0; t < R; t++) {
            const int i = lane + 32 * t;
            if (i < m) a_g[(int64_t)j * m + i] = Q[j * LDQ + i];
        }
    }
}

// One block of 4 warps per least-squares system: the factors and taus (from
// the workspace) and the original A (still in A) are staged in shared memory
// with asynchronous copies, all in flight at once, then ls_solve_block.
template <int R>
__global__ void __launch_bounds__(128)
    k_ls_solve(int m, int n, int nrhs, float *__restrict__ A, int64_t sA, const float *__restrict__ F,
               const float *__restrict__ tau_g, float *__restrict__ B, int64_t sB, int refine, int batch) {
    extern __shared__ __align__(16) float lsm[];
    constexpr int LDM = 32 * R, LDQ = QrSmem<R>::LDQ;
    float *Q = lsm;                // n columns x LDQ: factors
    float *A0 = Q + 32 * LDQ;      // n columns x LDM: original matrix (refinement only)
    float *taus = A0 + (refine > 0 ? 32 * LDM : 0);  // 32
    const int64_t mat = blockIdx.x;
    if (mat >= batch) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float *f = F + mat * (int64_t)m * n;
    float *a_g = A + mat * sA;
    for (int j = warp; j < n; j += 4) {
#pragma unroll
        for (int t = 0; t < R; t++) {
            const int i = lane + 32 * t;
            const bool ok = i < m;
            cp_async4(Q + j * LDQ + i, f + (ok ? (int64_t)j * m + i : 0), ok);
            if (refine > 0) cp_async4(A0 + j * LDM + i, a_g + (ok ? (int64_t)j * m + i : 0), ok);
        }
    }
    if (tid < 32) taus[tid] = tid < n ? tau_g[mat * 32 + tid] : 0.f;
    cp_async_wait_all();
    __syncthreads();
    ls_solve_block<R>(m, n, nrhs, Q, A0, taus, a_g, B + mat * sB, refine, warp, lane);
}

// Total over the warp of 8 slots, reduce-scattered: on return lanes
// 4 s .. 4 s + 3 hold the total of slot s.  The additions pair lanes in the
// same order as reduce_scatter32 (bit 4 first), so a slot's total is the
// same value either function computes.
__device__ __forceinline__ float reduce_scatter8(const float (&p)[8], int lane) {
    float q[4];
    const bool b4 = lane & 16;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float mine = b4 ? p[i + 4] : p[i], other = b4 ? p[i] : p[i + 4];
        q[i] = mine + shfl_xor(other, 16);
    }
    const bool b3 = lane & 8;
    float r[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const float mine = b3 ? q[i + 2] : q[i], other = b3 ? q[i] : q[i + 2];
        r[i] = mine + shfl_xor(other, 8);
    }
    const bool b2 = lane & 4;
    float s = (b2 ? r[1] : r[0]) + shfl_xor(b2 ? r[0] : r[1], 4);
    s += shfl_xor(s, 2);
    s += shfl_xor(s, 1);
    return s;
}

// Least squares, one block of 4 warps per system, everything on chip.
// Factorisation: warp w holds columns w, w + 4, ..., w + 28 (rows lane + 32 t
// in registers, 8 R values per lane).  At step k the owner of column k
// (warp k mod 4) forms the Householder vector exactly as QrWarp::factor does
// and publishes it (explicit unit diagonal, double-buffered) in shared
// memory; after one block barrier every warp applies the reflector to its
// columns j > k.  The per-lane partial dot products and the reduction tree
// are those of QrWarp::factor, so factors and info are bit-identical to
// k_qr_warp's, and the solutions to the two-kernel schedule's (both solve
// through QrSmem).  Then the factors go to shared memory and ls_solve_block
// solves one right-hand side per warp.
template <int R>
__global__ void __launch_bounds__(128)
    k_gels_cta(int m, int n, int nrhs, float *__restrict__ A, int64_t sA, float *__restrict__ B, int64_t sB,
               int *__restrict__ info, int refine, int batch) {
    extern __shared__ __align__(16) float gsm[];
    constexpr int LDM = 32 * R, LDQ = QrSmem<R>::LDQ;
    float *Q = gsm;                           // 32 columns x LDQ: factors
    float *vbuf = Q + 32 * LDQ;               // 2 x LDM: Householder vector of the step (double-buffered)
    float *taus = vbuf + 2 * LDM;             // 32
    float *A0 = taus + 32;                    // 32 columns x LDM: original matrix (refinement only)
    const int64_t mat = blockIdx.x;
    if (mat >= batch) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float *a_g = A + mat * sA;
    float a[R][8];  // column warp + 4 c, rows lane + 32 t
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const int j = warp + 4 * c;
#pragma unroll
        for (int t = 0; t < R; t++) {
            const int r = lane + 32 * t;
            const float v = (j < n && r < m) ? a_g[(int64_t)j * m + r] : 0.f;
            a[t][c] = v;
            if (refine > 0) A0[j * LDM + r] = v;
        }
    }
    // Steps k = 4 kb + kk: the pivot column is slot kb of warp kk, so with kb
    // unrolled every register index is a compile-time constant and a warp
    // visits only its slots c >= kb (slot kb only while its column is > k).
#pragma unroll
    for (int kb = 0; kb < 8; kb++) {
        for (int kk = 0; kk < 4; kk++) {
            const int k = 4 * kb + kk;
            if (k >= n) break;
            float *vb = vbuf + (k & 1) * LDM;
            if (warp == kk) {
                float x2 = 0.f;
#pragma unroll
                for (int t = 0; t < R; t++) {
                    const int r = lane + 32 * t;
                    if (r > k && r < m) x2 = fmaf(a[t][kb], a[t][kb], x2);
                }
                x2 = warp_sum(x2);
                const float alpha = shfl(a[0][kb], k);
                float tau = 0.f;
                if (x2 > 0.f) {
                    float beta, scal;
                    house_coeffs<float>(alpha, x2, beta, tau, scal);
#pragma unroll
                    for (int t = 0; t < R; t++)
                        if (lane + 32 * t > k) a[t][kb] *= scal;
                    if (lane == k) a[0][kb] = beta;
                }
#pragma unroll
                for (int t = 0; t < R; t++) {
                    const int r = lane + 32 * t;
                    vb[r] = r > k ? a[t][kb] : (r == k ? 1.f : 0.f);
                }
                // tau != 0 exactly when x2 > 0 (then tau = 1 - alpha / beta is in [1, 2])
                if (lane == 0) taus[k] = tau;
            }
            __syncthreads();
            const float tau = taus[k];
            if (tau != 0.f) {
                float v[R];
#pragma unroll
                for (int t = 0; t < R; t++) v[t] = vb[lane + 32 * t];
                const bool own_active = warp > kk;  // slot kb holds column warp + 4 kb > k
                float p[8];
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    float sdot = 0.f;
                    if (c > kb || (c == kb && own_active)) {
#pragma unroll
                        for (int t = 0; t < R; t++) sdot = fmaf(v[t], a[t][c], sdot);
                    }
                    p[c] = sdot;
                }
                const float w = reduce_scatter8(p, lane);
#pragma unroll
                for (int c = kb; c < 8; c++) {
                    if ((c > kb || own_active) && warp + 4 * c < n) {
                        const float twj = tau * shfl(w, 4 * c);
#pragma unroll
                        for (int t = 0; t < R; t++) a[t][c] = fmaf(-twj, v[t], a[t][c]);
                    }
                }
            }
        }
    }
    // factors to shared memory (all 32 columns: zeros beyond n)
#pragma unroll
    for (int c = 0; c < 8; c++)
#pragma unroll
        for (int t = 0; t < R; t++) Q[(warp + 4 * c) * LDQ + lane + 32 * t] = a[t][c];
    __syncthreads();
    if (warp == 0) {
        // info: first k whose diagonal entry R_kk is exactly zero (1-based)
        const unsigned zero = __ballot_sync(FULL, lane < n && Q[lane * LDQ + lane] == 0.f);
        if (info && lane == 0) info[mat] = zero ? __ffs(zero) : 0;
    }
    ls_solve_block<R>(m, n, nrhs, Q, A0, taus, a_g, B + mat * sB, refine, warp, lane);
}

// --------------------------------------------- standalone ormqr / trsm
// ormqr (left): C <- Q^T C (trans) or Q C, reflectors from a geqrf output.
template <typename T, int R>
__global__ void __launch_bounds__(128) k_ormqr_warp(int trans, int m, int nc, int kk, const T *__restrict__ A,
                                                    int64_t sA, const T *__restrict__ tau, int64_t sTau,
                                                    T *__restrict__ Cm, int64_t sC, int batch) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mat = (int64_t)blockIdx.x * 4 + warp;
    if (mat >= batch) return;
    const T *a = A + mat * sA;
    const T *tg = tau + mat * sTau;
    for (int c = 0; c < nc; c++) {
        T *col = Cm + mat * sC + (int64_t)c * m;
        T y[R];
#pragma unroll
        for (int t = 0; t < R; t++) {
            int r = lane + 32 * t;
            y[t] = r < m ? col[r] : T(0);
        }
        for (int s = 0; s < kk; s++) {
            int k = trans ? s : kk - 1 - s;
            T tk = tg[k];
            T v[R];
            T p = T(0);
#pragma unroll
            for (int t = 0; t < R; t++) {
                int r = lane + 32 * t;
                v[t] = r > k && r < m ? a[(int64_t)k * m + r] : (r == k ? T(1) : T(0));
                p = fma(v[t], y[t], p);
            }
            p = tk * warp_sum(p);
#pragma unroll
            for (int t = 0; t < R; t++) y[t] = fma(-p, v[t], y[t]);
        }
#pragma unroll
        for (int t = 0; t < R; t++) {
            int r = lane + 32 * t;
            if (r < m) col[r] = y[t];
        }
    }
}

// trsm (left, upper, no transpose, non-unit): B(0:n, :) <- R^-1 B(0:n, :),
// R = upper triangle of the leading n x n block of a matrix with leading
// dimension ldr; B has leading dimension ldb.
template <typename T>
__global__ void __launch_bounds__(128) k_trsm_upper_warp(int n, int nc, const T *__restrict__ Rm, int64_t ldr,
                                                         int64_t sR, T *__restrict__ Bm, int64_t ldb, int64_t sB,
                                                         int batch) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mat = (int64_t)blockIdx.x * 4 + warp;
    if (mat >= batch) return;
    const T *r = Rm + mat * sR;
    for (int c = 0; c < nc; c++) {
        T *col = Bm + mat * sB + (int64_t)c * ldb;
        for (int j = n - 1; j >= 0; j--) {
            __syncwarp();
            T xj = col[j] / r[(int64_t)j * ldr + j];
            __syncwarp();
            for (int i = lane; i < j; i += 32) col[i] = fma(-r[(int64_t)j * ldr + i], xj, col[i]);
            if (lane == 0) col[j] = xj;
        }
        __syncwarp();
    }
}

template <typename T>
static inline gbla_status qr_launch(int m, int n, int nrhs, T *A, int64_t sA, T *B, int64_t sB, T *tau, int64_t sTau,
                             int *info, int flags, int refine, int batch, cudaStream_t st) {
    if (m < 0 || n < 0 || nrhs < 0 || batch < 0 || refine < 0 || m < n) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0) return GBLA_SUCCESS;
    if (!A || sA < (int64_t)m * n) return GBLA_INVALID_VALUE;
    if ((flags & QR_SOLVE) && nrhs > 0 && (!B || sB < (int64_t)m * nrhs)) return GBLA_INVALID_VALUE;
    if ((flags & QR_WRITE_TAU) && (!tau || sTau < n)) return GBLA_INVALID_VALUE;
    if (sizeof(T) != 4) refine = 0;
    if (m > 128 || n > 32) return qr_big_launch<T>(m, n, nrhs, A, sA, B, sB, tau, sTau, info, flags, refine, batch, st);
    const int R = (m + 31) / 32;
    const unsigned grid = (unsigned)((batch + 3) / 4);
    auto go = [&](auto kern) -> gbla_status {
        kern<<<grid, 128, 0, st>>>(m, n, nrhs, A, sA, B, sB, tau, sTau, info, flags, batch, (T *)nullptr, (int64_t)0);
        return launch_status();
    };
    if constexpr (sizeof(T) == 8) {
        // FP64 (geqrf and least squares): one instantiation per row count;
        // the solve is skipped at run time when not requested
        switch (R) {
            case 1: return go(k_qr_warp<T, 1>);
            case 2: return go(k_qr_warp<T, 2>);
            case 3: return go(k_qr_warp<T, 3>);
            default: return go(k_qr_warp<T, 4>);
        }
    } else {
        // FP32 factorisation only (geqrf; FP32 least squares runs k_gels_cta):
        // the variant without the solve code fits three blocks per SM
        if ((flags & QR_SOLVE) && nrhs > 0) return GBLA_NOT_SUPPORTED;
        switch (R) {
            case 1: return go(k_qr_warp<T, 1, false>);
            case 2: return go(k_qr_warp<T, 2, false>);
            case 3: return go(k_qr_warp<T, 3, false>);
            default: return go(k_qr_warp<T, 4, false>);
        }
    }
}

template <typename T>
static inline gbla_status ormqr_launch(int trans, int m, int nc, int k, const T *A, int64_t sA, const T *tau, int64_t sTau,
                                T *Cm, int64_t sC, int batch, cudaStream_t st) {
    if (m < 0 || nc < 0 || k < 0 || k > m || batch < 0) return GBLA_INVALID_VALUE;
    if (batch == 0 || nc == 0 || k == 0 || m == 0) return GBLA_SUCCESS;
    if (!A || !tau || !Cm || sA < (int64_t)m * k || sTau < k || sC < (int64_t)m * nc) return GBLA_INVALID_VALUE;
    if (m > 128) return ormqr_big_launch<T>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, batch, st);
    const unsigned grid = (unsigned)((batch + 3) / 4);
    switch ((m + 31) / 32) {
        case 1: k_ormqr_warp<T, 1><<<grid, 128, 0, st>>>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, batch); break;
        case 2: k_ormqr_warp<T, 2><<<grid, 128, 0, st>>>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, batch); break;
        case 3: k_ormqr_warp<T, 3><<<grid, 128, 0, st>>>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, batch); break;
        default: k_ormqr_warp<T, 4><<<grid, 128, 0, st>>>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, batch); break;
    }
    return launch_status();
}

template <typename T>
static inline gbla_status trsm_launch(int n, int nc, const T *Rm, int64_t ldr, int64_t sR, T *Bm, int64_t ldb, int64_t sB,
                               int batch, cudaStream_t st) {
    if (n < 0 || nc < 0 || batch < 0 || ldr < n || ldb < n) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0 || nc == 0) return GBLA_SUCCESS;
    if (!Rm || !Bm || sR < ldr * n || sB < ldb * nc) return GBLA_INVALID_VALUE;
    k_trsm_upper_warp<T><<<(unsigned)((batch + 3) / 4), 128, 0, st>>>(n, nc, Rm, ldr, sR, Bm, ldb, sB, batch);
    return launch_status();
}

}  // namespace gbla
