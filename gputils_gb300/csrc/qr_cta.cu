// qr_cta.cu -- batched Householder QR, least squares and Q application for
// any m >= n: the shapes beyond the register-resident warp kernels of
// qr_common.cuh (m <= 128, n <= 32).
//
// One block of QB_THREADS threads per matrix (persistent grid).  The working
// matrix W lives in shared memory (column stride m | 1, odd, so that a row
// of R read by consecutive lanes is conflict-free) when it fits, else in A
// itself (global memory, column stride m; the factorisation overwrites A in
// any case).  Householder steps follow LAPACK dgeqr2/dlarfg as the warp
// kernels do (beta = -sign(alpha) ||x||, tau = (beta - alpha) / beta, v with
// an implicit unit entry at row k): per column k the block reduces the
// squared norm below the diagonal, scales the reflector, and every warp
// applies it to its own trailing columns (one warp reduction per column).
//
// Least squares: warps take one right-hand side each (as many warps as the
// per-warp vectors fit in shared memory), y = Q^T b, x = R^-1 y(0:n).  In
// single precision refine_iters steps of augmented-system refinement follow
// (the scheme of qr_common.cuh: residuals f = b - r - A x and g = -A^T r in
// double-FP32 arithmetic against the original A, which stays in global
// memory until the factors are stored; corrections solved with the FP32
// factors).  A lane owns the rows i = lane (mod 32) of every per-warp vector,
// so a vector entry is only ever read and written by the same lane.
#include "qr_big.cuh"
#include "xprec.cuh"

namespace gbla {

constexpr int QB_THREADS = 256;
constexpr int QB_WARPS = QB_THREADS / 32;
constexpr size_t QB_SMEM_MAX = 226 * 1024;  // below the 227 KB opt-in, leaving room for static shared memory

template <typename T>
__device__ __forceinline__ T qb_block_sum(T v, T *red, int warp, int lane) {
    v = warp_sum(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    T s = T(0);
#pragma unroll
    for (int w = 0; w < QB_WARPS; w++) s += red[w];  // same order in every thread
    return s;
}

// y <- Q^T y (trans) or Q y for one vector in per-warp shared memory; the
// reflectors are columns 0..kk-1 of W (stride ldw).
template <typename T>
__device__ __forceinline__ void qb_apply_q(bool trans, int m, int kk, const T *W, int64_t ldw, const T *taus, T *y,
                                           int lane) {
    for (int s = 0; s < kk; s++) {
        const int k = trans ? s : kk - 1 - s;
        const T *v = W + (int64_t)k * ldw;
        T p = T(0);
        for (int i = lane; i < m; i += 32)
            if (i >= k) p = fma(i == k ? T(1) : v[i], y[i], p);
        p = taus[k] * warp_sum(p);
        for (int i = lane; i < m; i += 32)
            if (i >= k) y[i] = fma(-p, i == k ? T(1) : v[i], y[i]);
    }
}

// Solve R z = y(0:n) in place (rows of y owned by lanes); R = upper triangle of W.
template <typename T>
__device__ __forceinline__ void qb_back_solve(int n, const T *W, int64_t ldw, const T *dinv, T *y, int lane) {
    for (int j = n - 1; j >= 0; j--) {
        const T zj = shfl(lane == (j & 31) ? y[j] * dinv[j] : T(0), j & 31);
        if (lane == (j & 31)) y[j] = zj;
        const T *rj = W + (int64_t)j * ldw;
        for (int i = lane; i < j; i += 32) y[i] = fma(-rj[i], zj, y[i]);
    }
}

// Solve R^T h = g in place (g(0:n) owned by lanes): once h_j is known every
// later entry l subtracts R(j, l) h_j.
template <typename T>
__device__ __forceinline__ void qb_forward_solve_rt(int n, const T *W, int64_t ldw, const T *dinv, T *g, int lane) {
    for (int j = 0; j < n; j++) {
        const T hj = shfl(lane == (j & 31) ? g[j] * dinv[j] : T(0), j & 31);
        if (lane == (j & 31)) g[j] = hj;
        for (int l = j + 1 + ((lane - (j + 1)) & 31); l < n; l += 32) g[l] = fma(-W[(int64_t)l * ldw + j], hj, g[l]);
    }
}

// Per-warp shared-memory vectors of the solve phase, in elements of T.
template <typename T>
__host__ __device__ constexpr int64_t qb_warp_elems(int m, int n, bool refine) {
    // refine (float): y, d, rh, rl (m each); xh, xl, g (n each); else y (m)
    return refine ? 4 * (int64_t)m + 3 * (int64_t)n : (int64_t)m;
}

template <typename T, bool SMEM>
__global__ void __launch_bounds__(QB_THREADS, 1) k_qr_cta(int m, int n, int nrhs, T *__restrict__ A, int64_t sA,
                                                       T *__restrict__ B, int64_t sB, T *__restrict__ tau_g,
                                                       int64_t sTau, int *__restrict__ info, int flags, int refine,
                                                       int solve_warps, int batch) {
    extern __shared__ __align__(16) unsigned char qb_raw[];
    T *sm = reinterpret_cast<T *>(qb_raw);
    const int64_t ldw = SMEM ? (int64_t)(m | 1) : (int64_t)m;
    T *Ws = sm;                                      // SMEM: n columns x ldw
    T *taus = sm + (SMEM ? (int64_t)n * ldw : 0);    // n
    T *dinv = taus + n;                              // n
    T *red = dinv + n;                               // 32
    T *wbuf = red + 32;                              // solve_warps x qb_warp_elems
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool do_solve = (flags & QR_SOLVE) && nrhs > 0;
    const bool do_refine = sizeof(T) == 4 && do_solve && refine > 0;

    for (int64_t mat = blockIdx.x; mat < batch; mat += gridDim.x) {
        T *a_g = A + mat * sA;
        T *W = SMEM ? Ws : a_g;
        if (SMEM) {
            for (int j = warp; j < n; j += QB_WARPS)
                for (int i = lane; i < m; i += 32) W[(int64_t)j * ldw + i] = a_g[(int64_t)j * m + i];
        }
        if (tid == 0) s_fail = 0;
        __syncthreads();
        // ---- factorisation
        for (int k = 0; k < n; k++) {
            T *vk = W + (int64_t)k * ldw;
            T part = T(0);
            for (int i = k + 1 + tid; i < m; i += QB_THREADS) part = fma(vk[i], vk[i], part);
            const T x2 = qb_block_sum<T>(part, red, warp, lane);
            const T alpha = vk[k];
            T tau = T(0), beta = alpha;
            if (x2 > T(0)) {
                beta = -copysign(dev_sqrt<T>(fma(alpha, alpha, x2)), alpha);
                tau = (beta - alpha) / beta;
                const T scal = T(1) / (alpha - beta);
                for (int i = k + 1 + tid; i < m; i += QB_THREADS) vk[i] *= scal;
            }
            __syncthreads();  // v complete; every thread has read red and vk[k]
            if (tid == 0) {
                vk[k] = beta;
                taus[k] = tau;
                dinv[k] = beta != T(0) ? T(1) / beta : T(0);
                if (beta == T(0) && s_fail == 0) s_fail = k + 1;
            }
            if (tau != T(0)) {
                for (int j = k + 1 + warp; j < n; j += QB_WARPS) {
                    T *aj = W + (int64_t)j * ldw;
                    T p = T(0);
                    for (int i = k + lane; i < m; i += 32) p = fma(i == k ? T(1) : vk[i], aj[i], p);
                    p = tau * warp_sum(p);
                    for (int i = k + lane; i < m; i += 32) aj[i] = fma(-p, i == k ? T(1) : vk[i], aj[i]);
                }
            }
            __syncthreads();
        }
        if (tid == 0 && info) info[mat] = s_fail;

        // ---- least squares, one right-hand side per solve warp
        if (do_solve && warp < solve_warps) {
            T *b_g = B + mat * sB;
            T *y = wbuf + (int64_t)warp * qb_warp_elems<T>(m, n, do_refine);
            for (int c = warp; c < nrhs; c += solve_warps) {
                T *bc = b_g + (int64_t)c * m;
                for (int i = lane; i < m; i += 32) y[i] = bc[i];
                qb_apply_q<T>(true, m, n, W, ldw, taus, y, lane);  // y = Q^T b
                if (!do_refine) {
                    qb_back_solve<T>(n, W, ldw, dinv, y, lane);
                    __syncwarp();
                    for (int i = lane; i < m; i += 32) bc[i] = y[i];  // x in rows < n, (Q^T b)(n:m) below
                    __syncwarp();
                    continue;
                }
                if constexpr (sizeof(T) == 4) {
                    float *d = y + m, *rh = d + m, *rl = rh + m, *xh = rl + m, *xl = xh + n, *g = xl + n;
                    const float *a0 = a_g;  // the original A: global memory is untouched until the factors are stored
                    for (int i = lane; i < n; i += 32) { d[i] = y[i]; }
                    qb_back_solve<float>(n, W, ldw, dinv, d, lane);
                    for (int i = lane; i < n; i += 32) { xh[i] = d[i]; xl[i] = 0.f; }
                    for (int i = lane; i < m; i += 32) { rh[i] = 0.f; rl[i] = 0.f; }
                    __syncwarp();
                    for (int it = 0; it <= refine; it++) {
                        // f = b - r - A x; skipped at it == 1 (r is the residual of the
                        // unchanged x adopted at it == 0, so f vanishes to ~2^-48)
                        const bool fzero = it == 1;
                        if (!fzero) {
                            for (int i = lane; i < m; i += 32) {
                                ff f;
                                f.h = bc[i];
                                f.l = 0.f;
                                ff_add(f, -rh[i], -rl[i]);
                                for (int j = 0; j < n; j++) ff_fma(f, -a0[(int64_t)j * m + i], xh[j], xl[j]);
                                if (it == 0) {
                                    const ff fn = ff_norm(f);
                                    rh[i] = fn.h;
                                    rl[i] = fn.l;
                                } else {
                                    d[i] = f.h + f.l;
                                }
                            }
                        } else {
                            for (int i = lane; i < m; i += 32) d[i] = 0.f;
                        }
                        __syncwarp();
                        if (it == 0) continue;
                        // g = -A^T r (entry j reduced over the warp, kept by lane j mod 32)
                        for (int j = 0; j < n; j++) {
                            ff acc;
                            acc.h = 0.f;
                            acc.l = 0.f;
                            for (int i = lane; i < m; i += 32) ff_fma(acc, a0[(int64_t)j * m + i], rh[i], rl[i]);
                            acc = ff_warp_sum(acc);
                            if (lane == (j & 31)) g[j] = -(acc.h + acc.l);
                        }
                        __syncwarp();
                        qb_forward_solve_rt<float>(n, W, ldw, dinv, g, lane);  // g <- h = R^-T g
                        if (!fzero) qb_apply_q<float>(true, m, n, W, ldw, taus, d, lane);  // d = Q^T f
                        __syncwarp();
                        // dx = R^-1 (d(0:n) - h); d(n:m) keeps d_2 for the residual update
                        float *dx = d;  // rows < n of d become dx
                        for (int i = lane; i < n; i += 32) dx[i] = d[i] - g[i];
                        __syncwarp();
                        qb_back_solve<float>(n, W, ldw, dinv, dx, lane);
                        __syncwarp();
                        for (int i = lane; i < n; i += 32) {
                            float s, e;
                            two_sum(xh[i], dx[i], s, e);
                            const float l = xl[i] + e;
                            xh[i] = s + l;
                            xl[i] = l - (xh[i] - s);
                        }
                        __syncwarp();
                        if (it < refine) {
                            // dr = Q [h; d_2]: rows < n take h, rows >= n keep d_2
                            for (int i = lane; i < n; i += 32) d[i] = g[i];
                            __syncwarp();
                            qb_apply_q<float>(false, m, n, W, ldw, taus, d, lane);
                            for (int i = lane; i < m; i += 32) {
                                float s, e;
                                two_sum(rh[i], d[i], s, e);
                                const float l = rl[i] + e;
                                rh[i] = s + l;
                                rl[i] = l - (rh[i] - s);
                            }
                            __syncwarp();
                        }
                    }
                    for (int i = lane; i < m; i += 32) bc[i] = i < n ? xh[i] + xl[i] : y[i];
                    __syncwarp();
                }
            }
        }
        __syncthreads();  // every solve warp is done with W and with A as the original
        if (SMEM && (flags & QR_WRITE_FACTORS)) {
            for (int j = warp; j < n; j += QB_WARPS)
                for (int i = lane; i < m; i += 32) a_g[(int64_t)j * m + i] = W[(int64_t)j * ldw + i];
        }
        if ((flags & QR_WRITE_TAU) && tau_g)
            for (int k = tid; k < n; k += QB_THREADS) tau_g[mat * sTau + k] = taus[k];
        __syncthreads();
    }
}

// ormqr for any m: one warp per (matrix, column of C), the column updated in
// place in global memory, reflectors read from A.
template <typename T>
__global__ void __launch_bounds__(256) k_ormqr_gen(int trans, int m, int nc, int kk, const T *__restrict__ A,
                                                   int64_t sA, const T *__restrict__ tau, int64_t sTau,
                                                   T *__restrict__ Cm, int64_t sC, int64_t total) {
    const int lane = threadIdx.x & 31;
    const int64_t job = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (job >= total) return;  // whole warps leave together
    const int64_t mat = job / nc;
    const int c = (int)(job % nc);
    const T *a = A + mat * sA;
    const T *tg = tau + mat * sTau;
    T *y = Cm + mat * sC + (int64_t)c * m;
    for (int s = 0; s < kk; s++) {
        const int k = trans ? s : kk - 1 - s;
        const T *v = a + (int64_t)k * m;
        T p = T(0);
        for (int i = k + lane; i < m; i += 32) p = fma(i == k ? T(1) : v[i], y[i], p);
        p = tg[k] * warp_sum(p);
        for (int i = k + lane; i < m; i += 32) y[i] = fma(-p, i == k ? T(1) : v[i], y[i]);
        __syncwarp();
    }
}

// ------------------------------------------------------------ launchers
template <typename T>
static size_t qb_fixed_bytes(int n) {
    return sizeof(T) * (2 * (size_t)n + 32) + 16;
}

template <typename T>
gbla_status qr_big_launch(int m, int n, int nrhs, T *A, int64_t sA, T *B, int64_t sB, T *tau, int64_t sTau,
                          int *info, int flags, int refine, int batch, cudaStream_t st) {
    const bool solve = (flags & QR_SOLVE) && nrhs > 0;
    const bool do_refine = sizeof(T) == 4 && solve && refine > 0;
    const size_t w_bytes = sizeof(T) * (size_t)n * (size_t)(m | 1);
    const size_t per_warp = solve ? sizeof(T) * (size_t)qb_warp_elems<T>(m, n, do_refine) : 0;
    const size_t fixed = qb_fixed_bytes<T>(n);
    bool in_smem = w_bytes + fixed + per_warp <= QB_SMEM_MAX;
    // refinement reads the original A from global memory while W is worked
    // on: W must then be in shared memory
    if (do_refine && !in_smem) return GBLA_NOT_SUPPORTED;
    const size_t base = fixed + (in_smem ? w_bytes : 0);
    if (base + per_warp > QB_SMEM_MAX) return GBLA_NOT_SUPPORTED;  // a single vector of the solve does not fit
    int sw = 0;
    if (solve) {
        sw = (int)((QB_SMEM_MAX - base) / per_warp);
        sw = sw < QB_WARPS ? sw : QB_WARPS;
        sw = sw < nrhs ? sw : nrhs;
    }
    const size_t smem = base + per_warp * (size_t)sw;
    auto go = [&](auto kern) -> gbla_status {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return from_cuda(e);
        }
        const int64_t grid = persistent_grid(reinterpret_cast<const void *>(kern), QB_THREADS, smem, batch);
        kern<<<(unsigned)grid, QB_THREADS, smem, st>>>(m, n, nrhs, A, sA, B, sB, tau, sTau, info, flags, refine, sw,
                                                       batch);
        return launch_status();
    };
    return in_smem ? go(k_qr_cta<T, true>) : go(k_qr_cta<T, false>);
}

template <typename T>
gbla_status ormqr_big_launch(int trans, int m, int nc, int k, const T *A, int64_t sA, const T *tau, int64_t sTau,
                             T *Cm, int64_t sC, int batch, cudaStream_t st) {
    const int64_t total = (int64_t)batch * nc;
    const int64_t blocks = (total * 32 + 255) / 256;
    if (blocks > 0x7fffffff) return GBLA_INVALID_VALUE;
    k_ormqr_gen<T><<<(unsigned)blocks, 256, 0, st>>>(trans, m, nc, k, A, sA, tau, sTau, Cm, sC, total);
    return launch_status();
}

template gbla_status qr_big_launch<float>(int, int, int, float *, int64_t, float *, int64_t, float *, int64_t, int *,
                                          int, int, int, cudaStream_t);
template gbla_status qr_big_launch<double>(int, int, int, double *, int64_t, double *, int64_t, double *, int64_t,
                                           int *, int, int, int, cudaStream_t);
template gbla_status ormqr_big_launch<float>(int, int, int, int, const float *, int64_t, const float *, int64_t,
                                             float *, int64_t, int, cudaStream_t);
template gbla_status ormqr_big_launch<double>(int, int, int, int, const double *, int64_t, const double *, int64_t,
                                              double *, int64_t, int, cudaStream_t);

}  // namespace gbla
