// svd_big.cu -- batched one-sided Jacobi SVD for the shapes beyond the warp
// and 64-column block kernels of svd.cu: n <= 128 columns, any m >= n rows.
//
// One block of 256 threads (32 groups of 8 lanes) per matrix, persistent
// grid.  V (n x n) is always in shared memory; A's working copy is too when
// it fits (f32 up to 256 x 128), otherwise the rotations run on A itself in
// global memory (the API destroys A).  Same method as the block kernel of
// svd.cu: round-robin pairs (a group takes pairs g and g + 32 of a round),
// cached column norms, rotation while |a_p.a_q| > tol' |a_p||a_q| with
// tol' = max(tol, 4 sqrt(m) u), the same rotation formulas, sweep loop ending
// after a sweep without rotations.  In shared memory the column strides are
// multiples of 32 words and the four groups of a warp start their row walk 8
// rows apart (conflict-free), with zero padding rows that every rotation
// keeps zero.
//
// Epilogue as the block kernel: V normalised; sigma_j = |A v_j| from the
// original A when the working copy was in shared memory (A untouched in
// global memory), else the rotated column norm; descending order; the
// largest-magnitude entry of each v_j made negative; U columns from the
// rotated columns, completed to an orthonormal basis of R^m by scanning
// e_0, e_1, ... -- each candidate projected out of the columns so far twice
// (classical Gram-Schmidt with one re-orthogonalisation; the first
// projection needs no dot products because U^T e_i is row i of U), accepted
// when its remaining norm exceeds 0.5 / sqrt(m), signs alternating.
#include <cfloat>
#include "common.cuh"
#include "svd_big.cuh"

namespace gbla {

constexpr int SB_THREADS = 256;
constexpr int SB_WARPS = SB_THREADS / 32;
constexpr int SB_GROUP = 8;
constexpr int SB_GROUPS = SB_THREADS / SB_GROUP;
constexpr size_t SB_SMEM_MAX = 226 * 1024;  // below the 227 KB opt-in, leaving room for static shared memory

template <typename T> __device__ __forceinline__ T sb_unit_roundoff();
template <> __device__ __forceinline__ float sb_unit_roundoff<float>() { return 5.9604645e-8f; }
template <> __device__ __forceinline__ double sb_unit_roundoff<double>() { return 1.1102230246251565e-16; }

// Rotation (c, s) of the pair with squared norms alpha, beta and inner
// product gamma; t = tan(theta) for the norm update.  Correctly rounded
// division and square roots (as the warp kernel of svd.cu).
template <typename T>
__device__ __forceinline__ bool sb_rotation(T alpha, T beta, T gamma, T tol, T small, T &c, T &s, T &t) {
    if (alpha <= small || beta <= small || gamma == T(0)) return false;
    if (!(fabs(gamma) > tol * sqrt(alpha) * sqrt(beta))) return false;
    const T zeta = (beta - alpha) / (T(2) * gamma);
    const T az = fabs(zeta);
    const T big = sizeof(T) == 4 ? T(1e18) : T(1e150);
    t = az < big ? copysign(T(1), zeta) / (az + sqrt(fma(zeta, zeta, T(1)))) : T(0.5) / zeta;
    if (t == T(0)) return false;
    c = T(1) / sqrt(fma(t, t, T(1)));
    s = c * t;
    return true;
}

template <typename T>
__device__ __forceinline__ T sb_block_sum(T v, T *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    v = warp_sum(v);
    __syncthreads();  // red is free (earlier readers are done)
    if (lane == 0) red[warp] = v;
    __syncthreads();
    T s = T(0);
#pragma unroll
    for (int w = 0; w < SB_WARPS; w++) s += red[w];
    return s;
}

template <typename T, bool A_SMEM>
__global__ void __launch_bounds__(SB_THREADS, 1) k_gesvj_big(int m, int n, T *__restrict__ A, int64_t sA,
                                                          T *__restrict__ S, int64_t sS, T *__restrict__ Vt,
                                                          int64_t sVt, T *__restrict__ U, int64_t sU, T tol,
                                                          int max_sweeps, int *__restrict__ info,
                                                          int *__restrict__ sweeps_out, int batch) {
    extern __shared__ __align__(16) unsigned char sb_raw[];
    T *sm = reinterpret_cast<T *>(sb_raw);
    const int lda = A_SMEM ? (int)round_up(m, 32) : m;
    const int ldv = (int)round_up(n, 32);
    T *As = sm;                                           // A_SMEM: n columns x lda
    T *v = sm + (A_SMEM ? (int64_t)n * lda : 0);          // n columns x ldv
    T *nrm = v + (int64_t)n * ldv;                        // n: cached |a_j|^2
    T *sig = nrm + n;                                     // n
    T *rinv = sig + n;                                    // n
    T *red = rinv + n;                                    // 32
    T *wv = red + 32;                                     // m: completion candidate
    T *dv = wv + m;                                       // m: its projections
    const int tid = threadIdx.x, g = tid / SB_GROUP, gl = tid % SB_GROUP;
    const int N = n + (n & 1), M = N - 1;
    const int w0 = gl + 8 * (g & 3);  // < 32 <= lda (shared) and ldv
    const int arows = A_SMEM ? lda : m;

    for (int64_t mat = blockIdx.x; mat < batch; mat += gridDim.x) {
        T *ag = A + mat * sA;
        T *a = A_SMEM ? As : ag;
        if (A_SMEM) {
            for (int64_t e = tid; e < (int64_t)lda * n; e += SB_THREADS) {
                const int i = (int)(e % lda), j = (int)(e / lda);
                a[e] = i < m ? ag[(int64_t)j * m + i] : T(0);
            }
        }
        for (int64_t e = tid; e < (int64_t)ldv * n; e += SB_THREADS) {
            const int i = (int)(e % ldv), j = (int)(e / ldv);
            v[e] = i == j ? T(1) : T(0);
        }
        T f = T(0);
        for (int64_t e = tid; e < (int64_t)m * n; e += SB_THREADS) f = fma(ag[e], ag[e], f);  // A not yet rotated
        const T fro2 = sb_block_sum<T>(f, red);  // its barriers also complete the loads above
        const T eps = T(2) * sb_unit_roundoff<T>();
        const T small = eps * eps * fro2;
        const T floor_ = T(4) * sqrt(T(m)) * sb_unit_roundoff<T>();
        const T tol_eff = tol > floor_ ? tol : floor_;
        int sweep = 0, converged = 0;
        for (sweep = 1; sweep <= max_sweeps; sweep++) {
            // refresh the cached norms (group g: columns g, g + 32, ...); the
            // trip count is the same in every lane of a warp
            for (int j0 = 0; j0 < n; j0 += SB_GROUPS) {
                const int j = j0 + g;
                T s2 = T(0);
                if (j < n) {
                    const T *col = a + (int64_t)j * lda;
                    for (int t = gl; t < arows; t += 8) {
                        const int i = A_SMEM ? (w0 + t - gl < lda ? w0 + t - gl : w0 + t - gl - lda) : t;
                        s2 = fma(col[i], col[i], s2);
                    }
                }
                s2 = group_sum(s2, SB_GROUP);
                if (gl == 0 && j < n) nrm[j] = s2;
            }
            __syncthreads();
            int rotated = 0;
            for (int r = 0; r < M; r++) {
                // the same trip count in every lane: the group sums shuffle across the warp
                for (int pb = 0; pb < N / 2; pb += SB_GROUPS) {
                    const int pg = pb + g;
                    int x, y;
                    if (pg == 0) {
                        x = M;
                        y = r;
                    } else {
                        x = r + pg;
                        if (x >= M) x -= M;
                        y = r - pg;
                        if (y < 0) y += M;
                    }
                    const int p = x < y ? x : y, q = x < y ? y : x;
                    const bool act = pg < N / 2 && q < n;
                    T gamma = T(0);
                    T *ap = a + (int64_t)(act ? p : 0) * lda, *aq = a + (int64_t)(act ? q : 0) * lda;
                    if (act) {
                        for (int t = gl; t < arows; t += 8) {
                            const int i = A_SMEM ? (w0 + t - gl < lda ? w0 + t - gl : w0 + t - gl - lda) : t;
                            gamma = fma(ap[i], aq[i], gamma);
                        }
                    }
                    gamma = group_sum(gamma, SB_GROUP);
                    T c, sn, tn;
                    if (act && sb_rotation<T>(nrm[p], nrm[q], gamma, tol_eff, small, c, sn, tn)) {
                        rotated = 1;
                        for (int t = gl; t < arows; t += 8) {
                            const int i = A_SMEM ? (w0 + t - gl < lda ? w0 + t - gl : w0 + t - gl - lda) : t;
                            const T xa = ap[i], ya = aq[i];
                            ap[i] = fma(c, xa, -sn * ya);
                            aq[i] = fma(sn, xa, c * ya);
                        }
                        T *vp = v + (int64_t)p * ldv, *vq = v + (int64_t)q * ldv;
                        for (int t = gl; t < ldv; t += 8) {
                            const int i = w0 + t - gl < ldv ? w0 + t - gl : w0 + t - gl - ldv;
                            const T xv = vp[i], yv = vq[i];
                            vp[i] = fma(c, xv, -sn * yv);
                            vq[i] = fma(sn, xv, c * yv);
                        }
                        __syncwarp(0xffu << (8 * ((tid & 31) / 8)));  // the group has read nrm[p], nrm[q]
                        if (gl == 0) {
                            const T al = nrm[p], be = nrm[q];
                            nrm[p] = fma(-tn, gamma, al);
                            nrm[q] = fma(tn, gamma, be);
                        }
                    }
                }
                __syncthreads();
            }
            if (!__syncthreads_or(rotated)) {
                converged = 1;
                break;
            }
        }
        const int total = converged ? sweep : max_sweeps;
        // ---- epilogue: normalise V
        const int warp = tid >> 5, lane = tid & 31;
        for (int j = warp; j < n; j += SB_WARPS) {
            T s2 = T(0);
            for (int i = lane; i < n; i += 32) s2 = fma(v[(int64_t)j * ldv + i], v[(int64_t)j * ldv + i], s2);
            s2 = warp_sum(s2);
            const T inv = s2 > T(0) ? T(1) / sqrt(s2) : T(0);
            for (int i = lane; i < n; i += 32) v[(int64_t)j * ldv + i] *= inv;
        }
        __syncthreads();
        for (int j = warp; j < n; j += SB_WARPS) {
            T r2 = T(0);
            for (int i = lane; i < m; i += 32) r2 = fma(a[(int64_t)j * lda + i], a[(int64_t)j * lda + i], r2);
            r2 = warp_sum(r2);
            T s2 = r2;
            if (A_SMEM) {
                // sigma_j = |A v_j| from the original A (second order in v_j's error)
                s2 = T(0);
                for (int i = lane; i < m; i += 32) {
                    T b = T(0);
                    for (int k = 0; k < n; k++) b = fma(ag[(int64_t)k * m + i], v[(int64_t)j * ldv + k], b);
                    s2 = fma(b, b, s2);
                }
                s2 = warp_sum(s2);
            }
            if (lane == 0) {
                sig[j] = sqrt(s2);
                rinv[j] = r2 > T(0) ? T(1) / sqrt(r2) : T(0);
            }
        }
        __syncthreads();
        T smax = T(0);
        for (int k = 0; k < n; k++) smax = fmax(smax, sig[k]);
        const T thr = smax * (T)(m > n ? m : n) * eps;
        // one warp per column: position, sign, S, V^T and U columns
        for (int j = warp; j < n; j += SB_WARPS) {
            int ps = 0;
            for (int k = lane; k < n; k += 32) ps += (sig[k] > sig[j] || (sig[k] == sig[j] && k < j)) ? 1 : 0;
            ps = warp_sum(ps);
            T vmax = T(-1);
            int imax = 0;
            for (int i = lane; i < n; i += 32) {
                const T av = fabs(v[(int64_t)j * ldv + i]);
                if (av > vmax) { vmax = av; imax = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {  // first index of the largest magnitude
                const T ov = shfl_xor(vmax, o);
                const int oi = shfl_xor(imax, o);
                if (ov > vmax || (ov == vmax && oi < imax)) { vmax = ov; imax = oi; }
            }
            const T sg = v[(int64_t)j * ldv + imax] > T(0) ? T(-1) : T(1);
            if (lane == 0) S[mat * sS + ps] = sig[j];
            for (int i = lane; i < n; i += 32) Vt[mat * sVt + (int64_t)i * n + ps] = sg * v[(int64_t)j * ldv + i];
            if (U && sig[j] > thr) {
                const T inv = sg * rinv[j];
                for (int i = lane; i < m; i += 32) U[mat * sU + (int64_t)ps * m + i] = a[(int64_t)j * lda + i] * inv;
            }
        }
        __syncthreads();
        if (U) {
            T *u = U + mat * sU;
            int c = 0;
            for (int k = 0; k < n; k++) c += sig[k] > thr ? 1 : 0;
            int ncomp = 0;
            const T accept = T(0.5) * rsqrt((T)m);
            for (int e = 0; e < m && c < m; e++) {
                // w = e_e - U(:, 0:c) U(e, 0:c)^T
                for (int i = tid; i < m; i += SB_THREADS) {
                    T acc = i == e ? T(1) : T(0);
                    for (int k = 0; k < c; k++) acc = fma(-u[(int64_t)k * m + i], u[(int64_t)k * m + e], acc);
                    wv[i] = acc;
                }
                __syncthreads();
                // re-orthogonalise: d = U^T w, w -= U d
                for (int k = warp; k < c; k += SB_WARPS) {
                    T p = T(0);
                    for (int i = lane; i < m; i += 32) p = fma(u[(int64_t)k * m + i], wv[i], p);
                    p = warp_sum(p);
                    if (lane == 0) dv[k] = p;
                }
                __syncthreads();
                T part = T(0);
                for (int i = tid; i < m; i += SB_THREADS) {
                    T acc = wv[i];
                    for (int k = 0; k < c; k++) acc = fma(-u[(int64_t)k * m + i], dv[k], acc);
                    wv[i] = acc;
                    part = fma(acc, acc, part);
                }
                const T nw = sqrt(sb_block_sum<T>(part, red));
                if (nw > accept) {
                    const T sc = ((ncomp & 1) ? T(-1) : T(1)) / nw;
                    for (int i = tid; i < m; i += SB_THREADS) u[(int64_t)c * m + i] = wv[i] * sc;
                    c++;
                    ncomp++;
                }
                __syncthreads();
            }
        }
        if (tid == 0) {
            if (info) info[mat] = converged ? 0 : 1;
            if (sweeps_out) sweeps_out[mat] = total;
        }
        __syncthreads();
    }
}

template <typename T>
static size_t sb_smem_bytes(int m, int n, bool a_smem) {
    const size_t lda = (size_t)round_up(m, 32), ldv = (size_t)round_up(n, 32);
    return sizeof(T) * ((a_smem ? (size_t)n * lda : 0) + (size_t)n * ldv + 3 * (size_t)n + 32 + 2 * (size_t)m) + 16;
}

template <typename T>
gbla_status svd_big_launch(int m, int n, T *A, int64_t sA, T *S, int64_t sS, T *Vt, int64_t sVt, T *U, int64_t sU,
                           T tol, int max_sweeps, int *info, int *sweeps, int batch, cudaStream_t st) {
    if (n > SVD_BIG_MAX_N) return GBLA_NOT_SUPPORTED;
    const bool a_smem = sb_smem_bytes<T>(m, n, true) <= SB_SMEM_MAX;
    const size_t smem = sb_smem_bytes<T>(m, n, a_smem);
    if (smem > SB_SMEM_MAX) return GBLA_NOT_SUPPORTED;  // the candidate vectors of a huge m do not fit
    auto go = [&](auto kern) -> gbla_status {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return from_cuda(e);
        }
        const int64_t grid = persistent_grid(reinterpret_cast<const void *>(kern), SB_THREADS, smem, batch);
        kern<<<(unsigned)grid, SB_THREADS, smem, st>>>(m, n, A, sA, S, sS, Vt, sVt, U, sU, tol, max_sweeps, info,
                                                       sweeps, batch);
        return launch_status();
    };
    return a_smem ? go(k_gesvj_big<T, true>) : go(k_gesvj_big<T, false>);
}

template gbla_status svd_big_launch<float>(int, int, float *, int64_t, float *, int64_t, float *, int64_t, float *,
                                           int64_t, float, int, int *, int *, int, cudaStream_t);
template gbla_status svd_big_launch<double>(int, int, double *, int64_t, double *, int64_t, double *, int64_t,
                                            double *, int64_t, double, int, int *, int *, int, cudaStream_t);

}  // namespace gbla
