// svd.cu -- batched one-sided (Hestenes) Jacobi SVD, rank count, null space.
//
// Replaces Svd<T>::factorise (a host loop of cusolverDn<t>gesvd, one call per
// matrix) and k_countNonzeroSingularValues.  The columns of A are rotated
// pairwise until they are mutually orthogonal; V accumulates the rotations.
// Every round rotates disjoint column pairs in parallel and a sweep meets
// every pair once, by recursive halving of the columns (n <= 64): level l
// cuts them into 2^l blocks [st, en) = [b n / 2^l, (b + 1) n / 2^l) (rounded
// down), each with halves [st, mid) and [mid, en), and pairs the halves in
// C = ceil(ceil(n / 2^l) / 2) rounds -- in round r, column st + i meets
// column mid + (i + r) mod cb, cb the larger half's size, while r < cb --
// until the blocks are single columns: n - 1 rounds for n a power of two,
// at most n + 3 otherwise.  (Measured on the 64 x 64 family: 8.4 sweeps
// against 9.1 for the round-robin circle tournament.)  A pair
// (p < q) is rotated when |a_p . a_q| > tol ||a_p|| ||a_q|| with the
// Rutishauser formulas (zeta = (|a_q|^2 - |a_p|^2) / (2 a_p.a_q),
// t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2))); the sweep loop ends after a
// sweep without rotations or after max_sweeps (info = 1 then).  Columns
// stored in FP32 cannot be orthogonal to better than about sqrt(m) u
// (u = 2^-24) relative, so the tolerance used is max(tol, 4 sqrt(m) u);
// below it a rotation would only stir rounding noise.
//
// Two kernel shapes:
//  * n <= 32, m <= 64 : one warp per matrix, lane j owns column j of A and of
//                       V in registers; the partner column arrives by shuffle
//                       (V's only in rounds where some pair of the warp rotates).
//  * n <= 64, m <= 128: one block per matrix, A and V in shared memory, a group
//                       of lanes per column pair (rows split across the group).
// Epilogue (both): singular values are the column norms, sorted descending;
// the singular pair's sign makes the largest-magnitude entry of v_j negative;
// U columns are a_j / sigma_j, completed to an orthonormal basis (Gram-Schmidt
// over e_0..e_{m-1}, the c-th completion column negated for odd c).
#include <cfloat>
#include "common.cuh"
#include "svd_big.cuh"

namespace gbla {

// Rotation for the pair (p, q): alpha = |a_p|^2, beta = |a_q|^2, gamma = a_p.a_q.
// Columns whose squared norm is <= small (FLT_EPSILON^2 |A|_F^2) are treated as
// zero.  c and s use correctly rounded division and square root: rsqrt's
// one-sided error would shrink the column norms over many rotations.
template <typename T>
__device__ __forceinline__ bool jacobi_rotation(T alpha, T beta, T gamma, T tol, T small, T &c, T &s) {
    if (alpha <= small || beta <= small || gamma == T(0)) return false;
    if (!(fabs(gamma) > tol * sqrt(alpha) * sqrt(beta))) return false;
    const T zeta = (beta - alpha) / (T(2) * gamma);
    const T az = fabs(zeta);
    const T big = sizeof(T) == 4 ? T(1e18) : T(1e150);
    const T t = az < big ? copysign(T(1), zeta) / (az + sqrt(fma(zeta, zeta, T(1)))) : T(0.5) / zeta;
    if (t == T(0)) return false;
    c = T(1) / sqrt(fma(t, t, T(1)));
    s = c * t;
    return true;
}

template <typename T> __device__ __forceinline__ T unit_roundoff();
template <> __device__ __forceinline__ float unit_roundoff<float>() { return 5.9604645e-8f; }
template <> __device__ __forceinline__ double unit_roundoff<double>() { return 1.1102230246251565e-16; }
template <typename T> __device__ __forceinline__ T mach_eps() { return T(2) * unit_roundoff<T>(); }

// 2^e and the binary exponent of x > 0 (x = f 2^e, f in [1, 2)).
template <typename T> __device__ __forceinline__ T pow2(int e);
template <> __device__ __forceinline__ float pow2<float>(int e) { return ldexpf(1.0f, e); }
template <> __device__ __forceinline__ double pow2<double>(int e) { return ldexp(1.0, e); }
__device__ __forceinline__ int ilogb_of(float x) { return ilogbf(x); }
__device__ __forceinline__ int ilogb_of(double x) { return ilogb(x); }

// Tolerance actually used: the request, but not below the FP32 noise floor
// of |a_p . a_q| / (|a_p| |a_q|) for m-row columns.
template <typename T>
__device__ __forceinline__ T jacobi_tol(T tol, int m) {
    const T floor_ = T(4) * sqrt(T(m)) * unit_roundoff<T>();
    return tol > floor_ ? tol : floor_;
}

// Rotation for the block kernel, with the column norms alpha, beta supplied
// (cached) and t = tan(theta) returned for the norm update.  FP32: the
// threshold test and the angle (zeta, t) use approximate reciprocals and
// square roots -- any t gives an exactly orthogonal (c, s) pair -- and c comes
// from a Newton-refined reciprocal square root, whose remaining bias
// (-1.5 e^2, e ~ 2^-22) is far below the rounding of the update itself.
template <typename T>
__device__ __forceinline__ bool jacobi_rotation_t(T alpha, T beta, T gamma, T tol, T small, T &c, T &s, T &t);

template <>
__device__ __forceinline__ bool jacobi_rotation_t<float>(float alpha, float beta, float gamma, float tol, float small,
                                                         float &c, float &s, float &t) {
    if (alpha <= small || beta <= small || gamma == 0.0f) return false;
    if (!(fabsf(gamma) * rsqrtf(alpha) * rsqrtf(beta) > tol)) return false;
    const float zeta = __fdividef(beta - alpha, 2.0f * gamma);
    const float az = fabsf(zeta);
    t = az < 1e18f ? copysignf(__frcp_rn(az + sqrtf(fmaf(zeta, zeta, 1.0f))), zeta) : __fdividef(0.5f, zeta);
    if (t == 0.0f) return false;
    const float x = fmaf(t, t, 1.0f);
    float y = rsqrtf(x);
    y = y * fmaf(-0.5f * x * y, y, 1.5f);
    c = y;
    s = c * t;
    return true;
}

template <>
__device__ __forceinline__ bool jacobi_rotation_t<double>(double alpha, double beta, double gamma, double tol,
                                                          double small, double &c, double &s, double &t) {
    if (alpha <= small || beta <= small || gamma == 0.0) return false;
    if (!(fabs(gamma) > tol * sqrt(alpha) * sqrt(beta))) return false;
    const double zeta = (beta - alpha) / (2.0 * gamma);
    const double az = fabs(zeta);
    t = az < 1e150 ? copysign(1.0, zeta) / (az + sqrt(fma(zeta, zeta, 1.0))) : 0.5 / zeta;
    if (t == 0.0) return false;
    c = 1.0 / sqrt(fma(t, t, 1.0));
    s = c * t;
    return true;
}

// FP32 block kernel, columns scaled so that |A|_F^2 < 4 (no square below can
// overflow): the threshold test as gamma^2 > tol^2 alpha beta, and with
// d = beta - alpha, t = 2 gamma / (d + sign(d) sqrt(d^2 + 4 gamma^2)), the
// same Rutishauser t (|t| <= 1) with one square root and one reciprocal in
// the dependency chain.
__device__ __forceinline__ bool jacobi_rotation_scaled(float alpha, float beta, float gamma, float tol, float small,
                                                       float &c, float &s, float &t) {
    if (alpha <= small || beta <= small || gamma == 0.0f) return false;
    if (!(gamma * gamma > (tol * tol) * alpha * beta)) return false;
    const float d = beta - alpha;
    const float r = sqrtf(fmaf(d, d, 4.0f * gamma * gamma));
    t = __fdividef(2.0f * gamma, d + copysignf(r, d));
    if (t == 0.0f) return false;
    const float x = fmaf(t, t, 1.0f);
    float y = rsqrtf(x);
    y = y * fmaf(-0.5f * x * y, y, 1.5f);
    c = y;
    s = c * t;
    return true;
}
__device__ __forceinline__ bool jacobi_rotation_scaled(double alpha, double beta, double gamma, double tol,
                                                       double small, double &c, double &s, double &t) {
    return jacobi_rotation_t<double>(alpha, beta, gamma, tol, small, c, s, t);
}

// ----------------------------------------------------------- warp kernel
// BUDGET: warm start with a sweep budget and cold restart (gbla_sgesvj_warm_batched);
// a separate instantiation, so the plain path keeps its register footprint.
template <typename T, int MR, bool BUDGET>
__global__ void __launch_bounds__(128, 1)
    k_gesvj_warp(int m, int n, const T *__restrict__ A, int64_t sA, T *__restrict__ S, int64_t sS,
                 T *__restrict__ Vt, int64_t sVt, T *__restrict__ U, int64_t sU, const T *__restrict__ V0,
                 int64_t sV0, T tol, int max_sweeps, int warm_budget, int *__restrict__ fallback_out,
                 int *__restrict__ info, int *__restrict__ sweeps_out, int batch) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mat = (int64_t)blockIdx.x * 4 + warp;
    if (mat >= batch) return;  // the whole warp leaves; no block barriers in this kernel
    const bool col = lane < n;
    T a[MR], v[32];
    const T *ag = A + mat * sA;
#pragma unroll
    for (int i = 0; i < MR; i++) a[i] = (col && i < m) ? ag[(int64_t)lane * m + i] : 0.f;
    if (V0) {
        // warm start: V = V0, A <- A V0 (column j of A V0 = sum_k a_k V0(k, j))
        const T *v0 = V0 + mat * sV0;
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = (col && i < n) ? v0[(int64_t)lane * n + i] : 0.f;
        T b[MR];
#pragma unroll
        for (int i = 0; i < MR; i++) b[i] = 0.f;
        for (int k = 0; k < n; k++) {
            T vk = 0.f;  // V0(k, lane)
#pragma unroll
            for (int i = 0; i < 32; i++)
                if (i == k) vk = v[i];
#pragma unroll
            for (int i = 0; i < MR; i++) b[i] = fma(shfl(a[i], k), vk, b[i]);
        }
#pragma unroll
        for (int i = 0; i < MR; i++) a[i] = col ? b[i] : 0.f;
    } else {
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = (col && i == lane) ? 1.f : 0.f;
    }

    T fro2 = 0.f;
#pragma unroll
    for (int i = 0; i < MR; i++) fro2 = fma(a[i], a[i], fro2);
    fro2 = warp_sum(fro2);
    // power-of-two scale (exact) bringing |A|_F^2 to [1, 4) (jacobi_rotation_scaled)
    const T psc = (fro2 > T(0) && isfinite(fro2)) ? pow2<T>(-(ilogb_of(fro2) >> 1)) : T(1);
#pragma unroll
    for (int i = 0; i < MR; i++) a[i] *= psc;
    const T small = mach_eps<T>() * mach_eps<T>() * (fro2 * psc * psc);
    tol = jacobi_tol<T>(tol, m);

    // warm start with a sweep budget: past it, restart cold from A (V = I)
    const bool budgeted = BUDGET && V0 && warm_budget > 0;
    int sweep = 0, total = 0, converged = 0, restarted = 0;
    int limit = budgeted ? warm_budget : max_sweeps;
    for (;;) {
    for (sweep = 1; sweep <= limit; sweep++) {
        total++;
        int rotated = 0;
        // this lane's column norm, recomputed once per sweep and carried through
        // the rotations (alpha - t gamma for column p, beta + t gamma for q)
        T own = 0.f;
#pragma unroll
        for (int i = 0; i < MR; i++) own = fma(a[i], a[i], own);
        // the pair ordering of the file header: in round r of level l, lane
        // st + i of a lower half meets lane mid + (i + r) mod cb
        for (int l = 0; ((n + (1 << l) - 1) >> l) >= 2; l++) {
        const int C = (((n + (1 << l) - 1) >> l) + 1) >> 1;
        const int b = col ? (((lane + 1) << l) - 1) / n : 0;
        const int st = (b * n) >> l, mid = ((2 * b + 1) * n) >> (l + 1), en = ((b + 1) * n) >> l;
        const int cb = mid - st > en - mid ? mid - st : en - mid;
        // per round: x = (lane - st + r) mod cb in the lower half, (lane - mid - r)
        // mod cb in the upper one; the partner is base + x if that column exists
        const bool lower = lane < mid;
        const int x0 = lower ? lane - st : lane - mid + cb, dx = lower ? 1 : -1;
        const int limit = col ? (lower ? en - mid : mid - st) : 0, base = lower ? mid : st;
        for (int r = 0; r < C; r++) {
            int x = x0 + dx * r;
            if (x >= cb) x -= cb;
            const int partner = (x < limit && r < cb) ? base + x : lane;
            const bool active = col && partner != lane;
            T gamma = 0.f;
            T o[MR];
#pragma unroll
            for (int i = 0; i < MR; i++) o[i] = shfl(a[i], partner);
            const T beta_o = shfl(own, partner);
            const bool low = lane < partner;  // this lane holds column p of the pair
#pragma unroll
            for (int i = 0; i < MR; i++) gamma = fma(low ? a[i] : o[i], low ? o[i] : a[i], gamma);
            T c = 1.f, s = 0.f, t = 0.f;
            const T ap = low ? own : beta_o, aq = low ? beta_o : own;
            bool rot = active && jacobi_rotation_scaled(ap, aq, gamma, tol, small, c, s, t);
            // a_p' = c a_p - s a_q ; a_q' = s a_p + c a_q
            const T cm = c, so = low ? -s : s;
            if (__any_sync(FULL, rot)) {  // V's partner column only when some pair of the warp rotates
                T ov[32];
#pragma unroll
                for (int i = 0; i < 32; i++) ov[i] = shfl(v[i], partner);
                if (rot) {
#pragma unroll
                    for (int i = 0; i < MR; i++) a[i] = fma(cm, a[i], so * o[i]);
#pragma unroll
                    for (int i = 0; i < 32; i++) v[i] = fma(cm, v[i], so * ov[i]);
                    own = low ? fma(-t, gamma, own) : fma(t, gamma, own);
                }
            }
            rotated |= rot;
        }
        }
        if (!__any_sync(FULL, rotated)) { converged = 1; break; }
    }
    if (converged || restarted || !budgeted) break;
    if constexpr (BUDGET) {
#pragma unroll
        for (int i = 0; i < MR; i++) a[i] = (col && i < m) ? ag[(int64_t)lane * m + i] * psc : 0.f;
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = (col && i == lane) ? 1.f : 0.f;
        restarted = 1;
        limit = max_sweeps;
    }
    }

    // ---- epilogue.  The rotated columns' norms drift by ~sqrt(#rotations) ulp;
    // sigma_j = |A v_j| / |v_j| from the original A is accurate to second order
    // in the error of v_j, so sigma is recomputed from A and V (row by row).
    // U takes the rotated columns themselves, which are orthogonal to the
    // rotation tolerance (A v_j / sigma_j would amplify v_j's error by 1/sigma_j).
    T nv2 = 0.f;
#pragma unroll
    for (int i = 0; i < 32; i++) nv2 = fma(v[i], v[i], nv2);
    const T inv_nv = nv2 > 0.f ? 1.f / sqrt(nv2) : 0.f;
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] *= inv_nv;
    T s2 = 0.f;
    for (int i = 0; i < m; i++) {
        T bi = 0.f;
#pragma unroll
        for (int k = 0; k < 32; k++)
            if (k < n) bi = fma(ag[(int64_t)k * m + i], v[k], bi);  // same address in every lane
        s2 = fma(bi, bi, s2);
    }
    T rot2 = 0.f;
#pragma unroll
    for (int i = 0; i < MR; i++) rot2 = fma(a[i], a[i], rot2);
    const T sigma = col ? sqrt(s2) : -1.f;
    int pos = 0;
    T smax = 0.f;
    for (int k = 0; k < n; k++) {
        T sk = shfl(sigma, k);
        smax = fmax(smax, sk);
        pos += (sk > sigma || (sk == sigma && k < lane)) ? 1 : 0;
    }
    int imax = 0;
    T vmax = -1.f;
#pragma unroll
    for (int i = 0; i < 32; i++)
        if (i < n && fabs(v[i]) > vmax) { vmax = fabs(v[i]); imax = i; }
    T vsel = 0.f;
#pragma unroll
    for (int i = 0; i < 32; i++)
        if (i == imax) vsel = v[i];
    const T sgn = vsel > 0.f ? -1.f : 1.f;
    const T thr = smax * (T)(m > n ? m : n) * mach_eps<T>();
    if (col) {
        S[mat * sS + pos] = sigma;
        T *vt = Vt + mat * sVt;
#pragma unroll
        for (int i = 0; i < 32; i++)
            if (i < n) vt[(int64_t)i * n + pos] = sgn * v[i];
    }
    if (U) {
        T *u = U + mat * sU;
        const T inv = (sigma > thr && rot2 > 0.f) ? sgn / sqrt(rot2) : 0.f;
        if (col && sigma > thr) {
#pragma unroll
            for (int i = 0; i < MR; i++)
                if (i < m) u[(int64_t)pos * m + i] = a[i] * inv;
        }
        int r = 0;
        for (int k = 0; k < n; k++) r += shfl(sigma, k) > thr ? 1 : 0;
        __syncwarp();
        // complete U: positions r..m-1
        int c = r, ncomp = 0;
        const T accept = T(0.5) * rsqrt((T)m);
        for (int e = 0; e < m && c < m; e++) {
            T w0 = lane == e ? 1.f : 0.f, w1 = lane + 32 == e ? 1.f : 0.f;
            for (int pass = 0; pass < 2; pass++) {
                for (int k = 0; k < c; k++) {
                    T u0 = lane < m ? u[(int64_t)k * m + lane] : 0.f;
                    T u1 = lane + 32 < m ? u[(int64_t)k * m + lane + 32] : 0.f;
                    T d = warp_sum(u0 * w0 + u1 * w1);
                    w0 = fma(-d, u0, w0);
                    w1 = fma(-d, u1, w1);
                }
            }
            T nw = sqrt(warp_sum(w0 * w0 + w1 * w1));
            if (nw > accept) {
                T sc = ((ncomp & 1) ? -1.f : 1.f) / nw;
                if (lane < m) u[(int64_t)c * m + lane] = w0 * sc;
                if (lane + 32 < m) u[(int64_t)c * m + lane + 32] = w1 * sc;
                __syncwarp();
                c++;
                ncomp++;
            }
        }
    }
    if (lane == 0) {
        if (info) info[mat] = converged ? 0 : 1;
        if (sweeps_out) sweeps_out[mat] = total;
        if (fallback_out) fallback_out[mat] = restarted;
    }
}

// ------------------------------------------------------------ CTA kernel
// One block per matrix: 32 column pairs x GL lanes per pair (GL = 4 or 8),
// rows split across the GL lanes; A (m x n) and V (n x n) in shared memory.
// Column strides are multiples of 32 words; a lane moves its rows of a
// column as 16-byte vectors (svj_ld / svj_st, conflict-free).  The pair
// ordering keeps one column of each pair (of A and of V) in the group's
// registers for a whole phase of rounds, so a round loads the partner column
// of A and, when the pair is rotated, stores it and loads and stores the
// partner column of V: half the shared-memory traffic of moving both columns,
// which bounds the kernel while most pairs rotate.  Column norms are cached
// (recomputed from the columns at the start of every sweep, updated by
// alpha - t gamma, beta + t gamma after a rotation), so a round computes one
// dot product per pair.

// Rows of one column held by lane gl of a GL-lane group (GL = 8 or 4), in
// 16-byte vectors: rows E v .. E v + E - 1 (E = 16 / sizeof(T) values per
// vector) for the vectors v = gl + GL s' (s' < CNT / E), where s' = s for
// even groups (sw = 0) and s ^ 1 for odd ones (sw = 1, GL = 4 only).  Column
// strides are multiples of 32 words, so with GL = 8 the group reads 128
// contiguous bytes per vector (one bank each) and the four groups of a warp
// (other columns) are served in separate phases; with GL = 4 the two groups
// that share a phase read opposite halves of the banks: conflict-free.
template <typename T, int CNT, int GL>
__device__ __forceinline__ void svj_ld(const T *col, int gl, int sw, T (&x)[CNT]) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int s = 0; s < CNT / 4; s++) {
            const float4 v = reinterpret_cast<const float4 *>(col)[gl + GL * (s ^ sw)];
            x[4 * s] = v.x; x[4 * s + 1] = v.y; x[4 * s + 2] = v.z; x[4 * s + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int s = 0; s < CNT / 2; s++) {
            const double2 v = reinterpret_cast<const double2 *>(col)[gl + GL * (s ^ sw)];
            x[2 * s] = v.x; x[2 * s + 1] = v.y;
        }
    }
}
template <typename T, int CNT, int GL>
__device__ __forceinline__ void svj_st(T *col, int gl, int sw, const T (&x)[CNT]) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int s = 0; s < CNT / 4; s++)
            reinterpret_cast<float4 *>(col)[gl + GL * (s ^ sw)] =
                make_float4(x[4 * s], x[4 * s + 1], x[4 * s + 2], x[4 * s + 3]);
    } else {
#pragma unroll
        for (int s = 0; s < CNT / 2; s++)
            reinterpret_cast<double2 *>(col)[gl + GL * (s ^ sw)] = make_double2(x[2 * s], x[2 * s + 1]);
    }
}

// Lanes per column pair: 4 for single precision up to 64 rows (16 rows a
// lane, one 128-thread block per matrix, four blocks per SM), otherwise 8
// (256 threads).  Fewer lanes per pair means fewer warp instructions per
// pair (the pair's indices, the reduction and the angle are computed once
// per group).  The register budgets keep the stationary and the moving
// column of A and of V in registers without spilling.
template <typename T, int MR>
constexpr int svj_group() { return (sizeof(T) == 4 && MR <= 64) ? 4 : 8; }
template <typename T, int MR>
constexpr int svj_min_blocks() {
    return sizeof(T) == 8 ? 2 : (svj_group<T, MR>() == 4 ? 4 : 2);
}

// MR, NR: row counts of A and V padded to 32, 64 or 128 (compile time).  The
// padding rows hold zeros, which every rotation maps to zeros, so the row
// loops need no bounds tests and unroll completely.  32 groups of GL lanes
// (one per column pair of a round).
template <typename T, int MR, int NR, int GL = svj_group<T, MR>()>
__global__ void __launch_bounds__(32 * GL, svj_min_blocks<T, MR>())
    k_gesvj_cta(int m, int n, const T *__restrict__ A, int64_t sA, T *__restrict__ S, int64_t sS,
                T *__restrict__ Vt, int64_t sVt, T *__restrict__ U, int64_t sU, const T *__restrict__ V0,
                int64_t sV0, T tol, int max_sweeps, int warm_budget, int *__restrict__ fallback_out,
                int *__restrict__ info, int *__restrict__ sweeps_out, int batch) {
    extern __shared__ __align__(16) unsigned char svsm_raw[];
    T *svsm = reinterpret_cast<T *>(svsm_raw);
    constexpr int lda = MR, ldv = NR;
    T *a = svsm;                      // n columns x lda
    T *v = a + (size_t)n * lda;       // n columns x ldv
    T *sig = v + (size_t)n * ldv;     // n
    T *rinv = sig + n;                // n: 1 / |rotated column j|
    T *nrm = rinv + n;                // n: cached |a_j|^2
    constexpr int THREADS = 32 * GL;
    const int tid = threadIdx.x, g = tid / GL, gl = tid % GL, sw = GL == 4 ? (g & 1) : 0;
    constexpr int MT = MR / GL, NT = NR / GL;  // rows of a column per lane

    for (int64_t mat = blockIdx.x; mat < batch; mat += gridDim.x) {
        const T *ag = A + mat * sA;
        for (int e = tid; e < MR * n; e += THREADS) {
            const int i = e % MR, j = e / MR;
            a[j * lda + i] = i < m ? ag[(int64_t)j * m + i] : T(0);
        }
        for (int e = tid; e < NR * n; e += THREADS) {
            const int i = e % NR, j = e / NR;
            v[j * ldv + i] = i >= n ? T(0) : V0 ? V0[mat * sV0 + (int64_t)j * n + i] : (i == j ? T(1) : T(0));
        }
        __syncthreads();
        if (V0) {
            // A <- A V0, column by column through registers (rows by thread)
            for (int i0 = 0; i0 < m; i0 += THREADS / 4) {
                // each thread: row i0 + tid % 64, columns j = tid / 64 + 4 t
                const int i = i0 + tid % (THREADS / 4);
                T acc[16];
                for (int t = 0; t < 16; t++) acc[t] = 0.f;
                if (i < m) {
                    for (int k = 0; k < n; k++) {
                        T aik = a[k * lda + i];
                        for (int t = 0; t < 16; t++) {
                            int j = tid / (THREADS / 4) + 4 * t;
                            if (j < n) acc[t] = fma(aik, v[j * ldv + k], acc[t]);
                        }
                    }
                }
                __syncthreads();
                if (i < m)
                    for (int t = 0; t < 16; t++) {
                        int j = tid / (THREADS / 4) + 4 * t;
                        if (j < n) a[j * lda + i] = acc[t];
                    }
                __syncthreads();
            }
        }
        // |A|_F^2 (rotations preserve it) -> threshold below which a column is zero
        if (tid < 32) {
            T f = 0.f;
            for (int j = 0; j < n; j++)
                for (int i = tid; i < m; i += 32) f = fma(a[j * lda + i], a[j * lda + i], f);
            f = warp_sum(f);
            if (tid == 0) sig[0] = f;
        }
        __syncthreads();
        // power-of-two scale (exact) bringing |A|_F^2 to [1, 4), so that the
        // squares in the rotation angle cannot overflow
        const T fro2 = sig[0];
        const T psc = (fro2 > T(0) && isfinite(fro2)) ? pow2<T>(-(ilogb_of(fro2) >> 1)) : T(1);
        if (psc != T(1))
            for (int e = tid; e < MR * n; e += THREADS) a[(e / MR) * lda + e % MR] *= psc;
        const T small = mach_eps<T>() * mach_eps<T>() * (fro2 * psc * psc);
        const T tol_eff = jacobi_tol<T>(tol, m);
        __syncthreads();
        const bool budgeted = V0 && warm_budget > 0;
        int sweep = 0, total = 0, converged = 0, restarted = 0;
        int limit = budgeted ? warm_budget : max_sweeps;
        for (;;) {
        for (sweep = 1; sweep <= limit; sweep++) {
            total++;
            int rotated = 0;
            // refresh the cached norms: group g takes columns g, g + 32.  The
            // trip count is the same for every lane (the group sum shuffles
            // across the whole warp); columns past n contribute nothing.
            for (int j0 = 0; j0 < n; j0 += THREADS / GL) {
                const int j = j0 + g;
                T f = 0.f;
                if (j < n) {
                    T x[MT];
                    svj_ld<T, MT, GL>(a + j * lda, gl, sw, x);
#pragma unroll
                    for (int t = 0; t < MT; t++) f = fma(x[t], x[t], f);
                }
                f = group_sum(f, GL);
                if (gl == 0 && j < n) nrm[j] = f;
            }
            __syncthreads();
            // Rounds (the ordering of the file header): level l splits the columns into 2^l blocks
            // [st, en) with halves [st, mid) and [mid, en); group g = (b, i)
            // (b = g / C, i = g % C) keeps column st + i of the lower half
            // (stationary, in registers for the whole level) and meets column
            // mid + (i + r) mod cb of the upper half in round r < cb, arriving
            // through shared memory.  The levels meet every pair once, in
            // n - 1 to n + 3 rounds (n <= 64), and a round moves one column of
            // A (and of V when rotated) per group instead of two.
            for (int l = 0; ((n + (1 << l) - 1) >> l) >= 2; l++) {
                const int C = (((n + (1 << l) - 1) >> l) + 1) >> 1;  // rounds of this level
                const int b = g / C, i = g - b * C;
                const int st = (b * n) >> l, mid = ((2 * b + 1) * n) >> (l + 1), en = ((b + 1) * n) >> l;
                const int cb = mid - st > en - mid ? mid - st : en - mid;
                const int sc = st + i;  // stationary column
                const bool s_ok = b < (1 << l) && i < mid - st;
                T sa[MT], sv[NT], s_nrm = T(0);
                if (s_ok) {
                    svj_ld<T, MT, GL>(a + sc * lda, gl, sw, sa);
                    svj_ld<T, NT, GL>(v + sc * ldv, gl, sw, sv);
                    s_nrm = nrm[sc];
                }
                bool s_dirty = false;
                for (int r = 0; r < C; r++) {
                    int mi = i + r;
                    if (mi >= cb) mi -= cb;
                    const int mc = mid + mi;  // moving column
                    const bool act = s_ok && r < cb && mc < en;
                    T gamma = T(0), g2 = T(0), beta = T(0);
                    T *am = a + (act ? mc : 0) * lda;
                    T xm[MT];
                    if (act) {
                        svj_ld<T, MT, GL>(am, gl, sw, xm);
                        T g3 = T(0), g4 = T(0);
#pragma unroll
                        for (int t = 0; t < MT; t += 4) {
                            gamma = fma(sa[t], xm[t], gamma);
                            g2 = fma(sa[t + 1], xm[t + 1], g2);
                            g3 = fma(sa[t + 2], xm[t + 2], g3);
                            g4 = fma(sa[t + 3], xm[t + 3], g4);
                        }
                        gamma = (gamma + g2) + (g3 + g4);
                        beta = nrm[mc];
                    }
                    gamma = group_sum(gamma, GL);
                    T c, sn, tn;
                    if (act && jacobi_rotation_scaled(s_nrm, beta, gamma, tol_eff, small, c, sn, tn)) {
                        rotated = 1;
                        s_dirty = true;
#pragma unroll
                        for (int t = 0; t < MT; t++) {
                            const T x = sa[t], y = xm[t];
                            sa[t] = fma(c, x, -sn * y);
                            xm[t] = fma(sn, x, c * y);
                        }
                        svj_st<T, MT, GL>(am, gl, sw, xm);
                        T *vm = v + mc * ldv;
                        T ym[NT];
                        svj_ld<T, NT, GL>(vm, gl, sw, ym);
#pragma unroll
                        for (int t = 0; t < NT; t++) {
                            const T x = sv[t], y = ym[t];
                            sv[t] = fma(c, x, -sn * y);
                            ym[t] = fma(sn, x, c * y);
                        }
                        svj_st<T, NT, GL>(vm, gl, sw, ym);
                        const T alpha = s_nrm;
                        s_nrm = fma(-tn, gamma, alpha);
                        if (gl == 0) nrm[mc] = fma(tn, gamma, beta);
                    }
                    __syncthreads();
                }
                // the stationary column goes back before the next phase regroups the players
                if (s_dirty) {
                    svj_st<T, MT, GL>(a + sc * lda, gl, sw, sa);
                    svj_st<T, NT, GL>(v + sc * ldv, gl, sw, sv);
                    if (gl == 0) nrm[sc] = s_nrm;
                }
                __syncthreads();
            }
            // block-wide OR in one barrier: every thread sees the same decision
            if (!__syncthreads_or(rotated)) { converged = 1; break; }
        }
        if (converged || restarted || !budgeted) break;
        // warm budget spent: restart cold from A (same power-of-two scale) with V = I
        for (int e = tid; e < MR * n; e += THREADS) {
            const int i = e % MR, j = e / MR;
            a[j * lda + i] = i < m ? ag[(int64_t)j * m + i] * psc : T(0);
        }
        for (int e = tid; e < NR * n; e += THREADS) {
            const int i = e % NR, j = e / NR;
            v[j * ldv + i] = (i == j) ? T(1) : T(0);
        }
        __syncthreads();
        restarted = 1;
        limit = max_sweeps;
        }
        // ---- epilogue: normalise V; sigma_j = |A v_j| from the original A (see
        // the warp kernel); U from the rotated columns, normalised
        for (int j = tid / 32; j < n; j += THREADS / 32) {
            T s2 = 0.f;
            for (int i = tid % 32; i < n; i += 32) s2 = fma(v[j * ldv + i], v[j * ldv + i], s2);
            s2 = warp_sum(s2);
            const T inv = s2 > 0.f ? 1.f / sqrt(s2) : 0.f;
            for (int i = tid % 32; i < n; i += 32) v[j * ldv + i] *= inv;
        }
        __syncthreads();
        for (int j = tid / 32; j < n; j += THREADS / 32) {
            T s2 = 0.f;
            for (int i = tid % 32; i < m; i += 32) {
                T b = 0.f;
                for (int k = 0; k < n; k++) b = fma(ag[(int64_t)k * m + i], v[j * ldv + k], b);
                s2 = fma(b, b, s2);
            }
            s2 = warp_sum(s2);
            T r2 = 0.f;
            for (int i = tid % 32; i < m; i += 32) r2 = fma(a[j * lda + i], a[j * lda + i], r2);
            r2 = warp_sum(r2);
            if (tid % 32 == 0) {
                sig[j] = sqrt(s2);
                rinv[j] = r2 > 0.f ? 1.f / sqrt(r2) : 0.f;
            }
        }
        __syncthreads();
        T smax = 0.f;
        for (int k = 0; k < n; k++) smax = fmax(smax, sig[k]);
        const T thr = smax * (T)(m > n ? m : n) * mach_eps<T>();
        for (int j = tid; j < n; j += THREADS) {
            int ps = 0;
            for (int k = 0; k < n; k++) ps += (sig[k] > sig[j] || (sig[k] == sig[j] && k < j)) ? 1 : 0;
            const T inv_rot = rinv[j];
            // sign: largest-magnitude entry of v_j made negative
            int imax = 0;
            T vmax = -1.f;
            for (int i = 0; i < n; i++)
                if (fabs(v[j * ldv + i]) > vmax) { vmax = fabs(v[j * ldv + i]); imax = i; }
            T sg = v[j * ldv + imax] > 0.f ? -1.f : 1.f;
            S[mat * sS + ps] = sig[j];
            for (int i = 0; i < n; i++) Vt[mat * sVt + (int64_t)i * n + ps] = sg * v[j * ldv + i];
            if (U && sig[j] > thr) {
                T inv = sg * inv_rot;
                for (int i = 0; i < m; i++) U[mat * sU + (int64_t)ps * m + i] = a[j * lda + i] * inv;
            }
        }
        __syncthreads();
        if (U && tid < 32) {
            // complete U (positions r..m-1) with warp 0, rows lane + 32 t
            T *u = U + mat * sU;
            int r = 0;
            for (int k = 0; k < n; k++) r += sig[k] > thr ? 1 : 0;
            int c = r, ncomp = 0;
            const T accept = T(0.5) * rsqrt((T)m);
            for (int e = 0; e < m && c < m; e++) {
                T w[4];
                for (int t = 0; t < 4; t++) w[t] = (tid + 32 * t == e) ? 1.f : 0.f;
                for (int pass = 0; pass < 2; pass++)
                    for (int k = 0; k < c; k++) {
                        T uk[4], d = 0.f;
                        for (int t = 0; t < 4; t++) {
                            int i = tid + 32 * t;
                            uk[t] = i < m ? u[(int64_t)k * m + i] : 0.f;
                            d = fma(uk[t], w[t], d);
                        }
                        d = warp_sum(d);
                        for (int t = 0; t < 4; t++) w[t] = fma(-d, uk[t], w[t]);
                    }
                T nw = 0.f;
                for (int t = 0; t < 4; t++) nw = fma(w[t], w[t], nw);
                nw = sqrt(warp_sum(nw));
                if (nw > accept) {
                    T sc = ((ncomp & 1) ? -1.f : 1.f) / nw;
                    for (int t = 0; t < 4; t++) {
                        int i = tid + 32 * t;
                        if (i < m) u[(int64_t)c * m + i] = w[t] * sc;
                    }
                    __syncwarp();
                    c++;
                    ncomp++;
                }
            }
        }
        if (tid == 0) {
            if (info) info[mat] = converged ? 0 : 1;
            if (sweeps_out) sweeps_out[mat] = total;
            if (fallback_out) fallback_out[mat] = restarted;
        }
        __syncthreads();
    }
}

// padded row count of the block kernel: 32, 64 or 128
static int svj_pad(int r) { return r <= 32 ? 32 : r <= 64 ? 64 : 128; }

template <typename T, int MR, int NR>
static gbla_status svj_cta_launch(int m, int n, const T *A, int64_t sA, T *S, int64_t sS, T *Vt, int64_t sVt, T *U,
                                  int64_t sU, const T *V0, int64_t sV0, T tol, int max_sweeps, int warm_budget,
                                  int *fallback, int *info, int *sweeps, int batch, size_t smem, cudaStream_t st) {
    constexpr int threads = 32 * svj_group<T, MR>();
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(k_gesvj_cta<T, MR, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return from_cuda(e);
    }
    const int64_t grid = persistent_grid(reinterpret_cast<const void *>(k_gesvj_cta<T, MR, NR>), threads, smem, batch);
    k_gesvj_cta<T, MR, NR><<<(unsigned)grid, threads, smem, st>>>(
        m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol, max_sweeps, warm_budget, fallback, info, sweeps, batch);
    return launch_status();
}

template <typename T>
static size_t svj_cta_smem(int m, int n) {
    return sizeof(T) * ((size_t)n * svj_pad(m) + (size_t)n * svj_pad(n) + 3 * (size_t)n) + 16;
}

// ---------------------------------------------------------------- rank
template <typename T>
__global__ void k_rank(int len, const T *__restrict__ S, int64_t sS, T eps, unsigned *__restrict__ rank, int batch) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= batch) return;
    unsigned c = 0;
    for (int i = lane; i < len; i += 32) c += S[(int64_t)warp * sS + i] > eps ? 1u : 0u;
    c = warp_sum(c);
    if (lane == 0) rank[warp] = c;
}

// ----------------------------------------------------------- null space
// From the SVD of A^T (n x m, U n x n, S of length m): nullity = n - rank;
// N gets U's columns rank..n-1 in its columns 0..nullity-1 (zero-padded);
// P = N N^T.  One block per matrix.
template <typename T>
__global__ void k_nullspace_finish(int n, int m, const T *__restrict__ Uall, const T *__restrict__ Sall, T eps,
                                   T *__restrict__ N, T *__restrict__ P, unsigned *__restrict__ nullity_out,
                                   int batch) {
    __shared__ int s_rank;
    for (int64_t mat = blockIdx.x; mat < batch; mat += gridDim.x) {
        if (threadIdx.x == 0) {
            // zero: below eps or below the working-precision noise of the SVD
            T smax = T(0);
            for (int i = 0; i < m; i++) smax = Sall[mat * m + i] > smax ? Sall[mat * m + i] : smax;
            T noise = smax * T(n) * (sizeof(T) == 4 ? T(FLT_EPSILON) : T(DBL_EPSILON));
            T thr = eps > noise ? eps : noise;
            int r = 0;
            for (int i = 0; i < m; i++) r += Sall[mat * m + i] > thr ? 1 : 0;
            s_rank = r;
        }
        __syncthreads();
        const int r = s_rank, nul = n - r;
        const T *u = Uall + mat * (int64_t)n * n;
        T *nn = N + mat * (int64_t)n * n;
        T *pp = P + mat * (int64_t)n * n;
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            int i = e % n, j = e / n;
            nn[e] = j < nul ? u[(int64_t)(r + j) * n + i] : T(0);
        }
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            int i = e % n, j = e / n;
            T acc = T(0);
            for (int k = 0; k < nul; k++) acc += u[(int64_t)(r + k) * n + i] * u[(int64_t)(r + k) * n + j];
            pp[e] = acc;
        }
        if (threadIdx.x == 0 && nullity_out) nullity_out[mat] = (unsigned)nul;
        __syncthreads();
    }
}

template <typename T>
static gbla_status svd_launch(int m, int n, const T *A, int64_t sA, T *S, int64_t sS, T *Vt, int64_t sVt, T *U,
                              int64_t sU, const T *V0, int64_t sV0, T tol, int max_sweeps, int *info, int *sweeps,
                              int batch, cudaStream_t st, int warm_budget = 0, int *fallback = nullptr) {
    if (m < 0 || n < 0 || batch < 0 || m < n || max_sweeps < 1 || !(tol > T(0))) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0) return GBLA_SUCCESS;
    if (!A || !S || !Vt || sA < (int64_t)m * n || sS < n || sVt < (int64_t)n * n) return GBLA_INVALID_VALUE;
    if (U && sU < (int64_t)m * m) return GBLA_INVALID_VALUE;
    if (V0 && sV0 < (int64_t)n * n) return GBLA_INVALID_VALUE;
    // the warp kernel keeps a column of A (MR rows) and of V in registers
    const int warp_m = sizeof(T) == 4 ? 64 : 32;
    if (n <= 32 && m <= warp_m) {
        const unsigned grid = (unsigned)((batch + 3) / 4);
        const bool budget = V0 && warm_budget > 0;
        if (m <= 32) {
            if (budget)
                k_gesvj_warp<T, 32, true><<<grid, 128, 0, st>>>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol,
                                                                max_sweeps, warm_budget, fallback, info, sweeps,
                                                                batch);
            else
                k_gesvj_warp<T, 32, false><<<grid, 128, 0, st>>>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol,
                                                                 max_sweeps, 0, fallback, info, sweeps, batch);
        } else if constexpr (sizeof(T) == 4) {
            if (budget)
                k_gesvj_warp<T, 64, true><<<grid, 128, 0, st>>>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol,
                                                                max_sweeps, warm_budget, fallback, info, sweeps,
                                                                batch);
            else
                k_gesvj_warp<T, 64, false><<<grid, 128, 0, st>>>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol,
                                                                 max_sweeps, 0, fallback, info, sweeps, batch);
        }
        return launch_status();
    }
    if (n <= 64 && m <= 128) {
        const size_t smem = svj_cta_smem<T>(m, n);
        const int mr = svj_pad(m), nr = svj_pad(n);
#define SVJ_LAUNCH(MRV, NRV)                                                                                      \
    if (mr == MRV && nr == NRV)                                                                                   \
        return svj_cta_launch<T, MRV, NRV>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol, max_sweeps,          \
                                           warm_budget, fallback, info, sweeps, batch, smem, st);
        SVJ_LAUNCH(32, 32)
        SVJ_LAUNCH(64, 32)
        SVJ_LAUNCH(128, 32)
        SVJ_LAUNCH(64, 64)
        SVJ_LAUNCH(128, 64)
#undef SVJ_LAUNCH
    }
    // wider or taller: one block per matrix, A in shared or global memory (no warm start)
    if (!V0 && n <= SVD_BIG_MAX_N)
        return svd_big_launch<T>(m, n, const_cast<T *>(A), sA, S, sS, Vt, sVt, U, sU, tol, max_sweeps, info, sweeps,
                                 batch, st);
    return GBLA_NOT_SUPPORTED;
}

template <typename T>
static gbla_status rank_launch(int len, const T *S, int64_t sS, T eps, unsigned *rank, int batch, cudaStream_t st) {
    if (len < 0 || batch < 0 || sS < len) return GBLA_INVALID_VALUE;
    if (batch == 0) return GBLA_SUCCESS;
    if (!rank || (len > 0 && !S)) return GBLA_INVALID_VALUE;
    k_rank<T><<<(unsigned)((batch * 32 + 255) / 256), 256, 0, st>>>(len, S, sS, eps, rank, batch);
    return launch_status();
}

// workspace layout for the null space: A^T (n x m), S (m), Vt (m x m), U (n x n) per matrix
static int64_t ns_elems(int m, int n) { return (int64_t)n * m + m + (int64_t)m * m + (int64_t)n * n; }

template <typename T>
static size_t ns_bytes(int m, int n, int batch) {
    if (m < 0 || n < 0 || batch < 0) return 0;
    return (size_t)(ns_elems(m, n) * batch) * sizeof(T) + 256;
}

template <typename T>
static gbla_status nullspace_launch(int m, int n, const T *A, int64_t sA, T *N, T *P, unsigned *nullity, T eps,
                                    int *info, void *workspace, size_t ws_bytes, int batch, cudaStream_t st) {
    if (m < 1 || n < 0 || m > n || batch < 0) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0) return GBLA_SUCCESS;
    if (!A || !N || !P || !workspace || sA < (int64_t)m * n) return GBLA_INVALID_VALUE;
    if (ws_bytes < ns_bytes<T>(m, n, batch)) return GBLA_WORKSPACE_TOO_SMALL;
    T *At = static_cast<T *>(workspace);
    T *S = At + (int64_t)n * m * batch;
    T *Vt = S + (int64_t)m * batch;
    T *U = Vt + (int64_t)m * m * batch;
    gbla_status s;
    if constexpr (sizeof(T) == 4) s = gbla_stranspose_batched(m, n, A, sA, At, (int64_t)n * m, batch, st);
    else s = gbla_dtranspose_batched(m, n, A, sA, At, (int64_t)n * m, batch, st);
    if (s != GBLA_SUCCESS) return s;
    // SVD of A^T (n x m, tall) with the full U (n x n), at working-precision tolerance
    s = svd_launch<T>(n, m, At, (int64_t)n * m, S, m, Vt, (int64_t)m * m, U, (int64_t)n * n, nullptr, 0,
                      sizeof(T) == 4 ? T(1e-7) : T(1e-15), 80, info, nullptr, batch, st);
    if (s != GBLA_SUCCESS) return s;
    int grid = batch < sm_count() * 4 ? batch : sm_count() * 4;
    k_nullspace_finish<T><<<grid, 256, 0, st>>>(n, m, U, S, eps, N, P, nullity, batch);
    return launch_status();
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_sgesvj_batched(int m, int n, float *A, int64_t sA, float *S, int64_t sS, float *Vt,
                                         int64_t sVt, float *U, int64_t sU, const float *V0, int64_t sV0, float tol,
                                         int max_sweeps, int *info, int *sweeps, int batch, cudaStream_t st) {
    return svd_launch<float>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol, max_sweeps, info, sweeps, batch, st);
}
GBLA_API gbla_status gbla_dgesvj_batched(int m, int n, double *A, int64_t sA, double *S, int64_t sS, double *Vt,
                                         int64_t sVt, double *U, int64_t sU, const double *V0, int64_t sV0, double tol,
                                         int max_sweeps, int *info, int *sweeps, int batch, cudaStream_t st) {
    return svd_launch<double>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol, max_sweeps, info, sweeps, batch, st);
}
GBLA_API gbla_status gbla_sgesvj_warm_batched(int m, int n, const float *A, int64_t sA, float *S, int64_t sS,
                                              float *Vt, int64_t sVt, float *U, int64_t sU, const float *V0,
                                              int64_t sV0, int warm_budget, float tol, int max_sweeps, int *info,
                                              int *sweeps, int *fallback, int batch, cudaStream_t st) {
    if (batch > 0 && n > 0 && (!V0 || warm_budget < 1)) return GBLA_INVALID_VALUE;
    return svd_launch<float>(m, n, A, sA, S, sS, Vt, sVt, U, sU, V0, sV0, tol, max_sweeps, info, sweeps, batch, st,
                             warm_budget, fallback);
}
GBLA_API gbla_status gbla_srank_batched(int len, const float *S, int64_t sS, float eps, unsigned *rank, int batch,
                                        cudaStream_t st) {
    return rank_launch<float>(len, S, sS, eps, rank, batch, st);
}
GBLA_API gbla_status gbla_drank_batched(int len, const double *S, int64_t sS, double eps, unsigned *rank, int batch,
                                        cudaStream_t st) {
    return rank_launch<double>(len, S, sS, eps, rank, batch, st);
}
GBLA_API size_t gbla_snullspace_workspace_bytes(int m, int n, int batch) { return ns_bytes<float>(m, n, batch); }
GBLA_API size_t gbla_dnullspace_workspace_bytes(int m, int n, int batch) { return ns_bytes<double>(m, n, batch); }
GBLA_API gbla_status gbla_snullspace_batched(int m, int n, const float *A, int64_t sA, float *N, float *P,
                                             unsigned *nullity, float eps, int *info, void *workspace,
                                             size_t ws_bytes, int batch, cudaStream_t st) {
    return nullspace_launch<float>(m, n, A, sA, N, P, nullity, eps, info, workspace, ws_bytes, batch, st);
}
GBLA_API gbla_status gbla_dnullspace_batched(int m, int n, const double *A, int64_t sA, double *N, double *P,
                                             unsigned *nullity, double eps, int *info, void *workspace,
                                             size_t ws_bytes, int batch, cudaStream_t st) {
    return nullspace_launch<double>(m, n, A, sA, N, P, nullity, eps, info, workspace, ws_bytes, batch, st);
}
