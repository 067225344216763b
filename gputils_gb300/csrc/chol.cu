// chol.cu -- batched Cholesky factor / solve / fused factor+solve+refine.
//
// Two kernel shapes, chosen by n:
//  * n <= 32  : "lane-row" kernel.  A group of NB lanes (NB = 8, 16 or 32)
//               owns one matrix, lane r holds row r in registers; the
//               right-looking factorisation and both triangular solves run
//               with warp shuffles only (no shared memory, no barriers).
//               32/NB matrices per warp, 4 warps per block.
//  * n <= 128+: "CTA" kernel.  One block (8 warps) per matrix, the matrix in
//               shared memory with an odd leading dimension; one barrier per
//               column (the owner warp of column k+1 finishes it while the
//               other warps still update), each right-hand side solved by
//               its own warp with shuffle broadcasts.
// Refinement (posv) recomputes r = b - A x from the lower triangle of the
// original A, which stays untouched in global memory until L is stored.
#include "common.cuh"
#include "chol_common.cuh"

namespace gbla {


// residual accumulation type of the refinement
template <typename T> struct ResT { using type = double; };

// y_r = (A x)_r for symmetric A given by its lower triangle in global memory.
template <typename T, int NB, typename R>
__device__ __forceinline__ R lr_symv_lower(const T *__restrict__ a, int n, int r, bool rowok, R x) {
    R acc = R(0);
#pragma unroll 4
    for (int j = 0; j < n; j++) {
        R xj = shfl(x, j, NB);
        R aij = (rowok && r >= j) ? R(a[(int64_t)j * n + r]) : R(0);
        acc += aij * xj;                           // lower part incl. diagonal
        R up = (r > j) ? aij * x : R(0);           // A(j, r) x_r for r > j
        up = group_sum(up, NB);
        if (r == j) acc += up;
    }
    return acc;
}

template <typename T, int NB>
__global__ void __launch_bounds__(128, 1) k_chol_lanerow(int n, int nrhs, T *__restrict__ A, int64_t sA,
                                                      T *__restrict__ B, int64_t sB, int *__restrict__ info,
                                                      int mode, int refine, int batch) {
    using R = typename ResT<T>::type;
    constexpr int GPW = 32 / NB;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane / NB, r = lane % NB;
    const int64_t mat = ((int64_t)blockIdx.x * 4 + warp) * GPW + g;
    const bool act = mat < batch;
    const bool rowok = act && r < n;
    T *a_g = A + (act ? mat : 0) * sA;
    // launched with programmatic stream serialization: let the next kernel
    // begin launching, and wait for the previous one before reading memory
    asm volatile("griddepcontrol.launch_dependents;");
    asm volatile("griddepcontrol.wait;" ::: "memory");

    T a[NB];
#pragma unroll
    for (int j = 0; j < NB; j++) {
        bool ld = rowok && j < n && j <= r;
        a[j] = ld ? a_g[(int64_t)j * n + r] : T(r == j ? 1 : 0);
    }
    T dinv = T(1);
    int fail = 0;
    if (mode & CH_FACTOR) {
        lr_factor<T, NB>(a, dinv, fail, n, r);
        if (act && r == 0 && info) info[mat] = fail;
    } else {
#pragma unroll
        for (int j = 0; j < NB; j++)
            if (j == r) dinv = T(1) / a[j];
    }
    if (mode & CH_SOLVE) {
        T *b_g = B + (act ? mat : 0) * sB;
        // a stored factor (solve-only call): also read it by columns, so the
        // transposed substitution needs no reductions
        T at[NB];
        if (!(mode & CH_FACTOR)) {
#pragma unroll
            for (int k = 0; k < NB; k++) at[k] = (rowok && k < n && k >= r) ? a_g[(int64_t)r * n + k] : T(0);
        }
        for (int c = 0; c < nrhs; c++) {
            T b = rowok ? b_g[(int64_t)c * n + r] : T(0);
            T x = (mode & CH_FACTOR) ? lr_solve<T, NB>(a, dinv, b, n, r) : lr_solve_cols<T, NB>(a, at, dinv, b, n, r);
            if ((mode & CH_FACTOR) && refine > 0) {
                R xr = R(x);
                for (int it = 0; it < refine; it++) {
                    R ax = lr_symv_lower<T, NB, R>(a_g, n, r, rowok, xr);
                    T res = rowok ? T(R(b) - ax) : T(0);
                    T d = lr_solve<T, NB>(a, dinv, res, n, r);
                    xr += R(d);
                }
                x = T(xr);
            }
            if (rowok) b_g[(int64_t)c * n + r] = x;
        }
    }
    if ((mode & CH_FACTOR) && rowok) {
#pragma unroll
        for (int j = 0; j < NB; j++)
            if (j < n && j <= r) a_g[(int64_t)j * n + r] = a[j];
    }
}

// ------------------------------------------------------------------ CTA kernel
// Per-warp solve columns of the CTA kernel: x, plus a residual column when
// refinement runs on n > 128 (the n <= 128 refinement keeps it in registers).
__host__ __device__ inline int cta_xcols(int n, int refine) { return (refine > 0 && n > 128) ? 2 : 1; }

// SMEM: the lower triangle is worked on in shared memory (odd leading
// dimension); otherwise (n beyond shared memory) in place in A, leading
// dimension n -- the factor overwrites A in any case, and without a copy of
// the original there is no refinement (the launcher refuses it).
template <typename T, bool SMEM>
__global__ void __launch_bounds__(CTA_THREADS, 1) k_chol_cta(int n, int nrhs, T *__restrict__ A, int64_t sA,
                                                          T *__restrict__ B, int64_t sB, int *__restrict__ info,
                                                          int mode, int refine, int batch) {
    using R = typename ResT<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *as = reinterpret_cast<T *>(smem_raw);
    const int ld = SMEM ? cta_ld(n) : n;
    const int xcols = cta_xcols(n, refine);
    T *xs = as + (SMEM ? (size_t)n * ld : 0);
    T *dinv = xs + (size_t)n * CTA_RHS_CHUNK * xcols;
    __shared__ int s_fail;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    for (int64_t mat = blockIdx.x; mat < batch; mat += gridDim.x) {
        T *a_g = A + mat * sA;
        T *a = SMEM ? as : a_g;
        // lower triangle -> shared memory (warp per column, lanes along rows)
        if (SMEM)
            for (int j = warp; j < n; j += CTA_WARPS)
                for (int i = j + lane; i < n; i += 32) a[(int64_t)j * ld + i] = a_g[(int64_t)j * n + i];
        if (threadIdx.x == 0) s_fail = 0;
        __syncthreads();

        if (mode & CH_FACTOR) {
            for (int k = 0; k < n; k++) {
                if (warp == k % CTA_WARPS) {
                    __syncwarp();
                    T d = a[(int64_t)k * ld + k];
                    if (!(d > T(0)) && lane == 0 && s_fail == 0) s_fail = k + 1;
                    T l = dev_sqrt<T>(d);
                    T il = T(1) / l;
                    for (int i = k + 1 + lane; i < n; i += 32) a[(int64_t)k * ld + i] *= il;
                    if (lane == 0) { a[(int64_t)k * ld + k] = l; dinv[k] = il; }
                }
                __syncthreads();
                // update own columns j > k (column k+1 first: it is next step's pivot)
                int j0 = k + 1 + ((warp - (k + 1) % CTA_WARPS) + CTA_WARPS) % CTA_WARPS;
                for (int j = j0; j < n; j += CTA_WARPS) {
                    T ljk = a[(int64_t)k * ld + j];
                    for (int i = j + lane; i < n; i += 32) a[(int64_t)j * ld + i] -= a[(int64_t)k * ld + i] * ljk;
                }
            }
            __syncthreads();
            if (threadIdx.x == 0 && info) info[mat] = s_fail;
        } else {
            for (int k = threadIdx.x; k < n; k += CTA_THREADS) dinv[k] = T(1) / a[(int64_t)k * ld + k];
            __syncthreads();
        }

        if (mode & CH_SOLVE) {
            T *b_g = B + mat * sB;
            for (int c0 = 0; c0 < nrhs; c0 += CTA_RHS_CHUNK) {
                int c = c0 + warp;
                if (c < nrhs) {
                    T *x = xs + (size_t)warp * n * xcols;
                    for (int i = lane; i < n; i += 32) x[i] = b_g[(int64_t)c * n + i];
                    __syncwarp();
                    cta_solve_col<T>(a, ld, dinv, x, n, lane);
                    if (SMEM && (mode & CH_FACTOR) && refine > 0 && n > 128) {
                        // any n: r = b - A x row by row from the original lower
                        // triangle (A(i, j) = A(j, i) above it), in R precision
                        T *d = x + n;
                        for (int it = 0; it < refine; it++) {
                            for (int i = lane; i < n; i += 32) {
                                R acc = R(b_g[(int64_t)c * n + i]);
                                for (int j = 0; j < n; j++) {
                                    const T aij = i >= j ? a_g[(int64_t)j * n + i] : a_g[(int64_t)i * n + j];
                                    acc -= R(aij) * R(x[j]);
                                }
                                d[i] = T(acc);
                            }
                            __syncwarp();
                            cta_solve_col<T>(a, ld, dinv, d, n, lane);
                            for (int i = lane; i < n; i += 32) x[i] += d[i];
                            __syncwarp();
                        }
                    } else if (SMEM && (mode & CH_FACTOR) && refine > 0) {
                        // x is kept in T; corrections come from an R-precision residual.
                        for (int it = 0; it < refine; it++) {
                            // r = b - A x (A symmetric, lower triangle of the original in global)
                            // each lane accumulates rows i = lane + 32 s
                            R acc[4] = {R(0), R(0), R(0), R(0)};
                            for (int j = 0; j < n; j++) {
                                R xj = R(x[j]);
                                R up = R(0);
#pragma unroll
                                for (int s = 0; s < 4; s++) {
                                    int i = lane + 32 * s;
                                    if (i < n && i >= j) {
                                        R aij = R(a_g[(int64_t)j * n + i]);
                                        acc[s] += aij * xj;
                                        if (i > j) up += aij * R(x[i]);
                                    }
                                }
                                up = warp_sum(up);
#pragma unroll
                                for (int s = 0; s < 4; s++)
                                    if (lane == (j & 31) && (j >> 5) == s) acc[s] += up;
                            }
                            __syncwarp();
                            T *d = x;  // reuse: store residual in a scratch column after x
                            T rv[4];
#pragma unroll
                            for (int s = 0; s < 4; s++) {
                                int i = lane + 32 * s;
                                rv[s] = i < n ? T(R(b_g[(int64_t)c * n + i]) - acc[s]) : T(0);
                            }
                            // keep x in registers while the residual is solved in place
                            T xv[4];
#pragma unroll
                            for (int s = 0; s < 4; s++) {
                                int i = lane + 32 * s;
                                xv[s] = i < n ? x[i] : T(0);
                            }
                            __syncwarp();
#pragma unroll
                            for (int s = 0; s < 4; s++) {
                                int i = lane + 32 * s;
                                if (i < n) d[i] = rv[s];
                            }
                            __syncwarp();
                            cta_solve_col<T>(a, ld, dinv, d, n, lane);
#pragma unroll
                            for (int s = 0; s < 4; s++) {
                                int i = lane + 32 * s;
                                if (i < n) x[i] = xv[s] + d[i];
                            }
                            __syncwarp();
                        }
                    }
                    for (int i = lane; i < n; i += 32) b_g[(int64_t)c * n + i] = x[i];
                }
            }
        }
        __syncthreads();
        if (SMEM && (mode & CH_FACTOR)) {
            for (int j = warp; j < n; j += CTA_WARPS)
                for (int i = j + lane; i < n; i += 32) a_g[(int64_t)j * n + i] = a[(int64_t)j * ld + i];
        }
        __syncthreads();
    }
}

// shared memory of the CTA kernel: matrix (SMEM only), solve columns, 1 / L_kk
template <typename T>
static size_t chol_cta_smem(int n, int refine, bool smem_matrix) {
    return sizeof(T) * ((smem_matrix ? (size_t)n * cta_ld(n) : 0) + (size_t)n * CTA_RHS_CHUNK * cta_xcols(n, refine) +
                        (size_t)n) + 16;
}
constexpr size_t CHOL_SMEM_MAX = 226 * 1024;  // below the 227 KB opt-in (room for static shared memory)

template <typename T>
static gbla_status chol_launch(int n, int nrhs, T *A, int64_t sA, T *B, int64_t sB, int *info, int mode,
                               int refine, int batch, cudaStream_t st) {
    if (n < 0 || batch < 0 || nrhs < 0 || refine < 0) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0) return GBLA_SUCCESS;
    if (!A || sA < (int64_t)n * n) return GBLA_INVALID_VALUE;
    if ((mode & CH_SOLVE) && (!B || sB < (int64_t)n * nrhs)) return GBLA_INVALID_VALUE;
    if ((mode & CH_SOLVE) && nrhs == 0 && !(mode & CH_FACTOR)) return GBLA_SUCCESS;
    if (n <= 32) {
        int nb = n <= 8 ? 8 : (n <= 16 ? 16 : 32);
        int mpb = 4 * (32 / nb);
        int64_t grid = (batch + mpb - 1) / mpb;
        if (grid > 0x7fffffff) return GBLA_INVALID_VALUE;
        // programmatic dependent launch: the kernel may start while the
        // previous kernel on the stream drains; it waits for it (and its
        // memory) before touching global memory (griddepcontrol.wait)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3(128);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaError_t e;
        if (nb == 8)
            e = cudaLaunchKernelEx(&cfg, k_chol_lanerow<T, 8>, n, nrhs, A, sA, B, sB, info, mode, refine, batch);
        else if (nb == 16)
            e = cudaLaunchKernelEx(&cfg, k_chol_lanerow<T, 16>, n, nrhs, A, sA, B, sB, info, mode, refine, batch);
        else
            e = cudaLaunchKernelEx(&cfg, k_chol_lanerow<T, 32>, n, nrhs, A, sA, B, sB, info, mode, refine, batch);
        if (e != cudaSuccess) return from_cuda(e);
        return launch_status();
    }
    const bool fits = chol_cta_smem<T>(n, refine, true) <= CHOL_SMEM_MAX;
    // beyond shared memory the factor is computed in place in A: the original
    // A is gone, so there is nothing to refine against
    if (!fits && refine > 0 && (mode & CH_FACTOR) && (mode & CH_SOLVE)) return GBLA_NOT_SUPPORTED;
    const size_t smem = chol_cta_smem<T>(n, refine, fits);
    if (smem > CHOL_SMEM_MAX) return GBLA_NOT_SUPPORTED;  // the solve columns alone do not fit
    auto go = [&](auto kern) -> gbla_status {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return from_cuda(e);
        }
        const int64_t grid = persistent_grid(reinterpret_cast<const void *>(kern), CTA_THREADS, smem, batch);
        kern<<<(unsigned)grid, CTA_THREADS, smem, st>>>(n, nrhs, A, sA, B, sB, info, mode, refine, batch);
        return launch_status();
    };
    return fits ? go(k_chol_cta<T, true>) : go(k_chol_cta<T, false>);
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_spotrf_batched(int n, float *A, int64_t sA, int *info, int batch, cudaStream_t st) {
    return chol_launch<float>(n, 0, A, sA, nullptr, 0, info, CH_FACTOR, 0, batch, st);
}
GBLA_API gbla_status gbla_dpotrf_batched(int n, double *A, int64_t sA, int *info, int batch, cudaStream_t st) {
    return chol_launch<double>(n, 0, A, sA, nullptr, 0, info, CH_FACTOR, 0, batch, st);
}
GBLA_API gbla_status gbla_spotrs_batched(int n, int nrhs, const float *L, int64_t sL, float *B, int64_t sB,
                                         int batch, cudaStream_t st) {
    return chol_launch<float>(n, nrhs, const_cast<float *>(L), sL, B, sB, nullptr, CH_SOLVE, 0, batch, st);
}
GBLA_API gbla_status gbla_dpotrs_batched(int n, int nrhs, const double *L, int64_t sL, double *B, int64_t sB,
                                         int batch, cudaStream_t st) {
    return chol_launch<double>(n, nrhs, const_cast<double *>(L), sL, B, sB, nullptr, CH_SOLVE, 0, batch, st);
}
GBLA_API gbla_status gbla_sposv_batched(int n, int nrhs, float *A, int64_t sA, float *B, int64_t sB, int *info,
                                        int refine, int batch, cudaStream_t st) {
    return chol_launch<float>(n, nrhs, A, sA, B, sB, info, CH_FACTOR | CH_SOLVE, refine, batch, st);
}
GBLA_API gbla_status gbla_dposv_batched(int n, int nrhs, double *A, int64_t sA, double *B, int64_t sB,
                                        int *info, int refine, int batch, cudaStream_t st) {
    return chol_launch<double>(n, nrhs, A, sA, B, sB, info, CH_FACTOR | CH_SOLVE, refine, batch, st);
}
