// chol_ragged.cu -- one call that factors and solves a ragged batch of SPD
// systems of mixed sizes (1 <= n <= 128, any nrhs), with iterative refinement.
//
// The reference has no ragged API: a mixed batch is one
// CholeskyBatchFactoriser per size and one potrs per right-hand-side column
// (include/tensor.cuh:2100-2197).  Here a host-built plan sorts the systems:
//   * n <= 32  : three size classes (n <= 8, 16, 32); each class runs the
//                lane-row kernel (NB lanes per system, rows in registers,
//                shuffles only).  Within a warp the loop bounds are the warp's
//                largest n / nrhs; smaller systems are padded with the
//                identity, which leaves their factor and solution unchanged.
//   * n > 32   : one block per system, shared-memory factor, one warp per
//                right-hand side; blocks are issued largest system first.
// The two families run on a forked stream pair (graph-capturable fork/join).
//
// Precision: the factorisation and the triangular solves run in FP32; each
// refinement step recomputes r = b - A x from the original, full symmetric A
// (lower and upper triangles) in extended precision -- double-FP32 for float
// data, FP64 for double data -- and adds the FP32 correction.
#include <algorithm>
#include <vector>
#include "chol_common.cuh"
#include "xprec.cuh"

struct RaggedSys {
    int64_t a_off, b_off;
    int n, nrhs, orig, pad;
};

struct gbla_ragged_plan {
    int device = -1;
    int count = 0;
    int first[4] = {0, 0, 0, 0};   // classes: NB 8, NB 16, NB 32, large
    int num[4] = {0, 0, 0, 0};
    int max_n_large = 0;
    RaggedSys *d_sys = nullptr;
    cudaStream_t aux = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

namespace gbla {

constexpr int RG_LARGE_THREADS = 256;
constexpr int RG_LARGE_WARPS = RG_LARGE_THREADS / 32;

// ------------------------------------------------------------ small systems
template <typename T, int NB>
__global__ void __launch_bounds__(128, 1)
    k_ragged_small(const RaggedSys *__restrict__ sys, int first, int count, const T *__restrict__ A_in,
                   T *__restrict__ A, T *__restrict__ B, int *__restrict__ info, int refine) {
    constexpr int GPW = 32 / NB;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane / NB, r = lane % NB;
    const int local = (blockIdx.x * 4 + warp) * GPW + g;
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
template <typename T>
__host__ __device__ inline size_t ragged_large_smem(int nmax) {
    const int ld = cta_ld(nmax);
    // float factor (n x ld) + float dinv (n) + float work (8 x n) + T x (8 x n)
    return sizeof(float) * ((size_t)nmax * ld + nmax + (size_t)RG_LARGE_WARPS * nmax) +
           sizeof(T) * (size_t)RG_LARGE_WARPS * nmax + 64;
}

template <typename T>
__global__ void __launch_bounds__(RG_LARGE_THREADS, 1)
    k_ragged_large(const RaggedSys *__restrict__ sys, int first, int nmax, const T *__restrict__ A_in,
                   T *__restrict__ A, T *__restrict__ B, int *__restrict__ info, int refine) {
    extern __shared__ __align__(16) unsigned char rsm[];
    const RaggedSys s = sys[first + blockIdx.x];
    const int n = s.n, nrhs = s.nrhs, ld = cta_ld(n);
    const int ldmax = cta_ld(nmax);
    float *a = reinterpret_cast<float *>(rsm);
    float *dinv = a + (size_t)nmax * ldmax;
    float *work = dinv + nmax;
    T *xs = reinterpret_cast<T *>(work + (size_t)RG_LARGE_WARPS * nmax);
    __shared__ int s_fail;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const T *ag = A_in + s.a_off;

    for (int j = warp; j < n; j += RG_LARGE_WARPS)
        for (int i = j + lane; i < n; i += 32) a[(int64_t)j * ld + i] = (float)ag[(int64_t)j * n + i];
    if (threadIdx.x == 0) s_fail = 0;
    __syncthreads();
    // right-looking factorisation, one barrier per column (as in the uniform kernel)
    for (int k = 0; k < n; k++) {
        if (warp == k % RG_LARGE_WARPS) {
            __syncwarp();
            const float d = a[(int64_t)k * ld + k];
            if (!(d > 0.f) && lane == 0 && s_fail == 0) s_fail = k + 1;
            const float l = sqrtf(d), il = 1.f / l;
            for (int i = k + 1 + lane; i < n; i += 32) a[(int64_t)k * ld + i] *= il;
            if (lane == 0) { a[(int64_t)k * ld + k] = l; dinv[k] = il; }
        }
        __syncthreads();
        const int j0 = k + 1 + ((warp - (k + 1) % RG_LARGE_WARPS) + RG_LARGE_WARPS) % RG_LARGE_WARPS;
        for (int j = j0; j < n; j += RG_LARGE_WARPS) {
            const float ljk = a[(int64_t)k * ld + j];
            for (int i = j + lane; i < n; i += 32) a[(int64_t)j * ld + i] -= a[(int64_t)k * ld + i] * ljk;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && info) info[s.orig] = s_fail;

    T *bg = B + s.b_off;
    float *w = work + (size_t)warp * nmax;
    T *x = xs + (size_t)warp * nmax;
    for (int c = warp; c < nrhs; c += RG_LARGE_WARPS) {
        const T *bc = bg + (int64_t)c * n;
        for (int i = lane; i < n; i += 32) w[i] = (float)bc[i];
        __syncwarp();
        cta_solve_col<float>(a, ld, dinv, w, n, lane);
        for (int i = lane; i < n; i += 32) x[i] = (T)w[i];
        __syncwarp();
        for (int it = 0; it < refine; it++) {
            // r = b - A x with the full symmetric A; rows lane + 32 t
            if constexpr (sizeof(T) == 4) {
                ff acc[4];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int i = lane + 32 * t;
                    acc[t].h = i < n ? (float)bc[i] : 0.f;
                    acc[t].l = 0.f;
                }
                for (int j = 0; j < n; j++) {
                    const float xj = (float)x[j];
#pragma unroll
                    for (int t = 0; t < 4; t++) {
                        const int i = lane + 32 * t;
                        if (i < n) ff_fma(acc[t], -(float)ag[(int64_t)j * n + i], xj, 0.f);
                    }
                }
                __syncwarp();
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int i = lane + 32 * t;
                    if (i < n) w[i] = acc[t].h + acc[t].l;
                }
            } else {
                double acc[4];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int i = lane + 32 * t;
                    acc[t] = i < n ? (double)bc[i] : 0.0;
                }
                for (int j = 0; j < n; j++) {
                    const double xj = (double)x[j];
#pragma unroll
                    for (int t = 0; t < 4; t++) {
                        const int i = lane + 32 * t;
                        if (i < n) acc[t] = fma(-(double)ag[(int64_t)j * n + i], xj, acc[t]);
                    }
                }
                __syncwarp();
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int i = lane + 32 * t;
                    if (i < n) w[i] = (float)acc[t];
                }
            }
            __syncwarp();
            cta_solve_col<float>(a, ld, dinv, w, n, lane);
            for (int i = lane; i < n; i += 32) x[i] = x[i] + (T)w[i];
            __syncwarp();
        }
        T *bo = bg + (int64_t)c * n;
        for (int i = lane; i < n; i += 32) bo[i] = x[i];
        __syncwarp();
    }
    // L (lower triangle, FP32 factor) back in place, once every warp has
    // finished reading the original A for its residuals
    __syncthreads();
    T *aw = A + s.a_off;
    for (int j = warp; j < n; j += RG_LARGE_WARPS)
        for (int i = j + lane; i < n; i += 32) aw[(int64_t)j * n + i] = (T)a[(int64_t)j * ld + i];
}

template <typename T>
static gbla_status ragged_launch(const gbla_ragged_plan *p, T *A, T *B, int *info, int refine, cudaStream_t st) {
    if (!p || refine < 0) return GBLA_INVALID_VALUE;
    if (p->count == 0) return GBLA_SUCCESS;
    if (!A || !B) return GBLA_INVALID_VALUE;
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != p->device) return GBLA_INVALID_VALUE;
    cudaError_t e;
    const bool fork = p->num[3] > 0 && (p->num[0] + p->num[1] + p->num[2]) > 0;
    cudaStream_t small_st = fork ? p->aux : st;
    if (fork) {
        if ((e = cudaEventRecord(p->fork, st)) != cudaSuccess) return from_cuda(e);
        if ((e = cudaStreamWaitEvent(p->aux, p->fork, 0)) != cudaSuccess) return from_cuda(e);
    }
    if (p->num[3] > 0) {
        const size_t smem = ragged_large_smem<T>(p->max_n_large);
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(k_ragged_large<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return from_cuda(e);
        }
        k_ragged_large<T><<<p->num[3], RG_LARGE_THREADS, smem, st>>>(p->d_sys, p->first[3], p->max_n_large, A, A, B,
                                                                      info, refine);
        gbla_status s = launch_status();
        if (s != GBLA_SUCCESS) return s;
    }
    const int gpw[3] = {4, 2, 1};
    for (int c = 0; c < 3; c++) {
        if (p->num[c] == 0) continue;
        const unsigned grid = (unsigned)((p->num[c] + 4 * gpw[c] - 1) / (4 * gpw[c]));
        if (c == 0)
            k_ragged_small<T, 8><<<grid, 128, 0, small_st>>>(p->d_sys, p->first[c], p->num[c], A, A, B, info, refine);
        else if (c == 1)
            k_ragged_small<T, 16><<<grid, 128, 0, small_st>>>(p->d_sys, p->first[c], p->num[c], A, A, B, info, refine);
        else
            k_ragged_small<T, 32><<<grid, 128, 0, small_st>>>(p->d_sys, p->first[c], p->num[c], A, A, B, info, refine);
        gbla_status s = launch_status();
        if (s != GBLA_SUCCESS) return s;
    }
    if (fork) {
        if ((e = cudaEventRecord(p->join, p->aux)) != cudaSuccess) return from_cuda(e);
        if ((e = cudaStreamWaitEvent(st, p->join, 0)) != cudaSuccess) return from_cuda(e);
    }
    return GBLA_SUCCESS;
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
    auto *p = new gbla_ragged_plan();
    p->count = count;
    for (int i = 0; i < count; i++) p->num[cls(v[i].n)]++;
    p->first[0] = 0;
    for (int c = 1; c < 4; c++) p->first[c] = p->first[c - 1] + p->num[c - 1];
    p->max_n_large = p->num[3] > 0 ? v[p->first[3]].n : 0;
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess && count > 0) e = cudaMalloc(&p->d_sys, sizeof(RaggedSys) * (size_t)count);
    if (e == cudaSuccess && count > 0)
        e = cudaMemcpy(p->d_sys, v.data(), sizeof(RaggedSys) * (size_t)count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (p->d_sys) cudaFree(p->d_sys);
        if (p->aux) cudaStreamDestroy(p->aux);
        if (p->fork) cudaEventDestroy(p->fork);
        if (p->join) cudaEventDestroy(p->join);
        delete p;
        return from_cuda(e);
    }
    *plan = p;
    return GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_ragged_plan_destroy(gbla_ragged_plan *p) {
    if (!p) return GBLA_SUCCESS;
    cudaError_t e = cudaSuccess;
    if (p->aux) e = cudaStreamSynchronize(p->aux);
    if (p->d_sys) cudaFree(p->d_sys);
    if (p->aux) cudaStreamDestroy(p->aux);
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->join) cudaEventDestroy(p->join);
    delete p;
    return from_cuda(e);
}

GBLA_API gbla_status gbla_sposv_ragged(const gbla_ragged_plan *plan, float *A, float *B, int *info, int refine_iters,
                                       cudaStream_t st) {
    return ragged_launch<float>(plan, A, B, info, refine_iters, st);
}

GBLA_API gbla_status gbla_dposv_ragged(const gbla_ragged_plan *plan, double *A, double *B, int *info,
                                       int refine_iters, cudaStream_t st) {
    return ragged_launch<double>(plan, A, B, info, refine_iters, st);
}
