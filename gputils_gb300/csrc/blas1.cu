// blas1.cu -- HBM-bound helpers of the DTensor API: batched transpose, axpy,
// scal, row extraction and deterministic whole-buffer reductions.
#include <cfloat>
#include <mutex>
#include "common.cuh"

namespace gbla {

// ---------------------------------------------------------------- transpose
// One 32x32 tile per block, staged through shared memory (padded to avoid
// bank conflicts) so both the read of A and the write of A^T are coalesced.
template <typename T>
__global__ void __launch_bounds__(256) k_transpose(int m, int n, const T *__restrict__ A, int64_t sA,
                                                   T *__restrict__ At, int64_t sAt, int batch) {
    __shared__ T tile[32][33];
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    for (int b = blockIdx.z; b < batch; b += gridDim.z) {
        const T *a = A + b * sA;
        T *at = At + b * sAt;
        for (int jj = threadIdx.y; jj < 32; jj += 8) {
            int i = i0 + threadIdx.x, j = j0 + jj;
            if (i < m && j < n) tile[jj][threadIdx.x] = a[(int64_t)j * m + i];
        }
        __syncthreads();
        for (int ii = threadIdx.y; ii < 32; ii += 8) {
            int j = j0 + threadIdx.x, i = i0 + ii;  // At is n x m: element (j, i)
            if (i < m && j < n) at[(int64_t)i * n + j] = tile[threadIdx.x][ii];
        }
        __syncthreads();
    }
}

template <typename T>
static gbla_status transpose(int m, int n, const T *A, int64_t sA, T *At, int64_t sAt, int batch,
                             cudaStream_t st) {
    if (m < 0 || n < 0 || batch < 0) return GBLA_INVALID_VALUE;
    if ((int64_t)m * n == 0 || batch == 0) return GBLA_SUCCESS;
    if (!A || !At || sA < (int64_t)m * n || sAt < (int64_t)m * n) return GBLA_INVALID_VALUE;
    dim3 grid((n + 31) / 32, (m + 31) / 32, batch < 65535 ? batch : 65535);
    k_transpose<T><<<grid, dim3(32, 8), 0, st>>>(m, n, A, sA, At, sAt, batch);
    return launch_status();
}

// --------------------------------------------------------------- axpy/scal
template <typename T>
__global__ void k_axpy(int64_t len, T alpha, const T *__restrict__ x, T *__restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(alpha, x[i], y[i]);
}

template <typename T>
__global__ void k_scal(int64_t len, T alpha, T *__restrict__ x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= alpha;
}

static int stream_grid(int64_t len) {
    int64_t g = (len + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

template <typename T>
static gbla_status axpy(int64_t len, T alpha, const T *x, T *y, cudaStream_t st) {
    if (len < 0) return GBLA_INVALID_VALUE;
    if (len == 0) return GBLA_SUCCESS;
    if (!x || !y) return GBLA_INVALID_VALUE;
    k_axpy<T><<<stream_grid(len), 256, 0, st>>>(len, alpha, x, y);
    return launch_status();
}

template <typename T>
static gbla_status scal(int64_t len, T alpha, T *x, cudaStream_t st) {
    if (len < 0) return GBLA_INVALID_VALUE;
    if (len == 0) return GBLA_SUCCESS;
    if (!x) return GBLA_INVALID_VALUE;
    k_scal<T><<<stream_grid(len), 256, 0, st>>>(len, alpha, x);
    return launch_status();
}

// ---------------------------------------------------------------- copy rows
template <typename T>
__global__ void k_copy_rows(int m, int n, int r0, int nr, const T *__restrict__ A, T *__restrict__ out) {
    int64_t tot = (int64_t)nr * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(e % nr), j = (int)(e / nr);
        out[e] = A[(int64_t)j * m + r0 + i];
    }
}

template <typename T>
static gbla_status copy_rows(int m, int n, int r0, int nr, const T *A, T *out, cudaStream_t st) {
    if (m < 0 || n < 0 || nr < 0 || r0 < 0 || r0 + nr > m) return GBLA_INVALID_VALUE;
    if ((int64_t)nr * n == 0) return GBLA_SUCCESS;
    if (!A || !out) return GBLA_INVALID_VALUE;
    k_copy_rows<T><<<stream_grid((int64_t)nr * n), 256, 0, st>>>(m, n, r0, nr, A, out);
    return launch_status();
}

// ------------------------------------------------------------- Givens
// x_i <- c x_i + s y_i,  y_i <- c y_i - s x_i  (cublas<t>rot semantics); c and
// s come either by value or from device memory (cs != nullptr: c = cs[0],
// s = cs[1]) so a rotation computed on the device needs no host round trip.
template <typename T>
__global__ void k_rot(int64_t len, T *__restrict__ x, int64_t incx, T *__restrict__ y, int64_t incy, T c, T s,
                      const T *__restrict__ cdev, const T *__restrict__ sdev) {
    if (cdev) { c = *cdev; s = *sdev; }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
        T xv = x[i * incx], yv = y[i * incy];
        x[i * incx] = c * xv + s * yv;
        y[i * incy] = c * yv - s * xv;
    }
}

template <typename T>
static gbla_status rot(int64_t len, T *x, int64_t incx, T *y, int64_t incy, T c, T s, const T *cdev, const T *sdev,
                       cudaStream_t st) {
    if (len < 0 || incx < 1 || incy < 1) return GBLA_INVALID_VALUE;
    if (len == 0) return GBLA_SUCCESS;
    if (!x || !y || (cdev == nullptr) != (sdev == nullptr)) return GBLA_INVALID_VALUE;
    k_rot<T><<<stream_grid(len), 256, 0, st>>>(len, x, incx, y, incy, c, s, cdev, sdev);
    return launch_status();
}

// out[0] = 1 / hypot(a_ij, a_kj), out[1] = a_ij out[0], out[2] = a_kj out[0]:
// the rotation of rows i and k that zeroes a_kj (GivensAnnihilator).
template <typename T>
__global__ void k_givens_coeffs(const T *__restrict__ A, int64_t ld, int i, int k, int j, T *__restrict__ out) {
    const T xi = A[(int64_t)j * ld + i], xk = A[(int64_t)j * ld + k];
    const T r = rhypot(xi, xk);
    out[0] = r;
    out[1] = xi * r;
    out[2] = xk * r;
}

// ------------------------------------------------------- batched Givens
// Rotation of two strided vectors in each of `batch` problems, each with its
// own (c, s) read from device memory: x_b, y_b start at x + b stride, y + b
// stride; c_b = c[b cs_stride], s_b = s[b cs_stride].
template <typename T>
__global__ void k_rot_batched(int64_t len, T *__restrict__ x, int64_t incx, T *__restrict__ y, int64_t incy,
                              int64_t stride, const T *__restrict__ c, const T *__restrict__ s, int64_t cs_stride,
                              int64_t total) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = e / len, i = e % len;
        const T cb = c[b * cs_stride], sb = s[b * cs_stride];
        T *xp = x + b * stride + i * incx, *yp = y + b * stride + i * incy;
        const T xv = *xp, yv = *yp;
        *xp = cb * xv + sb * yv;
        *yp = cb * yv - sb * xv;
    }
}

// GivensAnnihilator::annihilate on every matrix of a batch in one launch: one
// warp per matrix reads A(i, j) and A(k, j), forms r = 1 / hypot, c = A(i, j) r
// and s = A(k, j) r (the reference's k_givensAnnihilateRHypot), then rotates
// rows i and k across all n columns (cublas<t>rot with c and -s = s), which
// zeroes A(k, j).  coeffs (nullable) receives (r, c, s) per matrix.
template <typename T>
__global__ void __launch_bounds__(256) k_givens_annihilate_batched(int m, int n, T *__restrict__ A, int64_t sA, int i,
                                                                   int k, int j, T *__restrict__ coeffs, int batch) {
    const int lane = threadIdx.x & 31;
    const int64_t mat = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (mat >= batch) return;  // whole warps leave together
    T *a = A + mat * sA;
    const T xij = a[(int64_t)j * m + i], xkj = a[(int64_t)j * m + k];
    const T r = rhypot(xij, xkj);
    const T c = xij * r, s = xkj * r;
    __syncwarp();  // every lane has read column j before any lane rotates it
    for (int col = lane; col < n; col += 32) {
        const T xv = a[(int64_t)col * m + i], yv = a[(int64_t)col * m + k];
        a[(int64_t)col * m + i] = c * xv + s * yv;
        a[(int64_t)col * m + k] = c * yv - s * xv;
    }
    if (coeffs && lane == 0) {
        coeffs[3 * mat] = r;
        coeffs[3 * mat + 1] = c;
        coeffs[3 * mat + 2] = s;
    }
}

template <typename T>
static gbla_status rot_batched(int64_t len, T *x, int64_t incx, T *y, int64_t incy, int64_t stride, const T *c,
                               const T *s, int64_t cs_stride, int batch, cudaStream_t st) {
    if (len < 0 || incx < 1 || incy < 1 || batch < 0 || stride < 0 || cs_stride < 0) return GBLA_INVALID_VALUE;
    if (len == 0 || batch == 0) return GBLA_SUCCESS;
    if (!x || !y || !c || !s) return GBLA_INVALID_VALUE;
    const int64_t total = len * batch;
    k_rot_batched<T><<<stream_grid(total), 256, 0, st>>>(len, x, incx, y, incy, stride, c, s, cs_stride, total);
    return launch_status();
}

template <typename T>
static gbla_status givens_annihilate_batched(int m, int n, T *A, int64_t sA, int i, int k, int j, T *coeffs, int batch,
                                             cudaStream_t st) {
    if (m < 0 || n < 0 || batch < 0 || sA < (int64_t)m * n) return GBLA_INVALID_VALUE;
    if (i < 0 || k < 0 || j < 0 || i >= m || k >= m || j >= n || i == k) return GBLA_INVALID_VALUE;
    if (batch == 0) return GBLA_SUCCESS;
    if (!A) return GBLA_INVALID_VALUE;
    const int64_t blocks = ((int64_t)batch * 32 + 255) / 256;
    k_givens_annihilate_batched<T><<<(unsigned)blocks, 256, 0, st>>>(m, n, A, sA, i, k, j, coeffs, batch);
    return launch_status();
}

// --------------------------------------------------------------- reductions
// Pass 1: a fixed number of blocks (depending only on len) each reduce a
// grid-strided slice into one partial; pass 2: one block reduces the
// partials in a fixed order.  The result is therefore bitwise reproducible.
enum RedOp { RED_DOT = 0, RED_ABS = 2, RED_AMAX = 3, RED_AMIN = 4 };
constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;

template <typename T, int OP>
__device__ __forceinline__ T red_identity() {
    if (OP == RED_AMAX) return T(0);
    if (OP == RED_AMIN) return T(INFINITY);
    return T(0);
}

template <typename T, int OP>
__device__ __forceinline__ T red_combine(T a, T b) {
    if (OP == RED_AMAX) return a > b ? a : (b == b ? b : a);
    if (OP == RED_AMIN) return a < b ? a : (b == b ? b : a);
    return a + b;
}

template <typename T, int OP>
__device__ __forceinline__ T block_reduce(T v) {
    __shared__ T sh[RED_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = red_combine<T, OP>(v, shfl_xor(v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < RED_THREADS / 32 ? sh[threadIdx.x] : red_identity<T, OP>();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = red_combine<T, OP>(v, shfl_xor(v, o));
    }
    return v;
}

template <typename T, int OP>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_pass1(int64_t len, const T *__restrict__ x,
                                                               const T *__restrict__ y, T *partials) {
    T acc = red_identity<T, OP>();
    for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * RED_THREADS) {
        T v = x[i];
        T t;
        if (OP == RED_DOT) t = v * y[i];
        else t = v < T(0) ? -v : v;
        acc = red_combine<T, OP>(acc, t);
    }
    acc = block_reduce<T, OP>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

template <typename T, int OP>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_pass2(int nparts, const T *partials, T *result) {
    T acc = red_identity<T, OP>();
    for (int i = threadIdx.x; i < nparts; i += RED_THREADS) acc = red_combine<T, OP>(acc, partials[i]);
    acc = block_reduce<T, OP>(acc);
    if (threadIdx.x == 0) *result = acc;
}

// ------------------------------------------------------------------ nrm2
// Euclidean norm without overflow or underflow, after Blue's three-
// accumulator method (J. L. Blue, "A portable Fortran program to find the
// Euclidean norm of a vector", ACM TOMS 4(1), 1978): entries of mid-range
// magnitude are squared as they are; large entries are scaled down by a power
// of two and small ones scaled up before squaring, each into its own sum, so
// no entry needs a division or a running rescale.  The thresholds leave every
// square (and any sum of up to 2^26 of them) inside the exponent range:
//   float : |x| > 2^50 -> (x 2^-76)^2, |x| < 2^-60 -> (x 2^80)^2
//   double: |x| > 2^480 -> (x 2^-600)^2, |x| < 2^-500 -> (x 2^600)^2
// Pass 1 writes the three sums of each block (partials[3 b + {0,1,2}] = small,
// mid, big); pass 2 adds them per class in a fixed order and combines the
// classes once.  Powers of two are exact, so the scaling adds no rounding.
template <typename T> struct Blue;
template <> struct Blue<float> {
    static constexpr float tbig = 0x1p50f, tsml = 0x1p-60f, sbig = 0x1p-76f, ssml = 0x1p80f;
    static constexpr float ibig = 0x1p76f, isml = 0x1p-80f;
};
template <> struct Blue<double> {
    static constexpr double tbig = 0x1p480, tsml = 0x1p-500, sbig = 0x1p-600, ssml = 0x1p600;
    static constexpr double ibig = 0x1p600, isml = 0x1p-600;
};

template <typename T>
__device__ __forceinline__ void blue_add(T v, T &sml, T &med, T &big) {
    const T a = fabs(v);
    if (a > Blue<T>::tbig) {
        const T s = a * Blue<T>::sbig;
        big = fma(s, s, big);
    } else if (a < Blue<T>::tsml) {
        const T s = a * Blue<T>::ssml;
        sml = fma(s, s, sml);
    } else {
        med = fma(a, a, med);
    }
}

template <typename T>
__device__ __forceinline__ T block_sum(T v) {
    return block_reduce<T, RED_DOT>(v);  // RED_DOT combines by addition
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_nrm2_pass1(int64_t len, const T *__restrict__ x, T *partials) {
    T sml = T(0), med = T(0), big = T(0);
    for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < len; i += (int64_t)gridDim.x * RED_THREADS)
        blue_add<T>(x[i], sml, med, big);
    sml = block_sum<T>(sml);
    __syncthreads();
    med = block_sum<T>(med);
    __syncthreads();
    big = block_sum<T>(big);
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x + 0] = sml;
        partials[3 * blockIdx.x + 1] = med;
        partials[3 * blockIdx.x + 2] = big;
    }
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_nrm2_pass2(int nparts, const T *partials, T *result) {
    T sml = T(0), med = T(0), big = T(0);
    for (int i = threadIdx.x; i < nparts; i += RED_THREADS) {
        sml += partials[3 * i + 0];
        med += partials[3 * i + 1];
        big += partials[3 * i + 2];
    }
    sml = block_sum<T>(sml);
    __syncthreads();
    med = block_sum<T>(med);
    __syncthreads();
    big = block_sum<T>(big);
    if (threadIdx.x == 0) {
        T r;
        if (big > T(0)) {
            // mid-range squares are negligible beside a big entry unless the
            // sum is finite: fold them in at the big scale (no overflow: the
            // scaled mid sum is tiny)
            r = Blue<T>::ibig * dev_sqrt<T>(big + (med * Blue<T>::sbig) * Blue<T>::sbig);
        } else if (med > T(0)) {
            // small squares folded in at the mid scale; they matter only when
            // the mid sum is itself near the small range
            r = dev_sqrt<T>(med + (sml * Blue<T>::isml) * Blue<T>::isml);
        } else {
            r = Blue<T>::isml * dev_sqrt<T>(sml);
        }
        *result = r;
    }
}

template <typename T, int OP>
static gbla_status reduce(int64_t len, const T *x, const T *y, T *result, void *ws, cudaStream_t st) {
    if (len < 0 || !result || !ws) return GBLA_INVALID_VALUE;
    if (len > 0 && (!x || (OP == RED_DOT && !y))) return GBLA_INVALID_VALUE;
    int64_t nb = (len + RED_THREADS * 4 - 1) / (RED_THREADS * 4);
    if (nb < 1) nb = 1;
    if (nb > RED_MAX_BLOCKS) nb = RED_MAX_BLOCKS;
    T *parts = reinterpret_cast<T *>(ws);
    k_reduce_pass1<T, OP><<<(int)nb, RED_THREADS, 0, st>>>(len, x, y, parts);
    gbla_status s = launch_status();
    if (s != GBLA_SUCCESS) return s;
    k_reduce_pass2<T, OP><<<1, RED_THREADS, 0, st>>>((int)nb, parts, result);
    return launch_status();
}

template <typename T>
static gbla_status nrm2(int64_t len, const T *x, T *result, void *ws, cudaStream_t st) {
    if (len < 0 || !result || !ws) return GBLA_INVALID_VALUE;
    if (len > 0 && !x) return GBLA_INVALID_VALUE;
    int64_t nb = (len + RED_THREADS * 4 - 1) / (RED_THREADS * 4);
    if (nb < 1) nb = 1;
    if (nb > RED_MAX_BLOCKS) nb = RED_MAX_BLOCKS;
    T *parts = reinterpret_cast<T *>(ws);
    k_nrm2_pass1<T><<<(int)nb, RED_THREADS, 0, st>>>(len, x, parts);
    gbla_status s = launch_status();
    if (s != GBLA_SUCCESS) return s;
    k_nrm2_pass2<T><<<1, RED_THREADS, 0, st>>>((int)nb, parts, result);
    return launch_status();
}

// Pass-1 block count (= partial sums) of reduce() for len elements; used by
// gbla_sdot_noalloc so that it launches exactly what gbla_sdot launches.
static int red_blocks(int64_t len) {
    int64_t nb = (len + RED_THREADS * 4 - 1) / (RED_THREADS * 4);
    if (nb < 1) nb = 1;
    if (nb > RED_MAX_BLOCKS) nb = RED_MAX_BLOCKS;
    return (int)nb;
}

// ------------------------------------------------ allocation-free dot product
// gbla_sdot_noalloc keeps the pass-1 partial sums of the float dot product in
// this fixed device array instead of a caller workspace.  It holds the most
// partial sums any length needs (RED_MAX_BLOCKS floats, 4 KB) and stays
// resident on every device that loads the library until the process exits.
// Host code may not use the symbol itself as a device address: its address is
// fetched once per device with cudaGetSymbolAddress (dot_scratch_address).
constexpr int NOALLOC_DOT_PARTIALS = RED_MAX_BLOCKS;
static __device__ __align__(256) float g_dot_scratch[NOALLOC_DOT_PARTIALS];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_dot_scratch_mu;
struct ScratchAddr {
    float *addr;
    unsigned long long ctx_id;  // context the address belongs to (0: none looked up)
};
static ScratchAddr g_dot_scratch_addr[NOALLOC_MAX_DEVICES] = {};

// Unique ID of the calling thread's current CUDA context, 0 if none is current
// or the driver cannot tell.  A device reset (cudaDeviceReset) destroys the
// primary context, and the next runtime call creates a new one, with a new ID,
// into which the library's module -- and g_dot_scratch -- is loaded afresh.
// The driver entry points come through the runtime, so the library does not
// link libcuda.
static unsigned long long current_context_id() {
    using GetCurrent = int (*)(void **);
    using GetId = int (*)(void *, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    if (!get_current || !get_id) return 0;
    void *ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return 0;
    unsigned long long id = 0;
    return get_id(ctx, &id) == 0 ? id : 0;
}

// Device address of g_dot_scratch on the current device.  Looked up with
// cudaGetSymbolAddress on the first call for each device (with that device
// current) and cached together with the ID of the context it belongs to; a
// call in another context of that device (after a device reset) looks it up
// again instead of using an address of a destroyed context.
static gbla_status dot_scratch_address(float **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return from_cuda(e);
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return GBLA_NOT_SUPPORTED;
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lock(g_dot_scratch_mu);
    ScratchAddr &c = g_dot_scratch_addr[dev];
    if (!c.addr || ctx == 0 || c.ctx_id != ctx) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_dot_scratch);
        if (e != cudaSuccess) return from_cuda(e);
        c.addr = static_cast<float *>(p);
        c.ctx_id = current_context_id();  // the lookup has made the device's context current
    }
    *out = c.addr;
    return GBLA_SUCCESS;
}

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_stranspose_batched(int m, int n, const float *A, int64_t sA, float *At, int64_t sAt,
                                             int batch, cudaStream_t st) {
    return transpose<float>(m, n, A, sA, At, sAt, batch, st);
}
GBLA_API gbla_status gbla_dtranspose_batched(int m, int n, const double *A, int64_t sA, double *At,
                                             int64_t sAt, int batch, cudaStream_t st) {
    return transpose<double>(m, n, A, sA, At, sAt, batch, st);
}
GBLA_API gbla_status gbla_saxpy(int64_t len, float alpha, const float *x, float *y, cudaStream_t st) {
    return axpy<float>(len, alpha, x, y, st);
}
GBLA_API gbla_status gbla_daxpy(int64_t len, double alpha, const double *x, double *y, cudaStream_t st) {
    return axpy<double>(len, alpha, x, y, st);
}
GBLA_API gbla_status gbla_sscal(int64_t len, float alpha, float *x, cudaStream_t st) {
    return scal<float>(len, alpha, x, st);
}
GBLA_API gbla_status gbla_dscal(int64_t len, double alpha, double *x, cudaStream_t st) {
    return scal<double>(len, alpha, x, st);
}
GBLA_API gbla_status gbla_scopy_rows(int m, int n, int r0, int nr, const float *A, float *out, cudaStream_t st) {
    return copy_rows<float>(m, n, r0, nr, A, out, st);
}
GBLA_API gbla_status gbla_dcopy_rows(int m, int n, int r0, int nr, const double *A, double *out,
                                     cudaStream_t st) {
    return copy_rows<double>(m, n, r0, nr, A, out, st);
}
// three partial sums per pass-1 block (nrm2), in the widest type
GBLA_API size_t gbla_reduce_workspace_bytes(void) { return 3 * RED_MAX_BLOCKS * sizeof(double); }

#define GBLA_RED(NAME, T, OP, HASY)                                                                    \
    GBLA_API gbla_status NAME(int64_t len, const T *x, HASY T *result, void *ws, cudaStream_t st) {   \
        return reduce<T, OP>(len, x, YARG, result, ws, st);                                            \
    }
#define YARG nullptr
GBLA_RED(gbla_sasum, float, RED_ABS, )
GBLA_RED(gbla_dasum, double, RED_ABS, )
GBLA_RED(gbla_samax, float, RED_AMAX, )
GBLA_RED(gbla_damax, double, RED_AMAX, )
GBLA_RED(gbla_samin, float, RED_AMIN, )
GBLA_RED(gbla_damin, double, RED_AMIN, )
#undef YARG
GBLA_API gbla_status gbla_snrm2(int64_t len, const float *x, float *result, void *ws, cudaStream_t st) {
    return nrm2<float>(len, x, result, ws, st);
}
GBLA_API gbla_status gbla_dnrm2(int64_t len, const double *x, double *result, void *ws, cudaStream_t st) {
    return nrm2<double>(len, x, result, ws, st);
}
GBLA_API gbla_status gbla_sdot(int64_t len, const float *x, const float *y, float *result, void *ws,
                               cudaStream_t st) {
    return reduce<float, RED_DOT>(len, x, y, result, ws, st);
}
GBLA_API gbla_status gbla_ddot(int64_t len, const double *x, const double *y, double *result, void *ws,
                               cudaStream_t st) {
    return reduce<double, RED_DOT>(len, x, y, result, ws, st);
}

// Same kernels and block count as gbla_sdot (so the same result bits); the
// partial sums go to g_dot_scratch.  Pass 1 writes every partial that pass 2
// reads, so nothing in the array has to start at zero.  Calls that overlap on
// the GPU share the array and race.
GBLA_API gbla_status gbla_sdot_noalloc(int64_t len, const float *x, const float *y, float *result, cudaStream_t st) {
    if (len < 0 || !result) return GBLA_INVALID_VALUE;
    if (len > 0 && (!x || !y)) return GBLA_INVALID_VALUE;
    const int nb = red_blocks(len);
    if (nb > NOALLOC_DOT_PARTIALS) return GBLA_WORKSPACE_TOO_SMALL;  // more partials than the array holds
    float *parts = nullptr;
    gbla_status s = dot_scratch_address(&parts);
    if (s != GBLA_SUCCESS) return s;
    k_reduce_pass1<float, RED_DOT><<<nb, RED_THREADS, 0, st>>>(len, x, y, parts);
    s = launch_status();
    if (s != GBLA_SUCCESS) return s;
    k_reduce_pass2<float, RED_DOT><<<1, RED_THREADS, 0, st>>>(nb, parts, result);
    return launch_status();
}

GBLA_API gbla_status gbla_srot(int64_t len, float *x, int64_t incx, float *y, int64_t incy, float c, float s,
                               cudaStream_t st) {
    return rot<float>(len, x, incx, y, incy, c, s, nullptr, nullptr, st);
}
GBLA_API gbla_status gbla_drot(int64_t len, double *x, int64_t incx, double *y, int64_t incy, double c, double s,
                               cudaStream_t st) {
    return rot<double>(len, x, incx, y, incy, c, s, nullptr, nullptr, st);
}
GBLA_API gbla_status gbla_srot_dev(int64_t len, float *x, int64_t incx, float *y, int64_t incy, const float *c,
                                   const float *s, cudaStream_t st) {
    if (!c || !s) return GBLA_INVALID_VALUE;
    return rot<float>(len, x, incx, y, incy, 0.f, 0.f, c, s, st);
}
GBLA_API gbla_status gbla_drot_dev(int64_t len, double *x, int64_t incx, double *y, int64_t incy, const double *c,
                                   const double *s, cudaStream_t st) {
    if (!c || !s) return GBLA_INVALID_VALUE;
    return rot<double>(len, x, incx, y, incy, 0.0, 0.0, c, s, st);
}
GBLA_API gbla_status gbla_srot_batched(int64_t len, float *x, int64_t incx, float *y, int64_t incy, int64_t stride,
                                       const float *c, const float *s, int64_t cs_stride, int batch, cudaStream_t st) {
    return rot_batched<float>(len, x, incx, y, incy, stride, c, s, cs_stride, batch, st);
}
GBLA_API gbla_status gbla_drot_batched(int64_t len, double *x, int64_t incx, double *y, int64_t incy, int64_t stride,
                                       const double *c, const double *s, int64_t cs_stride, int batch,
                                       cudaStream_t st) {
    return rot_batched<double>(len, x, incx, y, incy, stride, c, s, cs_stride, batch, st);
}
GBLA_API gbla_status gbla_sgivens_annihilate_batched(int m, int n, float *A, int64_t sA, int i, int k, int j,
                                                     float *coeffs, int batch, cudaStream_t st) {
    return givens_annihilate_batched<float>(m, n, A, sA, i, k, j, coeffs, batch, st);
}
GBLA_API gbla_status gbla_dgivens_annihilate_batched(int m, int n, double *A, int64_t sA, int i, int k, int j,
                                                     double *coeffs, int batch, cudaStream_t st) {
    return givens_annihilate_batched<double>(m, n, A, sA, i, k, j, coeffs, batch, st);
}
GBLA_API gbla_status gbla_sgivens_coeffs(const float *A, int64_t ld, int i, int k, int j, float *out,
                                         cudaStream_t st) {
    if (!A || !out || i < 0 || k < 0 || j < 0 || i >= ld || k >= ld) return GBLA_INVALID_VALUE;
    k_givens_coeffs<float><<<1, 1, 0, st>>>(A, ld, i, k, j, out);
    return launch_status();
}
GBLA_API gbla_status gbla_dgivens_coeffs(const double *A, int64_t ld, int i, int k, int j, double *out,
                                         cudaStream_t st) {
    if (!A || !out || i < 0 || k < 0 || j < 0 || i >= ld || k >= ld) return GBLA_INVALID_VALUE;
    k_givens_coeffs<double><<<1, 1, 0, st>>>(A, ld, i, k, j, out);
    return launch_status();
}
