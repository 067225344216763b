/*
 * gbla.h -- C ABI of libgbla.so, the GB300 (sm_103a) batched small-matrix
 * linear-algebra library behind the GPUtils-compatible tensor.cuh.
 *
 * Every entry point replaces one cuBLAS / cuSOLVER call (or a host loop of
 * them) made by GPUtils' include/tensor.cuh; the comment above each one cites
 * the reference call site it replaces.  The functions take plain device
 * pointers, sizes and batch strides (in elements), never pointer arrays:
 * DTensor keeps its matrices back to back, so base pointer + stride covers
 * every case the reference builds, including axis-2 slices.
 *
 * Conventions
 *  - Matrices are column-major with leading dimension = number of rows.
 *  - All calls are asynchronous on the given stream and allocate nothing;
 *    reductions that need scratch take a caller-provided workspace.  The
 *    exceptions are objects made at set-up time (ragged plans, stream
 *    pipelines, the warm-start network), which own their device memory.
 *  - Errors are returned as gbla_status; nothing is thrown or printed and the
 *    process is never terminated.  Numerical failures are reported per matrix
 *    through device `info` arrays with cuSOLVER's meaning (0 = success).
 *  - Pointer arguments documented as "nullable" may be NULL.
 */
#ifndef GBLA_H
#define GBLA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without requiring the CUDA headers (same typedef as CUDA's). */
struct CUstream_st;
typedef struct CUstream_st *cudaStream_t;

typedef enum gbla_status {
    GBLA_SUCCESS = 0,
    GBLA_INVALID_VALUE = 1,    /* a size, stride or pointer argument is invalid */
    GBLA_NOT_SUPPORTED = 2,    /* valid request outside what this library implements */
    GBLA_CUDA_ERROR = 3,       /* a CUDA runtime call or kernel launch failed */
    GBLA_WORKSPACE_TOO_SMALL = 4
} gbla_status;

/* Precision schedule for single-precision GEMM. */
typedef enum gbla_gemm_mode {
    GBLA_GEMM_AUTO = 0,   /* tensor-core split path where the shape allows it, else FP32 FFMA */
    GBLA_GEMM_FP32 = 1,   /* plain FP32 fused multiply-add on the CUDA cores */
    GBLA_GEMM_BF16X6 = 2  /* operands split into three BF16 terms, six tcgen05 products,
                             FP32 accumulation in tensor memory */
} gbla_gemm_mode;

/* Human-readable name of a status code. */
const char *gbla_status_string(gbla_status s);
/* Library version, major*10000 + minor*100 + patch. */
int gbla_version(void);
/* Last CUDA runtime error code seen by the library (0 if none). */
int gbla_last_cuda_error(void);
/* Bit mask of device-side bounded waits that ran out since the previous call
 * (bit 0: tensor-core GEMM mbarrier wait).  Reading clears it; -1 if the
 * flags could not be read.  Synchronises the current device. */
int gbla_device_error_flags(void);

/* ------------------------------------------------------------------ GEMM */
/* C_i <- alpha * A_i * B_i + beta * C_i for i < batch.  A_i is m x k,
 * B_i is k x n, C_i is m x n.  C must not overlap A or B.
 * Replaces cublas<t>gemmBatched / cublas<t>gemm in DTensor::addAB
 * (include/tensor.cuh:1286-1338). */
gbla_status gbla_sgemm_batched(int m, int n, int k, float alpha, const float *A, int64_t strideA,
                               const float *B, int64_t strideB, float beta, float *C,
                               int64_t strideC, int batch, gbla_gemm_mode mode, cudaStream_t stream);
gbla_status gbla_dgemm_batched(int m, int n, int k, double alpha, const double *A, int64_t strideA,
                               const double *B, int64_t strideB, double beta, double *C,
                               int64_t strideC, int batch, cudaStream_t stream);

/* -------------------------------------------------------------- Cholesky */
/* In-place lower Cholesky A_i = L_i L_i^T of n x n matrices.  The strictly
 * upper triangle is not touched.  info[i] = 0 on success, j if the leading
 * minor of order j is not positive definite.
 * Replaces cusolverDn<t>potrfBatched (include/tensor.cuh:2135-2159) and
 * cusolverDn<t>potrf (include/tensor.cuh:1742-1761).  Any n: n <= 32 one
 * group of lanes per matrix in registers; larger n one block per matrix, the
 * matrix in shared memory when it fits (n up to ~230 float / ~160 double),
 * else factored in place in A (n up to ~6400 float / ~3200 double, where the
 * block's solve columns still fit in shared memory). */
gbla_status gbla_spotrf_batched(int n, float *A, int64_t strideA, int *info, int batch,
                                cudaStream_t stream);
gbla_status gbla_dpotrf_batched(int n, double *A, int64_t strideA, int *info, int batch,
                                cudaStream_t stream);

/* In-place lower Cholesky of ONE large n x n FP32 matrix (column stride
 * lda >= n) on the whole GPU: right-looking blocked factorisation with
 * 128-column panels -- the diagonal block by one thread block, the panel
 * below it by n / 64 blocks, and the trailing update A22 -= L21 L21^T on the
 * tensor cores (tcgen05; L21 split exactly into three BF16 parts, the six
 * largest of the nine products accumulated in FP32).  The strictly upper
 * triangle is not touched; *info as gbla_spotrf_batched (set to 0 first).
 * Any n >= 0; the workspace (gbla_spotrf_large_workspace_bytes, 6 KB per
 * row, none for n <= 128) holds two sets of the BF16 operands (the update of
 * the rest of the matrix runs on a side stream, overlapping the next panel;
 * the side stream and its events are made on a thread's first call on a
 * device, so make that call before capturing a CUDA graph).  Replaces cusolverDnSpotrf
 * (include/tensor.cuh:1742-1761: CholeskyFactoriser::factorise) for the sizes
 * where gbla_spotrf_batched with batch = 1 would leave all but one SM idle. */
size_t gbla_spotrf_large_workspace_bytes(int n);
gbla_status gbla_spotrf_large(int n, float *A, int64_t lda, int *info, void *workspace,
                              size_t workspace_bytes, cudaStream_t stream);

/* Solve L L^T X = B in place for ONE large FP32 lower factor L (column stride
 * lda >= n) and nrhs columns of B (column stride ldb >= n), in 128-row
 * blocks: each diagonal block solved by one thread block (a warp per
 * right-hand side), the rows below it (forward) or above it (backward)
 * updated by n / 128 thread blocks, a thread per row.  No workspace.
 * Replaces cusolverDnSpotrs (include/tensor.cuh:1775-1783:
 * CholeskyFactoriser<float>::solve) for the sizes where gbla_spotrs_batched
 * with batch = 1 runs on one thread block. */
gbla_status gbla_spotrs_large(int n, int nrhs, const float *L, int64_t lda, float *B, int64_t ldb,
                              cudaStream_t stream);

/* Solve L_i L_i^T X_i = B_i in place (B_i is n x nrhs) with the lower factor
 * in L_i.  Replaces cusolverDn<t>potrsBatched (include/tensor.cuh:2161-2197)
 * and cusolverDn<t>potrs (include/tensor.cuh:1763-1783); nrhs >= 1 (the
 * reference supports nrhs = 1 only).  Sizes as gbla_spotrf_batched. */
gbla_status gbla_spotrs_batched(int n, int nrhs, const float *L, int64_t strideL, float *B,
                                int64_t strideB, int batch, cudaStream_t stream);
gbla_status gbla_dpotrs_batched(int n, int nrhs, const double *L, int64_t strideL, double *B,
                                int64_t strideB, int batch, cudaStream_t stream);

/* Fused factor + solve + iterative refinement: one pass that leaves L_i in
 * A_i and X_i in B_i.  refine_iters refinement steps use an extended-
 * precision residual B_i - A_i X_i computed from the original A_i.  Equivalent
 * to CholeskyBatchFactoriser::factorise() followed by solve()
 * (include/tensor.cuh:2135-2197) for any nrhs.  Sizes as gbla_spotrf_batched;
 * refinement needs the matrix in shared memory (n up to ~230 float / ~160
 * double: the original stays in A meanwhile) and returns GBLA_NOT_SUPPORTED
 * beyond it (refine_iters = 0 works for every size). */
gbla_status gbla_sposv_batched(int n, int nrhs, float *A, int64_t strideA, float *B,
                               int64_t strideB, int *info, int refine_iters, int batch,
                               cudaStream_t stream);
gbla_status gbla_dposv_batched(int n, int nrhs, double *A, int64_t strideA, double *B,
                               int64_t strideB, int *info, int refine_iters, int batch,
                               cudaStream_t stream);

/* Ragged batches: SPD systems of mixed size in one call.  System i has its
 * n_i x n_i matrix at A + a_offsets[i] and its n_i x nrhs_i right-hand sides
 * at B + b_offsets[i] (element offsets, column-major, 1 <= n_i <= 128).
 * The plan sorts the systems (size class, then largest first) and cuts them
 * into tasks once; a call is then ONE persistent kernel launch whose blocks
 * take tasks from a device queue.  The plan owns small device tables and the
 * queue counter, so create it at set-up time (it allocates and synchronises),
 * and do not run calls of one plan concurrently (two host threads, or two
 * streams whose calls overlap on the GPU): they share the queue.  No
 * reference counterpart: GPUtils needs one CholeskyBatchFactoriser per size
 * and one potrs per column (include/tensor.cuh:2100-2197). */
typedef struct gbla_ragged_plan gbla_ragged_plan;
gbla_status gbla_ragged_plan_create(const int64_t *a_offsets, const int64_t *b_offsets, const int *n,
                                    const int *nrhs, int count, gbla_ragged_plan **plan);
gbla_status gbla_ragged_plan_destroy(gbla_ragged_plan *plan);

/* Launch configuration of a plan: threads per block (128, 256, 512 with 128
 * registers a thread, or 768 with 80) and the most systems with n > 32 that
 * one block factors at once (1, 2, 4, 8; at most threads / 64), each with
 * threads / 32 / count warps and its own
 * shared-memory slot (sized for the group's largest system; the block's
 * shared memory -- and so the blocks per SM -- is that many slots of the
 * plan's largest system).  Systems with n <= 32 run the lane-row method,
 * 32 / NB systems per warp.  Default {256, 2}.  Set-up calls: set_config
 * waits for the device and uploads the new task table, so a CUDA graph
 * captured before it must be captured again (its launch keeps the old grid
 * and shared-memory size; a task that no longer fits is skipped and reports
 * info = -1 for its systems).  The result of a call does not depend on the
 * configuration (bit-identical). */
typedef struct gbla_ragged_config {
    int threads;
    int systems_per_block;
} gbla_ragged_config;
gbla_status gbla_ragged_plan_get_config(const gbla_ragged_plan *plan, gbla_ragged_config *config);
gbla_status gbla_ragged_plan_set_config(gbla_ragged_plan *plan, const gbla_ragged_config *config);
/* Tasks of the current configuration and the dynamic shared memory of a block
 * (either pointer nullable). */
gbla_status gbla_ragged_plan_tasks(const gbla_ragged_plan *plan, int *ntasks, size_t *smem_bytes);

/* Autotuner: times every valid configuration (threads x systems per block,
 * 13 candidates) on this batch -- best of `reps` runs after a warm-up, each on
 * fresh copies of A and B -- and keeps the fastest in the plan.  A and B are
 * not modified.  best / best_ms (nullable) receive the choice and its time.
 * Allocates scratch copies and synchronises: a set-up call. */
gbla_status gbla_sragged_autotune(gbla_ragged_plan *plan, const float *A, const float *B, int refine_iters,
                                  int reps, gbla_ragged_config *best, float *best_ms, cudaStream_t stream);
gbla_status gbla_dragged_autotune(gbla_ragged_plan *plan, const double *A, const double *B, int refine_iters,
                                  int reps, gbla_ragged_config *best, float *best_ms, cudaStream_t stream);

/* Factor + solve every system of the plan (device on which the plan was
 * created; one kernel launch, stream-ordered, graph-capturable: the queue
 * counter is reset by the launch itself).  A_i receives its FP32 Cholesky
 * factor (lower triangle), B_i the solutions, info[i] the potrf status.  The
 * factorisation runs in FP32; refine_iters refinement steps recompute
 * B - A X from the full symmetric original A_i (both triangles must be
 * stored) in double-FP32 (float) or FP64 (double) and add the FP32 correction. */
gbla_status gbla_sposv_ragged(const gbla_ragged_plan *plan, float *A, float *B, int *info, int refine_iters,
                              cudaStream_t stream);
gbla_status gbla_dposv_ragged(const gbla_ragged_plan *plan, double *A, double *B, int *info, int refine_iters,
                              cudaStream_t stream);

/* -------------------------------------------------------------------- QR */
/* Householder QR of m x n matrices (any m >= n): R in the upper triangle,
 * the Householder vectors below it (LAPACK dgeqrf convention), tau (n per
 * matrix, batch stride strideTau).  info[i] = j if R(j-1, j-1) is exactly
 * zero, else 0 (nullable).  m <= 128 and n <= 32 run one warp per matrix in
 * registers; larger shapes one block per matrix, the matrix in shared memory
 * when it fits (m n elements up to ~57k floats / ~28k doubles), else worked
 * on in place in A.
 * Replaces cusolverDn<t>geqrf (include/tensor.cuh:1866-1889). */
gbla_status gbla_sgeqrf_batched(int m, int n, float *A, int64_t strideA, float *tau, int64_t strideTau,
                                int *info, int batch, cudaStream_t stream);
gbla_status gbla_dgeqrf_batched(int m, int n, double *A, int64_t strideA, double *tau, int64_t strideTau,
                                int *info, int batch, cudaStream_t stream);

/* C_i <- Q_i^T C_i (trans != 0) or Q_i C_i, Q_i = H_0 ... H_{k-1} from a
 * geqrf result (A_i m x k, tau_i), C_i m x nc.  Any m (m <= 128: one warp per
 * matrix in registers; larger: one warp per column of C, in place).
 * Replaces cusolverDn<t>ormqr (include/tensor.cuh:1891-1927, 1946-1952). */
gbla_status gbla_sormqr_batched(int trans, int m, int nc, int k, const float *A, int64_t strideA,
                                const float *tau, int64_t strideTau, float *C, int64_t strideC, int batch,
                                cudaStream_t stream);
gbla_status gbla_dormqr_batched(int trans, int m, int nc, int k, const double *A, int64_t strideA,
                                const double *tau, int64_t strideTau, double *C, int64_t strideC, int batch,
                                cudaStream_t stream);

/* B_i(0:n, :) <- R_i^-1 B_i(0:n, :) with R_i the upper triangle of the leading
 * n x n block of a matrix stored with leading dimension ldr; B_i has nc
 * columns and leading dimension ldb.
 * Replaces cublas<t>trsm (left, upper, no-trans, non-unit; include/tensor.cuh:1903-1907). */
gbla_status gbla_strsm_upper_batched(int n, int nc, const float *R, int64_t ldr, int64_t strideR, float *B,
                                     int64_t ldb, int64_t strideB, int batch, cudaStream_t stream);
gbla_status gbla_dtrsm_upper_batched(int n, int nc, const double *R, int64_t ldr, int64_t strideR, double *B,
                                     int64_t ldb, int64_t strideB, int batch, cudaStream_t stream);

/* Least squares min ||A_i x - b_i|| for each of nrhs columns (any m >= n):
 * A_i is overwritten with its QR factors and rows [0, n) of each B_i column
 * with the solution (rows [n, m) hold (Q^T b)(n:m)).  Single precision:
 * refine_iters steps of augmented-system refinement with double-FP32
 * residuals recover FP64-level accuracy of x.  info as geqrf.
 * m <= 128, n <= 32: single precision runs one block of four warps per
 * system, on chip from load to store (each warp factorises a quarter of the
 * columns, then solves one right-hand side at a time); double precision one
 * warp per system.  Larger shapes: one block per system (the geqrf block
 * kernel, then one warp per right-hand side); single-precision refinement
 * needs the working copy in shared memory (m n up to ~50k) and returns
 * GBLA_NOT_SUPPORTED beyond it (refine_iters = 0 works for any shape).
 * Replaces cublas<t>gelsBatched in DTensor::leastSquaresBatched
 * (include/tensor.cuh:1340-1394), which allows nrhs = 1 only. */
gbla_status gbla_sgels_batched(int m, int n, int nrhs, float *A, int64_t strideA, float *B, int64_t strideB,
                               int *info, int refine_iters, int batch, cudaStream_t stream);
gbla_status gbla_dgels_batched(int m, int n, int nrhs, double *A, int64_t strideA, double *B, int64_t strideB,
                               int *info, int batch, cudaStream_t stream);
/* The same least squares on another schedule, in two kernels with a
 * workspace: one warp per system factorises in registers and writes the
 * factors and taus to the workspace (the original A stays in place for the
 * refinement residuals), then one block per system solves and refines its
 * right-hand sides with one warp each from the factors in shared memory and
 * finally copies the factors into A.  Results are bit-identical to
 * gbla_sgels_batched.  workspace: at least
 * gbla_sgels_batched_workspace_bytes(m, n, batch) bytes of device memory. */
size_t gbla_sgels_batched_workspace_bytes(int m, int n, int batch);
gbla_status gbla_sgels_batched_ws(int m, int n, int nrhs, float *A, int64_t strideA, float *B, int64_t strideB,
                                  int *info, int refine_iters, void *workspace, size_t workspace_bytes, int batch,
                                  cudaStream_t stream);

/* ------------------------------------------------------ host-buffer calls */
/* A stream pipeline: `streams` worker streams (1..8, 3 recommended) with
 * their events and device staging buffers (grow-only; allocated by the first
 * call that needs them, so make that call outside stream capture).  The
 * *_host calls below take HOST matrices (page-locked for the copies to be
 * asynchronous), split the batch into chunks of `chunk` matrices (0: about
 * an eighth of the batch, at least 1024) and rotate the chunks over the
 * workers, so that copies in, kernels and copies out of consecutive chunks
 * overlap.  The calls are ordered on `stream` like a kernel launch: host
 * buffers must stay valid, and results are available, once `stream` has
 * reached that point.  One pipeline serves one stream at a time, on the
 * device that was current when it was created (other devices: invalid value).  Replaces
 * the synchronous upload -> call -> download sequence of DTensor
 * (include/tensor.cuh:875-884, 1129-1154) around addAB and
 * leastSquaresBatched. */
typedef struct gbla_stream_pipeline gbla_stream_pipeline;
gbla_status gbla_pipeline_create(int streams, gbla_stream_pipeline **pipeline);
gbla_status gbla_pipeline_destroy(gbla_stream_pipeline *pipeline);
/* gbla_sgemm_batched on host A, B, C (C read only when beta != 0). */
gbla_status gbla_sgemm_batched_host(gbla_stream_pipeline *pipeline, int m, int n, int k, float alpha,
                                    const float *A, int64_t strideA, const float *B, int64_t strideB, float beta,
                                    float *C, int64_t strideC, int batch, gbla_gemm_mode mode, int chunk,
                                    cudaStream_t stream);
/* gbla_sgels_batched on host matrices: A and B are inputs; X (stride
 * strideB, may equal B) receives what gbla_sgels_batched leaves in B (the
 * solution in rows [0, n)); F (nullable, stride strideA, may equal A) the QR
 * factors; info (nullable) the per-system status. */
gbla_status gbla_sgels_batched_host(gbla_stream_pipeline *pipeline, int m, int n, int nrhs, const float *A,
                                    int64_t strideA, float *F, const float *B, int64_t strideB, float *X,
                                    int *info, int refine_iters, int batch, int chunk, cudaStream_t stream);

/* ------------------------------------------------------------------- SVD */
/* One-sided (Hestenes) Jacobi SVD A_i = U_i diag(S_i) Vt_i of m x n matrices
 * (any m >= n, n <= 128; warm start V0: n <= 64, m <= 128), in the precision of the data (s: FP32,
 * d: FP64; tol' below uses the unit roundoff of that precision).
 * S_i: n singular values, descending.  Vt_i: n x n (= V^T, as Svd::
 * rightSingularVectors returns).  U_i: m x m, nullable (computeU = false).
 * A_i is destroyed (it ends as A_i V_i).  V0 (nullable): n x n orthogonal warm
 * start; A_i V0_i is orthogonalised and V starts at V0.  A pair of columns is
 * rotated while |a_p.a_q| > tol' |a_p||a_q|, tol' = max(tol, 4 sqrt(m) u)
 * (stored columns cannot be more orthogonal than that); singular values are
 * recomputed as |A v_j| at the end.  info[i] = 1 if max_sweeps sweeps
 * did not converge (nullable), sweeps[i] = sweeps used (nullable).  Sign
 * rule: the largest-magnitude entry of each v_j is negative.
 * Replaces the host loop of cusolverDn<t>gesvd in Svd<T>::factorise
 * (include/tensor.cuh:1624-1676). */
gbla_status gbla_sgesvj_batched(int m, int n, float *A, int64_t strideA, float *S, int64_t strideS, float *Vt,
                                int64_t strideVt, float *U, int64_t strideU, const float *V0, int64_t strideV0,
                                float tol, int max_sweeps, int *info, int *sweeps, int batch,
                                cudaStream_t stream);
gbla_status gbla_dgesvj_batched(int m, int n, double *A, int64_t strideA, double *S, int64_t strideS, double *Vt,
                                int64_t strideVt, double *U, int64_t strideU, const double *V0, int64_t strideV0,
                                double tol, int max_sweeps, int *info, int *sweeps, int batch,
                                cudaStream_t stream);

/* rank[i] = number of entries of S_i (length len) greater than eps.  Unlike
 * Svd::rank (include/tensor.cuh:1600-1609, kernel :1484-1491) the count is
 * written, not accumulated, so repeated calls agree. */
gbla_status gbla_srank_batched(int len, const float *S, int64_t strideS, float eps, unsigned int *rank, int batch,
                               cudaStream_t stream);
gbla_status gbla_drank_batched(int len, const double *S, int64_t strideS, double eps, unsigned int *rank,
                               int batch, cudaStream_t stream);

/* Null space of square or fat m x n matrices (1 <= m <= n, m <= 128): N_i (n x n)
 * holds an orthonormal basis of ker(A_i) in its first nullity_i columns
 * (zero-padded), P_i = N_i N_i^T (n x n).  Singular values <= eps, or
 * below the FP32 noise level n * FLT_EPSILON * sigma_max, count as zero.  nullity (nullable) receives n - rank.  info as gesvj (nullable).
 * `workspace` must hold gbla_snullspace_workspace_bytes(m, n, batch) bytes.
 * Replaces the Nullspace constructor (include/tensor.cuh:2044-2079: tr, Svd of
 * A^T with U, rank, and per-matrix copies and gemms). */
size_t gbla_snullspace_workspace_bytes(int m, int n, int batch);
size_t gbla_dnullspace_workspace_bytes(int m, int n, int batch);
gbla_status gbla_snullspace_batched(int m, int n, const float *A, int64_t strideA, float *N, float *P,
                                    unsigned int *nullity, float eps, int *info, void *workspace,
                                    size_t workspace_bytes, int batch, cudaStream_t stream);
gbla_status gbla_dnullspace_batched(int m, int n, const double *A, int64_t strideA, double *N, double *P,
                                    unsigned int *nullity, double eps, int *info, void *workspace,
                                    size_t workspace_bytes, int batch, cudaStream_t stream);

/* ------------------------------------------------------- level-1 / copy */
/* Per-matrix transpose: At_i (n x m) = A_i^T (A_i is m x n).
 * Replaces the host loop of cublas<t>geam in DTensor::tr (include/tensor.cuh:1167-1197). */
gbla_status gbla_stranspose_batched(int m, int n, const float *A, int64_t strideA, float *At,
                                    int64_t strideAt, int batch, cudaStream_t stream);
gbla_status gbla_dtranspose_batched(int m, int n, const double *A, int64_t strideA, double *At,
                                    int64_t strideAt, int batch, cudaStream_t stream);

/* y <- alpha x + y over len elements.  Replaces cublas<t>axpy in
 * DTensor::operator+= / -= (include/tensor.cuh:1239-1276). */
gbla_status gbla_saxpy(int64_t len, float alpha, const float *x, float *y, cudaStream_t stream);
gbla_status gbla_daxpy(int64_t len, double alpha, const double *x, double *y, cudaStream_t stream);

/* x <- alpha x.  Replaces cublas<t>scal in DTensor::operator*= (include/tensor.cuh:1210-1237). */
gbla_status gbla_sscal(int64_t len, float alpha, float *x, cudaStream_t stream);
gbla_status gbla_dscal(int64_t len, double alpha, double *x, cudaStream_t stream);

/* Whole-buffer reductions with a deterministic fixed-order two-pass tree.
 * The scalar result is written to the device pointer `result`; `workspace`
 * must hold gbla_reduce_workspace_bytes() bytes.
 *   dot  : sum x_i y_i          replaces cublas<t>dot   (include/tensor.cuh:968-992)
 *   nrm2 : sqrt(sum x_i^2)      replaces cublas<t>nrm2  (include/tensor.cuh:994-1010); entries are
 *          scaled by powers of two into three magnitude classes before squaring (Blue's method),
 *          so the result neither overflows nor underflows where the norm itself is representable
 *   asum : sum |x_i|            replaces cublas<t>asum  (include/tensor.cuh:1012-1028)
 *   amax : max |x_i|            replaces cublasI<t>amax + element read (include/tensor.cuh:1030-1050)
 *   amin : min |x_i|            replaces cublasI<t>amin + element read (include/tensor.cuh:1052-1072) */
size_t gbla_reduce_workspace_bytes(void);
gbla_status gbla_sdot(int64_t len, const float *x, const float *y, float *result, void *workspace,
                      cudaStream_t stream);
gbla_status gbla_ddot(int64_t len, const double *x, const double *y, double *result,
                      void *workspace, cudaStream_t stream);
gbla_status gbla_snrm2(int64_t len, const float *x, float *result, void *workspace, cudaStream_t stream);
gbla_status gbla_dnrm2(int64_t len, const double *x, double *result, void *workspace, cudaStream_t stream);
gbla_status gbla_sasum(int64_t len, const float *x, float *result, void *workspace, cudaStream_t stream);
gbla_status gbla_dasum(int64_t len, const double *x, double *result, void *workspace, cudaStream_t stream);
gbla_status gbla_samax(int64_t len, const float *x, float *result, void *workspace, cudaStream_t stream);
gbla_status gbla_damax(int64_t len, const double *x, double *result, void *workspace, cudaStream_t stream);
gbla_status gbla_samin(int64_t len, const float *x, float *result, void *workspace, cudaStream_t stream);
gbla_status gbla_damin(int64_t len, const double *x, double *result, void *workspace, cudaStream_t stream);

/* Allocation-free variant of gbla_sdot, for callers that cannot allocate
 * device memory: a real-time control loop that must not call cudaMalloc
 * after start-up, code running while a stream is being captured, or a host
 * application that owns all device allocation.  It needs no workspace: the
 * partial sums live in a fixed 4 KB device array inside libgbla.so (1024
 * floats, the most any length needs; every device that loads the library
 * keeps it until the process exits).  Same kernels, block count and result
 * as gbla_sdot.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  The address is cached with the ID of the
 * device's context; after a device reset the next call looks it up again in
 * the new context (again outside capture).  All calls share the array, so calls that
 * overlap on the GPU (other streams, other host threads) race; serialise them.
 * Returns GBLA_WORKSPACE_TOO_SMALL if a length would need more than 1024
 * partial sums (none does with the current block count).  No counterpart in
 * the reference: GPUtils' dotF (include/tensor.cuh:968-992) goes through
 * cuBLAS, which manages its own workspace. */
gbla_status gbla_sdot_noalloc(int64_t len, const float *x, const float *y, float *result,
                              cudaStream_t stream);

/* Rows [row_from, row_from + nrows) of the m x n matrix A, copied into the
 * nrows x n matrix out.  Replaces the loop of cublas<t>copy in
 * DTensor::getRows (include/tensor.cuh:1396-1424). */
gbla_status gbla_scopy_rows(int m, int n, int row_from, int nrows, const float *A, float *out,
                            cudaStream_t stream);
gbla_status gbla_dcopy_rows(int m, int n, int row_from, int nrows, const double *A, double *out,
                            cudaStream_t stream);

/* -------------------------------------------------------------- Givens */
/* x_i <- c x_i + s y_i, y_i <- c y_i - s x_i for i < len (strides incx, incy).
 * Replaces cublas<t>rot in DTensor::applyRightGivensRotation /
 * applyLeftGivensRotation (include/tensor.cuh:1074-1104).  The _dev forms
 * read c and s from device memory (GivensAnnihilator, tensor.cuh:2296-2311). */
gbla_status gbla_srot(int64_t len, float *x, int64_t incx, float *y, int64_t incy, float c, float s,
                      cudaStream_t stream);
gbla_status gbla_drot(int64_t len, double *x, int64_t incx, double *y, int64_t incy, double c, double s,
                      cudaStream_t stream);
gbla_status gbla_srot_dev(int64_t len, float *x, int64_t incx, float *y, int64_t incy, const float *c,
                          const float *s, cudaStream_t stream);
gbla_status gbla_drot_dev(int64_t len, double *x, int64_t incx, double *y, int64_t incy, const double *c,
                          const double *s, cudaStream_t stream);
/* out[0..2] = (1/hypot(A(i,j), A(k,j)), A(i,j) out[0], A(k,j) out[0]) for the
 * column-major matrix A with leading dimension ld: the rotation of rows i and
 * k that zeroes A(k,j).  Replaces k_givensAnnihilateRHypot
 * (include/tensor.cuh:2270-2281). */
gbla_status gbla_sgivens_coeffs(const float *A, int64_t ld, int i, int k, int j, float *out, cudaStream_t stream);
gbla_status gbla_dgivens_coeffs(const double *A, int64_t ld, int i, int k, int j, double *out,
                                cudaStream_t stream);

/* Batched forms of the two Givens calls above.  GPUtils applies a rotation
 * to one matrix at a time (applyLeft/RightGivensRotation and
 * GivensAnnihilator throw for tensors with numMats > 1, include/tensor.cuh:
 * 1074-1104, 2200-2312); these rotate every matrix of a batch in one launch.
 * rot_batched: problem b rotates x + b stride and y + b stride (len entries,
 * increments incx, incy) with c = c[b cs_stride], s = s[b cs_stride] (device
 * memory): x <- c x + s y, y <- c y - s x.  The left rotation of rows i, k of
 * every m x n matrix is x = A + i, y = A + k, incx = incy = m, stride = m n;
 * the right rotation of columns i, k is x = A + i m, y = A + k m, inc 1. */
gbla_status gbla_srot_batched(int64_t len, float *x, int64_t incx, float *y, int64_t incy, int64_t stride,
                              const float *c, const float *s, int64_t cs_stride, int batch, cudaStream_t stream);
gbla_status gbla_drot_batched(int64_t len, double *x, int64_t incx, double *y, int64_t incy, int64_t stride,
                              const double *c, const double *s, int64_t cs_stride, int batch, cudaStream_t stream);
/* GivensAnnihilator::annihilate(i, k, j) on every m x n matrix of a batch:
 * each matrix gets its own rotation of rows i and k that zeroes its (k, j)
 * entry (r = 1 / hypot(A(i,j), A(k,j)), c = A(i,j) r, s = A(k,j) r, as
 * k_givensAnnihilateRHypot + cublas<t>rot, include/tensor.cuh:2270-2311).
 * coeffs (nullable) receives (r, c, s) per matrix (3 batch entries).
 * i != k, i, k < m, j < n (invalid value otherwise). */
gbla_status gbla_sgivens_annihilate_batched(int m, int n, float *A, int64_t strideA, int i, int k, int j,
                                            float *coeffs, int batch, cudaStream_t stream);
gbla_status gbla_dgivens_annihilate_batched(int m, int n, double *A, int64_t strideA, int i, int k, int j,
                                            double *coeffs, int batch, cudaStream_t stream);

/* ------------------------------------------ BF16 tensor-core GEMM (TN) */
/* Fused epilogue of gbla_gemm_bf16_tn, applied per element in this order:
 * t = alpha * acc; t += bias[n] (nullable); t = max(t, 0) if relu;
 * t = 0 where mask[m][n] <= 0 (nullable; the ReLU derivative of a stored
 * activation).  t is then written to every non-null output: out_f32 [M][N]
 * FP32, out_bf16 [M][N] and out_bf16_t [N][M] (transposed) as BF16 bit
 * patterns.  ld_* are row strides in elements. */
typedef struct gbla_bf16_epilogue {
    float alpha;
    const float *bias;
    int relu;
    const uint16_t *mask;
    int64_t ld_mask;
    float *out_f32;
    int64_t ld_f32;
    uint16_t *out_bf16;
    int64_t ld_bf16;
    uint16_t *out_bf16_t;
    int64_t ld_bf16_t;
} gbla_bf16_epilogue;

/* C[M x N] = A[M x K] * B[N x K]^T with BF16 operands (row-major, K
 * contiguous: lda, ldb >= K, multiples of 8; 16-byte aligned bases) and FP32
 * accumulation in tensor memory (tcgen05, TMA-fed).  Any M, N, K >= 1; tails
 * are zero-filled.  No reference counterpart: it carries the warm-start
 * network below. */
gbla_status gbla_gemm_bf16_tn(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb,
                              const gbla_bf16_epilogue *epi, cudaStream_t stream);

/* ------------------------------------------- learned Jacobi warm start */
/* A small network maps an n x n matrix A (n*n inputs, column-major order) to
 * the P = n(n-1)/2 strictly-upper entries of a skew matrix S (row-major upper
 * triangle order: (0,1), (0,2), ..., (0,n-1), (1,2), ...), and the warm-start
 * frame is V0 = Vb * (I - S)^{-1} (I + S) (a Cayley transform about a fixed
 * base frame Vb).  Layers: n*n -> hidden -> hidden -> P, ReLU after the two
 * hidden layers; BF16 weights and activations, FP32 accumulation (tcgen05),
 * FP32 master weights and Adam state.
 * Training loss per matrix (mean over the batch): || V0 - V Pi D ||_F^2,
 * where V is the converged Jacobi frame of A and the column permutation Pi
 * and signs D are chosen greedily (largest |V0^T V| entry first) so that the
 * loss measures the distance to the nearest exact eigenbasis.
 * No reference counterpart: the reference always starts Jacobi cold. */
typedef struct gbla_wsnet gbla_wsnet;

/* n <= 64 with n*n and n(n-1)/2 multiples of 8 ... (n in {16, 32, 48, 64});
 * hidden a multiple of 64; max_batch >= 1.  Allocates device memory (not a
 * hot-path call).  Weights: He-uniform for the hidden layers, zero for the
 * output layer (so the first prediction is V0 = Vb); Vb = identity. */
gbla_status gbla_wsnet_create(int n, int hidden, int max_batch, uint64_t seed, gbla_wsnet **net);
gbla_status gbla_wsnet_destroy(gbla_wsnet *net);
/* Number of FP32 parameters, laid out flat as W1 [hidden][n*n], b1 [hidden],
 * W2 [hidden][hidden], b2 [hidden], W3 [P][hidden], b3 [P] (row-major). */
int64_t gbla_wsnet_param_count(const gbla_wsnet *net);
/* Device copies of the parameters (set also refreshes the BF16 weights and
 * clears the Adam state) and of the base frame (n x n column-major). */
gbla_status gbla_wsnet_get_params(const gbla_wsnet *net, float *params, cudaStream_t stream);
gbla_status gbla_wsnet_set_params(gbla_wsnet *net, const float *params, cudaStream_t stream);
gbla_status gbla_wsnet_get_base(const gbla_wsnet *net, float *Vb, cudaStream_t stream);
gbla_status gbla_wsnet_set_base(gbla_wsnet *net, const float *Vb, cudaStream_t stream);
/* Loss and gradient of a batch without updating: matrices idx[b] (idx
 * nullable = 0..batch-1) of A (n x n, stride strideA) and their Jacobi
 * frames V (stride strideV).  grad: param_count floats (device); loss: one
 * float (device, mean over the batch); assign (nullable): batch x n ints,
 * the true column matched to each predicted column as sign * (1 + index). */
gbla_status gbla_wsnet_gradients(gbla_wsnet *net, const float *A, int64_t strideA, const float *V, int64_t strideV,
                                 const int *idx, int batch, float *grad, float *loss, int *assign,
                                 cudaStream_t stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) at learning rate lr on
 * the batch; loss (nullable, device) receives the batch loss before the step. */
gbla_status gbla_wsnet_train_step(gbla_wsnet *net, const float *A, int64_t strideA, const float *V,
                                  int64_t strideV, const int *idx, int batch, float lr, float *loss,
                                  cudaStream_t stream);
/* Warm-start frames V0 (n x n column-major, stride strideV0) for a batch of
 * at most max_batch matrices. */
gbla_status gbla_wsnet_predict(gbla_wsnet *net, const float *A, int64_t strideA, float *V0, int64_t strideV0,
                               int batch, cudaStream_t stream);

/* Warm-started one-sided Jacobi SVD with cold fallback: as gbla_sgesvj_batched
 * (n <= 64, m <= 128, U nullable) starting from V0, but a matrix that has not
 * converged after warm_budget sweeps restarts from A with V = I and runs to
 * convergence (max_sweeps more at most).  sweeps (nullable) counts all sweeps
 * of the matrix; fallback (nullable) is 1 where the cold restart ran.  A is
 * not modified. */
gbla_status gbla_sgesvj_warm_batched(int m, int n, const float *A, int64_t strideA, float *S, int64_t strideS,
                                     float *Vt, int64_t strideVt, float *U, int64_t strideU, const float *V0,
                                     int64_t strideV0, int warm_budget, float tol, int max_sweeps, int *info,
                                     int *sweeps, int *fallback, int batch, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* GBLA_H */
