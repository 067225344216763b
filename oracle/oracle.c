/*
 * oracle.c -- FP64 CPU oracle for the GPUtils batched-matrix hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libgbla.so, the include/ headers,
 * the drop-in tensor.cuh) links, loads or calls this file.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and only as
 * the reference values of the parity tests / the timed host baseline.
 *
 * The reference (GPUEngineering/GPUtils, include/tensor.cuh) has no CPU code:
 * every numeric call on the path goes to cuBLAS 13.1 / cuSOLVER 12.0 (CUDA
 * 13.0 toolkit), whose source is not part of the reference.  This file restates
 * the published LAPACK/BLAS algorithms those calls implement, in double
 * precision, with the conventions the reference relies on:
 *
 *   orc_gemm_batched     cublas<t>gemmBatched NN        tensor.cuh:1286-1338
 *   orc_potrf_batched    cusolverDn<t>potrf(Batched)    tensor.cuh:1742-1761, 2135-2159
 *   orc_potrs_batched    cusolverDn<t>potrs(Batched)    tensor.cuh:1763-1783, 2161-2197
 *   orc_geqrf_batched    cusolverDn<t>geqrf (dgeqr2 + dlarfg conventions)  tensor.cuh:1866-1889
 *   orc_ormqr_batched    cusolverDn<t>ormqr (left side)  tensor.cuh:1891-1927, 1946-1952
 *   orc_trsm_upper_batched cublas<t>trsm (left, upper, no-trans, non-unit) tensor.cuh:1903-1907
 *   orc_gels_batched     cublas<t>gelsBatched (QR least squares)  tensor.cuh:1340-1394
 *   orc_gesvj_batched    the SVD Svd<T>::factorise obtains from gesvd    tensor.cuh:1624-1676,
 *                        computed here by one-sided (Hestenes) Jacobi in FP64
 *   orc_posv_ragged      a loop of potrf+potrs over a ragged descriptor table
 *                        (the reference's per-size loop of CholeskyBatchFactoriser)
 *
 * Storage: column-major matrices stored back to back (DTensor (m,n,k) layout,
 * tensor.cuh:264-281), leading dimension = rows.  Batched entry points run an
 * OpenMP parallel-for over matrices when built with -fopenmp.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(i, j, ld) ((int64_t)(i) + (int64_t)(j) * (int64_t)(ld))

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

/* ------------------------------------------------------------------ GEMM */
/* C <- alpha*A*B + beta*C, A m x k, B k x n, C m x n, all leading dim = rows.
 * Semantics of cublas<t>gemm(N, N) as called by DTensor::addAB
 * (tensor.cuh:1294-1309): lda = m, ldb = k, ldc = m.  beta == 0 ignores C. */
static void gemm1(int m, int n, int k, double alpha, const double *A, const double *B,
                  double beta, double *C) {
    for (int j = 0; j < n; j++) {
        double *c = C + IDX(0, j, m);
        if (beta == 0.0) {
            for (int i = 0; i < m; i++) c[i] = 0.0;
        } else if (beta != 1.0) {
            for (int i = 0; i < m; i++) c[i] *= beta;
        }
        for (int p = 0; p < k; p++) {
            double b = alpha * B[IDX(p, j, k)];
            const double *a = A + IDX(0, p, m);
            for (int i = 0; i < m; i++) c[i] += a[i] * b;
        }
    }
}

void orc_gemm_batched(int m, int n, int k, double alpha, const double *A, const double *B,
                      double beta, double *C, int batch) {
    int64_t sA = (int64_t)m * k, sB = (int64_t)k * n, sC = (int64_t)m * n;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < batch; b++) gemm1(m, n, k, alpha, A + b * sA, B + b * sB, beta, C + b * sC);
}

/* -------------------------------------------------------------- Cholesky */
/* Lower Cholesky in place (left-looking / Crout order).  The strictly upper
 * triangle is left untouched, as cusolverDn<t>potrf with CUBLAS_FILL_MODE_LOWER
 * does (tensor.cuh:1745, 2138).  Returns 0, or j+1 when the leading minor of
 * order j+1 is not positive definite (LAPACK/cuSOLVER info convention). */
static int potrf1(int n, double *A, int lda) {
    for (int j = 0; j < n; j++) {
        double d = A[IDX(j, j, lda)];
        for (int p = 0; p < j; p++) d -= A[IDX(j, p, lda)] * A[IDX(j, p, lda)];
        if (!(d > 0.0)) return j + 1;
        double ljj = sqrt(d);
        A[IDX(j, j, lda)] = ljj;
        for (int i = j + 1; i < n; i++) {
            double s = A[IDX(i, j, lda)];
            for (int p = 0; p < j; p++) s -= A[IDX(i, p, lda)] * A[IDX(j, p, lda)];
            A[IDX(i, j, lda)] = s / ljj;
        }
    }
    return 0;
}

/* Solve L L^T X = B with the lower factor in L (potrs, tensor.cuh:1766-1771). */
static void potrs1(int n, int nrhs, const double *L, int ldl, double *B, int ldb) {
    for (int r = 0; r < nrhs; r++) {
        double *x = B + IDX(0, r, ldb);
        for (int i = 0; i < n; i++) {
            double s = x[i];
            for (int p = 0; p < i; p++) s -= L[IDX(i, p, ldl)] * x[p];
            x[i] = s / L[IDX(i, i, ldl)];
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = x[i];
            for (int p = i + 1; p < n; p++) s -= L[IDX(p, i, ldl)] * x[p];
            x[i] = s / L[IDX(i, i, ldl)];
        }
    }
}

void orc_potrf_batched(int n, double *A, int *info, int batch) {
    int64_t s = (int64_t)n * n;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < batch; b++) info[b] = potrf1(n, A + b * s, n);
}

void orc_potrs_batched(int n, int nrhs, const double *L, double *B, int batch) {
    int64_t sL = (int64_t)n * n, sB = (int64_t)n * nrhs;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < batch; b++) potrs1(n, nrhs, L + b * sL, n, B + b * sB, n);
}

/* Ragged factor + solve: system i has an n_i x n_i matrix at A + a_off[i] and
 * an n_i x nrhs_i right-hand side at B + b_off[i] (both column-major).
 * A is overwritten by L, B by X.  Restates the reference's only way to do
 * this: one CholeskyBatchFactoriser factorise()+solve() per size group. */
void orc_posv_ragged(int count, const int64_t *a_off, const int64_t *b_off, const int *n,
                     const int *nrhs, double *A, double *B, int *info) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < count; i++) {
        info[i] = potrf1(n[i], A + a_off[i], n[i]);
        if (info[i] == 0) potrs1(n[i], nrhs[i], A + a_off[i], n[i], B + b_off[i], n[i]);
    }
}

/* ------------------------------------------------------------------- QR */
/* Householder vector in LAPACK dlarfg form: on entry x = (alpha, x(1:)),
 * on exit x(1:) holds v(1:) (v(0) = 1 implied), returns beta in *beta and tau. */
static double larfg(int len, double *alpha, double *x, int incx) {
    double xnorm = 0.0;
    for (int i = 0; i < len; i++) xnorm = hypot(xnorm, x[(int64_t)i * incx]);
    if (xnorm == 0.0) return 0.0;
    double a = *alpha;
    double beta = -copysign(hypot(a, xnorm), a);
    double tau = (beta - a) / beta;
    double scal = 1.0 / (a - beta);
    for (int i = 0; i < len; i++) x[(int64_t)i * incx] *= scal;
    *alpha = beta;
    return tau;
}

/* apply H = I - tau v v^T (v(0) = 1, v(1:) in vtail) to rows [k, m) of C. */
static void apply_h(int m, int k, const double *vtail, double tau, double *C, int ldc, int ncols) {
    if (tau == 0.0) return;
    for (int j = 0; j < ncols; j++) {
        double *c = C + IDX(0, j, ldc);
        double w = c[k];
        for (int i = k + 1; i < m; i++) w += vtail[i - k - 1] * c[i];
        w *= tau;
        c[k] -= w;
        for (int i = k + 1; i < m; i++) c[i] -= vtail[i - k - 1] * w;
    }
}

/* Householder QR (dgeqr2 order): R in the upper triangle, reflectors below. */
static void geqrf1(int m, int n, double *A, int lda, double *tau) {
    int kmax = m < n ? m : n;
    for (int k = 0; k < kmax; k++) {
        double *col = A + IDX(0, k, lda);
        tau[k] = larfg(m - k - 1, &col[k], col + k + 1, 1);
        if (k + 1 < n) {
            apply_h(m, k, col + k + 1, tau[k], A + IDX(0, k + 1, lda), lda, n - k - 1);
        }
    }
}

/* Left-side ormqr: trans != 0 applies Q^T = H_{kk-1}...H_0, else Q = H_0...H_{kk-1}. */
static void ormqr1(int trans, int m, int nrhs, int kk, const double *A, int lda,
                   const double *tau, double *C, int ldc) {
    if (trans) {
        for (int k = 0; k < kk; k++) apply_h(m, k, A + IDX(k + 1, k, lda), tau[k], C, ldc, nrhs);
    } else {
        for (int k = kk - 1; k >= 0; k--) apply_h(m, k, A + IDX(k + 1, k, lda), tau[k], C, ldc, nrhs);
    }
}

/* Back substitution R X = B with R the n x n upper triangle of R (ld ldr). */
static void trsm_upper1(int n, int nrhs, const double *R, int ldr, double *B, int ldb) {
    for (int r = 0; r < nrhs; r++) {
        double *x = B + IDX(0, r, ldb);
        for (int i = n - 1; i >= 0; i--) {
            double s = x[i];
            for (int p = i + 1; p < n; p++) s -= R[IDX(i, p, ldr)] * x[p];
            x[i] = s / R[IDX(i, i, ldr)];
        }
    }
}

void orc_geqrf_batched(int m, int n, double *A, double *tau, int batch) {
    int kmax = m < n ? m : n;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < batch; b++) geqrf1(m, n, A + (int64_t)b * m * n, m, tau + (int64_t)b * kmax);
}

void orc_ormqr_batched(int trans, int m, int nrhs, int kk, const double *A, int n_cols_a,
                       const double *tau, double *C, int batch) {
#pragma omp parallel for schedule(static)
    for (int b = 0; b < batch; b++)
        ormqr1(trans, m, nrhs, kk, A + (int64_t)b * m * n_cols_a, m, tau + (int64_t)b * kk,
               C + (int64_t)b * m * nrhs, m);
}

void orc_trsm_upper_batched(int n, int nrhs, const double *R, int ldr, int64_t strideR,
                            double *B, int ldb, int64_t strideB, int batch) {
#pragma omp parallel for schedule(static)
    for (int b = 0; b < batch; b++) trsm_upper1(n, nrhs, R + b * strideR, ldr, B + b * strideB, ldb);
}

/* QR least squares, gels semantics (tensor.cuh:1354-1365): A (m x n, m >= n)
 * is overwritten with its QR factors, B (m x nrhs) on exit holds X in rows
 * [0, n). */
void orc_gels_batched(int m, int n, int nrhs, double *A, double *B, int batch) {
#pragma omp parallel for schedule(static)
    for (int b = 0; b < batch; b++) {
        double tau[512];
        double *Ab = A + (int64_t)b * m * n, *Bb = B + (int64_t)b * m * nrhs;
        double *t = n <= 512 ? tau : (double *)malloc(sizeof(double) * n);
        geqrf1(m, n, Ab, m, t);
        ormqr1(1, m, nrhs, n, Ab, m, t, Bb, m);
        trsm_upper1(n, nrhs, Ab, m, Bb, m);
        if (t != tau) free(t);
    }
}

/* ---------------------------------------------------------- Jacobi SVD */
/* Canonical sign of a singular pair: the entry of v with the largest
 * magnitude (the first one on ties) is made negative.  The GPU kernels apply
 * the same rule.  On the reference's pinned 3x2 case
 * (test/testTensor.cu:1137-1161) it reproduces the signs gesvd returned. */
static void canon_sign(int m, int n, double *u, double *v) {
    int imax = 0;
    double vmax = -1.0;
    for (int i = 0; i < n; i++) {
        double a = fabs(v[i]);
        if (a > vmax) { vmax = a; imax = i; }
    }
    if (v[imax] > 0.0) {
        for (int i = 0; i < n; i++) v[i] = -v[i];
        if (u) for (int i = 0; i < m; i++) u[i] = -u[i];
    }
}

/* One-sided Jacobi (Hestenes) SVD of an m x n matrix, cyclic-by-rows
 * ordering, Rutishauser rotation formulas.  A pair (p,q) is rotated when
 * |a_p . a_q| > tol * ||a_p|| ||a_q||; the sweep loop stops after a sweep
 * with no rotation or after max_sweeps (info = 1 then).
 * Outputs: S (n column norms, sorted descending), V (n x n), and, when U is
 * non-NULL, U (m x m): the normalised columns for the nonzero singular
 * values, completed to an orthonormal basis by one forward scan of Gram-Schmidt
 * over e_0..e_{m-1}: e_i is accepted when its residual norm exceeds
 * 0.5/sqrt(m) (some e_i always has residual >= 1/sqrt(m), so the scan
 * completes), and the c-th accepted column is multiplied by (-1)^c.  A is overwritten
 * with A V (unsorted). */
static int gesvj1(int m, int n, double *A, double *S, double *V, double *U, double tol,
                  int max_sweeps, int *sweeps_out) {
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) V[IDX(i, j, n)] = (i == j) ? 1.0 : 0.0;
    int sweep = 0, info = 1;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        int rotated = 0;
        for (int p = 0; p < n - 1; p++) {
            for (int q = p + 1; q < n; q++) {
                double *ap = A + IDX(0, p, m), *aq = A + IDX(0, q, m);
                double alpha = 0, beta = 0, gamma = 0;
                for (int i = 0; i < m; i++) {
                    alpha += ap[i] * ap[i];
                    beta += aq[i] * aq[i];
                    gamma += ap[i] * aq[i];
                }
                if (gamma == 0.0 || !(fabs(gamma) > tol * sqrt(alpha * beta))) continue;
                double zeta = (beta - alpha) / (2.0 * gamma);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
                for (int i = 0; i < m; i++) {
                    double x = ap[i], y = aq[i];
                    ap[i] = c * x - s * y;
                    aq[i] = s * x + c * y;
                }
                double *vp = V + IDX(0, p, n), *vq = V + IDX(0, q, n);
                for (int i = 0; i < n; i++) {
                    double x = vp[i], y = vq[i];
                    vp[i] = c * x - s * y;
                    vq[i] = s * x + c * y;
                }
                rotated++;
            }
        }
        if (rotated == 0) { info = 0; break; }
    }
    if (sweeps_out) *sweeps_out = sweep > max_sweeps ? max_sweeps : sweep;

    /* column norms, then a stable descending sort of (norm, index) */
    int *ord = (int *)malloc(sizeof(int) * n);
    double *nrm = (double *)malloc(sizeof(double) * n);
    for (int j = 0; j < n; j++) {
        double s2 = 0;
        for (int i = 0; i < m; i++) s2 += A[IDX(i, j, m)] * A[IDX(i, j, m)];
        nrm[j] = sqrt(s2);
        ord[j] = j;
    }
    for (int i = 1; i < n; i++) { /* insertion sort, stable */
        int o = ord[i];
        int k = i - 1;
        while (k >= 0 && nrm[ord[k]] < nrm[o]) { ord[k + 1] = ord[k]; k--; }
        ord[k + 1] = o;
    }
    double *Vs = (double *)malloc(sizeof(double) * n * n);
    double *Us = (double *)malloc(sizeof(double) * m * (n > m ? n : m));
    for (int j = 0; j < n; j++) {
        int o = ord[j];
        S[j] = nrm[o];
        memcpy(Vs + IDX(0, j, n), V + IDX(0, o, n), sizeof(double) * n);
        for (int i = 0; i < m; i++) Us[IDX(i, j, m)] = nrm[o] > 0 ? A[IDX(i, o, m)] / nrm[o] : 0.0;
    }
    double smax = n > 0 ? S[0] : 0.0;
    int r = 0; /* numerical rank used for the U completion */
    double rtol = smax * 1e-12 * (m > n ? m : n);
    for (int j = 0; j < n && j < m; j++) if (S[j] > rtol) r++;
    for (int j = 0; j < n; j++) canon_sign(m, n, j < r ? Us + IDX(0, j, m) : NULL, Vs + IDX(0, j, n));
    memcpy(V, Vs, sizeof(double) * n * n);
    if (U) {
        for (int j = 0; j < r; j++) memcpy(U + IDX(0, j, m), Us + IDX(0, j, m), sizeof(double) * m);
        int c = r, ncomp = 0;
        double accept = 0.5 / sqrt((double)m);
        for (int e = 0; e < m && c < m; e++) {
            double *w = U + IDX(0, c, m);
            for (int i = 0; i < m; i++) w[i] = (i == e) ? 1.0 : 0.0;
            for (int pass = 0; pass < 2; pass++) {
                for (int j = 0; j < c; j++) {
                    double *u = U + IDX(0, j, m);
                    double d = 0;
                    for (int i = 0; i < m; i++) d += u[i] * w[i];
                    for (int i = 0; i < m; i++) w[i] -= d * u[i];
                }
            }
            double s2 = 0;
            for (int i = 0; i < m; i++) s2 += w[i] * w[i];
            double nw = sqrt(s2);
            if (nw > accept) {
                double sg = (ncomp % 2 == 0) ? 1.0 : -1.0;
                for (int i = 0; i < m; i++) w[i] = sg * w[i] / nw;
                c++;
                ncomp++;
            }
        }
    }
    free(ord); free(nrm); free(Vs); free(Us);
    return info;
}

/* Batched driver.  S holds n values per matrix (the first min(m,n) are the
 * singular values), V n x n, U m x m (optional). */
void orc_gesvj_batched(int m, int n, double *A, double *S, double *V, double *U, double tol,
                       int max_sweeps, int *sweeps, int *info, int batch) {
#pragma omp parallel for schedule(dynamic, 8)
    for (int b = 0; b < batch; b++) {
        int sw = 0;
        info[b] = gesvj1(m, n, A + (int64_t)b * m * n, S + (int64_t)b * n, V + (int64_t)b * n * n,
                         U ? U + (int64_t)b * m * m : NULL, tol, max_sweeps, &sw);
        if (sweeps) sweeps[b] = sw;
    }
}
