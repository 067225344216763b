"""Seeded synthetic inputs for the benchmark configurations.

Each generator returns numpy batches of shape (k, m, n) (k matrices of
m x n); the same seed always gives the same inputs.  The distributions are
the ones the benchmark configurations are quoted on:

  d1  Cholesky factor+solve: 4096 SPD 16x16 fp32, M = G^T G / 16 + I, G ~ N(0,1),
      one RHS b ~ N(0,1)
  d2a addAB: 16384 pairs of 64x64 fp32, entries U[-1, 1]
  d2b least squares: 8192 tall 128x32 fp32, A = U diag(s) V^T (Haar U, V;
      s log-spaced 1..1e3), 4 RHS ~ N(0,1)
  d3  ragged Cholesky: 20000 SPD systems, n = round(exp(U(ln 4, ln 128))),
      nrhs ~ U{1..8}, M = G^T G / n + 0.1 I
  d4  Jacobi SVD: 8192 32x32 fp32 from A(theta) = A0 + sum_j theta_j A_j,
      A0, A_j ~ N(0,1)/sqrt(32) fixed by the seed, theta ~ U[-1,1]^4
  d5  as d4 at 64x64, batch 32768
"""
from __future__ import annotations

import numpy as np


def d1_cholesky(k: int = 4096, n: int = 16, seed: int = 1):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((k, n, n))
    M = G.transpose(0, 2, 1) @ G / n + np.eye(n)
    b = rng.standard_normal((k, n, 1))
    return M.astype(np.float32), b.astype(np.float32)


def d2a_gemm(k: int = 16384, n: int = 64, seed: int = 2):
    rng = np.random.default_rng(seed)
    A = rng.uniform(-1.0, 1.0, (k, n, n)).astype(np.float32)
    B = rng.uniform(-1.0, 1.0, (k, n, n)).astype(np.float32)
    return A, B


def _haar(rng, k: int, m: int, n: int) -> np.ndarray:
    """k matrices with orthonormal columns, Haar distributed (QR of a
    Gaussian with the sign of R's diagonal folded into Q)."""
    Z = rng.standard_normal((k, m, n))
    Q, R = np.linalg.qr(Z)
    d = np.sign(np.diagonal(R, axis1=1, axis2=2))
    d[d == 0] = 1.0
    return Q * d[:, None, :]


def d2b_least_squares(k: int = 8192, m: int = 128, n: int = 32, nrhs: int = 4, cond: float = 1e3,
                      seed: int = 3):
    rng = np.random.default_rng(seed)
    U = _haar(rng, k, m, n)
    V = _haar(rng, k, n, n)
    s = np.logspace(0.0, np.log10(cond), n)[::-1]
    A = (U * s[None, None, :]) @ V.transpose(0, 2, 1)
    B = rng.standard_normal((k, m, nrhs))
    return A.astype(np.float32), B.astype(np.float32)


def d3_ragged(count: int = 20000, nmin: int = 4, nmax: int = 128, rhs_max: int = 8, seed: int = 4,
              dtype=np.float32):
    """Returns (n, nrhs, a_off, b_off, A_arena, B_arena): system i has its
    n_i x n_i matrix at A_arena[a_off[i]:] and its n_i x nrhs_i right-hand
    side at B_arena[b_off[i]:], both column-major."""
    rng = np.random.default_rng(seed)
    n = np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), count))).astype(np.int32)
    nrhs = rng.integers(1, rhs_max + 1, count).astype(np.int32)
    a_sz = n.astype(np.int64) ** 2
    b_sz = n.astype(np.int64) * nrhs
    a_off = np.concatenate([[0], np.cumsum(a_sz)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(b_sz)[:-1]]).astype(np.int64)
    A = np.empty(int(a_sz.sum()), dtype=dtype)
    B = np.empty(int(b_sz.sum()), dtype=dtype)
    for ni in np.unique(n):
        idx = np.nonzero(n == ni)[0]
        G = rng.standard_normal((len(idx), ni, ni))
        M = G.transpose(0, 2, 1) @ G / ni + 0.1 * np.eye(ni)
        flat = M.transpose(0, 2, 1).reshape(len(idx), -1)  # column-major per matrix
        for j, i in enumerate(idx):
            A[a_off[i]:a_off[i] + a_sz[i]] = flat[j]
    B[:] = rng.standard_normal(B.shape[0])
    return n, nrhs, a_off, b_off, A, B


def svd_family(k: int, n: int, seed: int, params: int = 4):
    """A(theta) = A0 + sum_j theta_j A_j with A0, A_j ~ N(0,1)/sqrt(n) fixed by
    `seed` and theta ~ U[-1,1]^params per matrix.  Returns (A, theta, basis)."""
    rng = np.random.default_rng(seed)
    basis = rng.standard_normal((params + 1, n, n)) / np.sqrt(n)
    theta = rng.uniform(-1.0, 1.0, (k, params))
    A = basis[0][None] + np.einsum("kp,pij->kij", theta, basis[1:])
    return A.astype(np.float32), theta, basis


def d4_svd32(k: int = 8192, seed: int = 5):
    return svd_family(k, 32, seed)[0]


def d5_svd64(k: int = 32768, seed: int = 6):
    return svd_family(k, 64, seed)[0]
