"""The seeded benchmark inputs have the shapes and distributions the
benchmark configurations are quoted on (CPU only, reduced batch counts)."""
import numpy as np

from gputils_gb300 import warmstart, workloads


def test_generators_are_deterministic():
    a1, b1 = workloads.d2b_least_squares(k=8)
    a2, b2 = workloads.d2b_least_squares(k=8)
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    g1, _ = workloads.d2a_gemm(k=4)
    g2, _ = workloads.d2a_gemm(k=4)
    assert np.array_equal(g1, g2)


def test_d1_cholesky_spd_and_well_conditioned():
    M, b = workloads.d1_cholesky(k=256)
    assert M.shape == (256, 16, 16) and b.shape == (256, 16, 1) and M.dtype == np.float32
    w = np.linalg.eigvalsh(M.astype(np.float64))
    assert (w > 0.99).all()                      # G^T G / 16 + I: every eigenvalue >= 1
    assert np.max(w[:, -1] / w[:, 0]) < 12       # kappa of a few units


def test_d2a_gemm_uniform_operands():
    A, B = workloads.d2a_gemm(k=64)
    assert A.shape == B.shape == (64, 64, 64) and A.dtype == np.float32
    assert A.min() >= -1 and A.max() <= 1 and abs(A.mean()) < 0.02


def test_d2b_least_squares_spectrum():
    A, B = workloads.d2b_least_squares(k=16)
    assert A.shape == (16, 128, 32) and B.shape == (16, 128, 4)
    s = np.linalg.svd(A.astype(np.float64), compute_uv=False)
    want = np.logspace(0.0, 3.0, 32)[::-1]
    assert np.abs(s / want - 1).max() < 1e-4     # log-spaced 1..1e3 up to FP32 rounding of A
    assert np.allclose(s[:, 0] / s[:, -1], 1e3, rtol=1e-3)


def test_d3_ragged_layout_and_sizes():
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(count=500)
    assert n.min() >= 4 and n.max() <= 128 and nrhs.min() >= 1 and nrhs.max() <= 8
    assert a_off[0] == 0 and np.array_equal(np.diff(a_off), n[:-1].astype(np.int64) ** 2)
    assert np.array_equal(np.diff(b_off), (n[:-1] * nrhs[:-1]).astype(np.int64))
    assert A.size == int((n.astype(np.int64) ** 2).sum()) and B.size == int((n * nrhs).sum())
    for i in (0, 1, 250, 499):
        Mi = A[a_off[i]:a_off[i] + n[i] ** 2].reshape(n[i], n[i]).astype(np.float64)
        assert np.allclose(Mi, Mi.T) and np.linalg.eigvalsh(Mi).min() > 0.09   # G^T G / n + 0.1 I


def test_svd_family_members_and_warmstart_basis_agree():
    A, theta, basis = workloads.svd_family(8, 64, seed=6)
    assert A.shape == (8, 64, 64) and np.abs(theta).max() <= 1
    assert np.allclose(A[0], basis[0] + np.tensordot(theta[0], basis[1:], axes=1), atol=1e-6)
    # the warm-start trainer draws the same fixed matrices from the same seed
    assert np.array_equal(warmstart.family_basis(64, 6), basis)
