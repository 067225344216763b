"""Pins the FP64 oracle (oracle/oracle.c) before the parity tests rely on it:
against every golden value the reference's own tests hold for the hot path
(read from test/testTensor.cu into tests/golden/reference_goldens.json) and
against numpy/scipy LAPACK on random inputs.  CPU only."""
import numpy as np
import pytest
import scipy.linalg as sla

from oracle import oracle as O
from tests.helpers import colmajor, goldens, rowmajor

G = goldens()
HIGH = G["precision_high"]  # the reference's double-precision tolerance


def test_gemm_golden():
    # test/testTensor.cu:828-853 (exact integer result)
    A = colmajor(G["addAB_a"], 2, 3, 3)
    B = colmajor(G["addAB_b"], 3, 2, 3)
    C = O.gemm(A, B)
    assert np.array_equal(C.transpose(0, 2, 1).ravel(), np.array(G["addAB_expected"]))


def test_gemm_random_vs_numpy():
    rng = np.random.default_rng(1)
    for (m, n, k) in [(1, 1, 1), (5, 7, 3), (64, 64, 64), (17, 3, 40)]:
        A = rng.uniform(-1, 1, (4, m, k)); B = rng.uniform(-1, 1, (4, k, n)); Cin = rng.standard_normal((4, m, n))
        np.testing.assert_allclose(O.gemm(A, B), A @ B, rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(O.gemm(A, B, Cin, 0.5, -2.0), 0.5 * A @ B - 2.0 * Cin, rtol=1e-13, atol=1e-12)


def test_cholesky_golden():
    # test/testTensor.cu:1218-1238 and :1244-1276
    A = colmajor(G["chol_a"], 3, 3)
    L, info = O.potrf(A)
    assert info[0] == 0
    assert abs(L[0, 0, 0] - G["chol_L00"]) < HIGH
    assert abs(L[0, 2, 1] - G["chol_L21"]) < HIGH
    assert abs(L[0, 2, 2] - G["chol_L22"]) < HIGH
    # the strict upper triangle is untouched (CUBLAS_FILL_MODE_LOWER)
    assert np.array_equal(np.triu(L[0], 1), np.triu(A[0], 1))
    x = O.potrs(L, np.array(G["chol_b"]).reshape(1, 3, 1))
    np.testing.assert_allclose(x[0, :, 0], G["chol_x"], atol=HIGH)
    # pre-factored L (test/testTensor.cu:1364-1413)
    low = rowmajor(G["chol_low_rowmajor"], 3, 3)
    x2 = O.potrs(low, np.array(G["chol_b"]).reshape(1, 3, 1))
    np.testing.assert_allclose(x2[0, :, 0], G["chol_x"], atol=HIGH)


def test_cholesky_info_semantics():
    A = np.eye(4)[None].copy()
    A[0, 2, 2] = -1.0   # third leading minor not positive definite
    _, info = O.potrf(A)
    assert info[0] == 3


def test_cholesky_random_vs_numpy():
    rng = np.random.default_rng(2)
    for n in (1, 2, 16, 33, 128):
        G_ = rng.standard_normal((3, n, n))
        M = G_.transpose(0, 2, 1) @ G_ / n + 0.1 * np.eye(n)
        L, info = O.potrf(M)
        assert (info == 0).all()
        np.testing.assert_allclose(np.tril(L), np.linalg.cholesky(M), atol=1e-11)
        b = rng.standard_normal((3, n, 5))
        np.testing.assert_allclose(O.potrs(L, b), np.linalg.solve(M, b), rtol=1e-9, atol=1e-10)


def test_ragged_vs_uniform():
    rng = np.random.default_rng(3)
    ns = [4, 9, 16, 1, 40]
    nr = [1, 3, 2, 8, 4]
    a_off, b_off, A, B, mats, rhs = [], [], [], [], [], []
    ao = bo = 0
    for n, r in zip(ns, nr):
        M = rng.standard_normal((n, n)); M = M.T @ M / n + 0.1 * np.eye(n)
        b = rng.standard_normal((n, r))
        a_off.append(ao); b_off.append(bo)
        A.append(M.T.ravel()); B.append(b.T.ravel()); mats.append(M); rhs.append(b)
        ao += n * n; bo += n * r
    Af, Bf, info = O.posv_ragged(np.concatenate(A), np.concatenate(B), a_off, b_off, ns, nr)
    assert (info == 0).all()
    for i, (n, r) in enumerate(zip(ns, nr)):
        x = Bf[b_off[i]:b_off[i] + n * r].reshape(r, n).T
        np.testing.assert_allclose(x, np.linalg.solve(mats[i], rhs[i]), rtol=1e-10, atol=1e-11)


def test_qr_golden_and_lapack():
    # tensorLeastSquares1 (test/testTensor.cu:1012-1039): square systems, residual ~ 0
    A = colmajor(G["ls1_a"], 2, 2, 3)
    b = colmajor(G["ls1_b"], 2, 1, 3)
    _, X = O.gels(A, b)
    assert np.linalg.norm(A @ X[:, :2] - b) < HIGH
    # qrLeastSquares (test/testTensor.cu:1496-1535): residual norm from MATLAB
    A = rowmajor(G["qr_ls_a_rowmajor"], 4, 3)
    b = np.array(G["qr_ls_b"]).reshape(1, 4, 1)
    _, X = O.gels(A, b)
    res = np.linalg.norm(A[0] @ X[0, :3, 0] - b[0, :, 0])
    assert abs(res - G["qr_ls_residual"]) < HIGH * 1e3  # MATLAB value printed to 17 digits
    # geqrf / ormqr agree with LAPACK dgeqrf / the explicit Q
    rng = np.random.default_rng(4)
    A = rng.standard_normal((2, 20, 3))
    QR, tau = O.geqrf(A)
    for i in range(2):
        qr_l, tau_l, _, _ = sla.lapack.dgeqrf(A[i])
        np.testing.assert_allclose(QR[i], qr_l, atol=1e-13)
        np.testing.assert_allclose(tau[i], tau_l, atol=1e-13)
    Q = O.ormqr(QR, tau, np.tile(np.eye(20)[:, :3], (2, 1, 1)), trans=False)
    np.testing.assert_allclose(Q @ np.triu(QR[:, :3, :3]), A, atol=1e-12)


def test_svd_goldens():
    # singularValuesComputation (test/testTensor.cu:1059-1084)
    B = colmajor(G["svd_b"], 8, 3)
    r = O.gesvj(B, compute_u=True)
    assert abs(r["S"][0, 0] - G["svd_sigma1"]) < HIGH
    assert abs(r["S"][0, 1] - G["svd_sigma2"]) < HIGH
    # singularValuesMultipleMatrices (test/testTensor.cu:1126-1171): signed V, S, signed U
    A = colmajor(G["svd_multi_a"], 3, 2, 3)
    r = O.gesvj(A, compute_u=True)
    Vt = r["V"].transpose(0, 2, 1)
    vt_flat = np.concatenate([Vt[i].T.ravel() for i in range(3)])
    np.testing.assert_allclose(vt_flat[:4], G["svd_multi_vt"][:4], atol=HIGH)   # the reference checks 4
    np.testing.assert_allclose(r["S"].ravel(), G["svd_multi_s"], atol=HIGH)
    u_flat = np.concatenate([r["U"][i].T.ravel() for i in range(3)])
    np.testing.assert_allclose(u_flat, G["svd_multi_u"], atol=HIGH)
    # singularValuesRankMultipleMatrices (test/testTensor.cu:1178-1199)
    A = colmajor(G["rank_a"], 4, 3, 3)
    S = O.gesvj(A)["S"]
    ranks = (S > HIGH).sum(axis=1)
    assert list(ranks) == [G["rank0"], G["rank1"], G["rank2"]]


def test_svd_random_vs_lapack():
    rng = np.random.default_rng(5)
    for (m, n) in [(32, 32), (64, 64), (40, 7), (5, 5)]:
        A = rng.standard_normal((3, m, n))
        r = O.gesvj(A, compute_u=True)
        np.testing.assert_allclose(r["S"], np.linalg.svd(A, compute_uv=False), rtol=1e-12, atol=1e-12)
        U, S, V = r["U"], r["S"], r["V"]
        rec = np.stack([U[i][:, :n] @ np.diag(S[i]) @ V[i].T for i in range(3)])
        np.testing.assert_allclose(rec, A, atol=1e-12)
        np.testing.assert_allclose(U.transpose(0, 2, 1) @ U, np.tile(np.eye(m), (3, 1, 1)), atol=1e-12)
        assert (r["info"] == 0).all()


@pytest.mark.parametrize("threads", [1, 2])
def test_oracle_threads(threads):
    O.set_threads(threads)
    rng = np.random.default_rng(6)
    A = rng.standard_normal((16, 8, 8))
    np.testing.assert_allclose(O.gemm(A, A), A @ A, atol=1e-12)
    O.set_threads(O.max_threads())
