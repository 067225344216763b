"""Batched Cholesky (potrf / potrs / fused posv) through the C ABI against
the FP64 oracle and the reference's golden values."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import colmajor, from_dev, goldens, ptr, rel_err, rowmajor, spd_batch, stream, to_dev

pytestmark = pytest.mark.gpu
G = goldens()
TOL = {np.float32: G["precision_low"], np.float64: G["precision_high"]}
PFX = {np.float32: "s", np.float64: "d"}


def _potrf(lib, A_dev, n, k, dt):
    import torch
    info = torch.full((k,), -7, dtype=torch.int32, device="cuda")
    st = getattr(lib, f"gbla_{PFX[dt]}potrf_batched")(n, ptr(A_dev), n * n, ptr(info), k, stream())
    assert st == 0
    return info


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_golden_factor_and_solve(gbla_lib, cuda, dt):
    # choleskyBatchFactorisation / choleskyBatchFactorSolve (test/testTensor.cu:1282-1358)
    A = np.repeat(colmajor(G["chol_a"], 3, 3), 2, axis=0)
    Ad = to_dev(A, dt)
    info = _potrf(gbla_lib, Ad, 3, 2, dt)
    L = from_dev(Ad, 2, 3, 3)
    for i in range(2):
        assert abs(L[i, 0, 0] - G["chol_L00"]) < TOL[dt]
        assert abs(L[i, 2, 1] - G["chol_L21"]) < TOL[dt]
        assert abs(L[i, 2, 2] - G["chol_L22"]) < TOL[dt]
        assert np.array_equal(np.triu(L[i], 1), np.triu(A[i], 1).astype(dt))  # upper untouched
    assert info.cpu().tolist() == [0, 0]
    b = np.repeat(np.array(G["chol_b"]).reshape(1, 3, 1), 2, axis=0)
    bd = to_dev(b, dt)
    assert getattr(gbla_lib, f"gbla_{PFX[dt]}potrs_batched")(3, 1, ptr(Ad), 9, ptr(bd), 3, 2, stream()) == 0
    x = from_dev(bd, 2, 3, 1)
    for i in range(2):
        np.testing.assert_allclose(x[i, :, 0], G["chol_x"], atol=TOL[dt])


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_golden_prefactored_solve(gbla_lib, cuda, dt):
    # choleskyBatchSolve with a supplied L (test/testTensor.cu:1364-1413)
    low = np.repeat(rowmajor(G["chol_low_rowmajor"], 3, 3), 2, axis=0)
    Ld = to_dev(low, dt)
    bd = to_dev(np.repeat(np.array(G["chol_b"]).reshape(1, 3, 1), 2, axis=0), dt)
    assert getattr(gbla_lib, f"gbla_{PFX[dt]}potrs_batched")(3, 1, ptr(Ld), 9, ptr(bd), 3, 2, stream()) == 0
    x = from_dev(bd, 2, 3, 1)
    np.testing.assert_allclose(x[:, :, 0], np.array([G["chol_x"]] * 2), atol=TOL[dt])


NS = [1, 2, 3, 5, 8, 9, 15, 16, 17, 31, 32, 33, 48, 64, 65, 100, 127, 128]


@pytest.mark.parametrize("n", NS)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_random_factor_solve_vs_oracle(gbla_lib, cuda, n, dt):
    rng = np.random.default_rng(100 + n)
    k = 37
    M = spd_batch(rng, k, n, shift=0.1).astype(dt)
    nrhs = 3
    b = rng.standard_normal((k, n, nrhs)).astype(dt)
    Lref, info_ref = O.potrf(M)
    xref = O.potrs(Lref, b)
    Ad = to_dev(M, dt)
    info = _potrf(gbla_lib, Ad, n, k, dt)
    assert (info.cpu().numpy() == 0).all()
    L = from_dev(Ad, k, n, n)
    tol = 2e-5 if dt == np.float32 else 1e-12
    assert rel_err(np.tril(L), np.tril(Lref)) < tol
    assert np.array_equal(np.triu(L, 1), np.triu(M, 1))
    bd = to_dev(b, dt)
    assert getattr(gbla_lib, f"gbla_{PFX[dt]}potrs_batched")(n, nrhs, ptr(Ad), n * n, ptr(bd), n * nrhs, k,
                                                              stream()) == 0
    x = from_dev(bd, k, n, nrhs)
    assert rel_err(x, xref) < (5e-5 if dt == np.float32 else 1e-11)


@pytest.mark.parametrize("n", [3, 16, 32, 48, 128])
@pytest.mark.parametrize("refine", [0, 2])
def test_fused_posv_refinement(gbla_lib, cuda, n, refine):
    import torch
    rng = np.random.default_rng(7 + n)
    k, nrhs = 29, 5
    M = spd_batch(rng, k, n, shift=0.1).astype(np.float32)
    b = rng.standard_normal((k, n, nrhs)).astype(np.float32)
    _, xref, _ = O.posv(M, b)
    Ad, bd = to_dev(M, np.float32), to_dev(b, np.float32)
    info = torch.full((k,), -1, dtype=torch.int32, device="cuda")
    assert gbla_lib.gbla_sposv_batched(n, nrhs, ptr(Ad), n * n, ptr(bd), n * nrhs, ptr(info), refine, k,
                                       stream()) == 0
    assert (info.cpu().numpy() == 0).all()
    err = rel_err(from_dev(bd, k, n, nrhs), xref)
    # FP32 factor: O(kappa * u); with extended-precision residual refinement: ~u
    assert err < (1e-6 if refine else 5e-5), err
    L = from_dev(Ad, k, n, n)
    Lref, _ = O.potrf(M)
    assert rel_err(np.tril(L), np.tril(Lref)) < 2e-5


def test_info_reports_first_bad_minor(gbla_lib, cuda):
    for n in (4, 20, 60):
        M = np.tile(np.eye(n), (3, 1, 1))
        M[1, 2, 2] = -1.0   # minor of order 3 fails
        M[2, n - 1, n - 1] = 0.0
        Ad = to_dev(M, np.float32)
        info = _potrf(gbla_lib, Ad, n, 3, np.float32)
        assert info.cpu().tolist() == [0, 3, n]


def test_d1_config_full_size_residual(gbla_lib, cuda):
    """Config D1 at full size: 4096 SPD 16x16 fp32, M = G^T G / 16 + I, one RHS.
    Size-independent check on every matrix (residual), oracle on a sample."""
    import torch
    rng = np.random.default_rng(2024)
    k, n = 4096, 16
    M = spd_batch(rng, k, n, shift=1.0, scale=16.0).astype(np.float32)
    b = rng.standard_normal((k, n, 1)).astype(np.float32)
    Ad, bd = to_dev(M, np.float32), to_dev(b, np.float32)
    info = torch.empty(k, dtype=torch.int32, device="cuda")
    assert gbla_lib.gbla_spotrf_batched(n, ptr(Ad), n * n, ptr(info), k, stream()) == 0
    assert gbla_lib.gbla_spotrs_batched(n, 1, ptr(Ad), n * n, ptr(bd), n, k, stream()) == 0
    x = from_dev(bd, k, n, 1).astype(np.float64)
    assert (info.cpu().numpy() == 0).all()
    res = np.linalg.norm(M.astype(np.float64) @ x - b, axis=(1, 2)) / np.linalg.norm(b, axis=(1, 2))
    assert res.max() < 1e-5
    idx = np.arange(0, k, 64)
    _, xref, _ = O.posv(M[idx], b[idx])
    assert rel_err(x[idx], xref) < 1e-6


# beyond 128: shared-memory working copy up to ~230 (f32) / ~160 (f64), then
# factored in place in global memory
BIG_NS = {np.float32: [129, 150, 200, 231, 300, 520], np.float64: [129, 150, 161, 200, 400]}


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("which", range(5))
def test_big_potrf_potrs_vs_oracle(gbla_lib, cuda, dt, which):
    """CholeskyBatchFactoriser::factorise + solve for n > 128 (cusolverDn
    potrfBatched has no size cap, include/tensor.cuh:2135-2197)."""
    n = BIG_NS[dt][which]
    rng = np.random.default_rng(n)
    k = 5
    A = spd_batch(rng, k, n, shift=0.5)
    Ad = to_dev(A, dt)
    info = _potrf(gbla_lib, Ad, n, k, dt)
    assert (info.cpu().numpy() == 0).all()
    L = from_dev(Ad, k, n, n)
    Lo, _ = O.potrf(A)
    tol = 2e-6 if dt == np.float32 else 1e-13
    assert rel_err(np.tril(L), np.tril(Lo)) < tol * np.sqrt(n)
    assert np.array_equal(np.triu(L, 1), np.triu(A.astype(dt), 1))  # strict upper triangle untouched
    b = rng.standard_normal((k, n, 3))
    bd = to_dev(b, dt)
    assert getattr(gbla_lib, f"gbla_{PFX[dt]}potrs_batched")(n, 3, ptr(Ad), n * n, ptr(bd), n * 3, k, stream()) == 0
    _, xo, _ = O.posv(A, b)
    kappa = max(np.linalg.cond(A[i]) for i in range(k))
    assert rel_err(from_dev(bd, k, n, 3), xo) < tol * kappa * np.sqrt(n)


@pytest.mark.parametrize("n,dt", [(150, np.float32), (200, np.float32), (231, np.float32), (140, np.float64),
                                  (161, np.float64)])
def test_big_posv_refined_vs_oracle(gbla_lib, cuda, n, dt):
    """Fused factor + solve with refinement above n = 128 (the residual runs
    over the whole original lower triangle, row by row)."""
    import torch
    rng = np.random.default_rng(n + 1)
    k = 4
    A = spd_batch(rng, k, n, shift=0.1)
    A[:, np.triu_indices(n, 1)[0], np.triu_indices(n, 1)[1]] = 7.0  # upper triangle is never read
    b = rng.standard_normal((k, n, 2))
    Ad, bd = to_dev(A, dt), to_dev(b, dt)
    info = torch.full((k,), -1, dtype=torch.int32, device="cuda")
    assert getattr(gbla_lib, f"gbla_{PFX[dt]}posv_batched")(n, 2, ptr(Ad), n * n, ptr(bd), n * 2, ptr(info), 2, k,
                                                             stream()) == 0
    assert (info.cpu().numpy() == 0).all()
    Afull = np.tril(A) + np.tril(A, -1).transpose(0, 2, 1)
    _, xo, _ = O.posv(Afull, b)
    assert rel_err(from_dev(bd, k, n, 2), xo) < (1e-6 if dt == np.float32 else 1e-13)


def test_big_posv_global_memory_refinement_refused(gbla_lib, cuda):
    import torch
    n, k = 300, 2
    A = spd_batch(np.random.default_rng(2), k, n, shift=0.5)
    b = np.ones((k, n, 1))
    Ad, bd = to_dev(A, np.float32), to_dev(b, np.float32)
    info = torch.zeros(k, dtype=torch.int32, device="cuda")
    assert gbla_lib.gbla_sposv_batched(n, 1, ptr(Ad), n * n, ptr(bd), n, ptr(info), 1, k, stream()) == 2
    assert gbla_lib.gbla_sposv_batched(n, 1, ptr(Ad), n * n, ptr(bd), n, ptr(info), 0, k, stream()) == 0
    _, xo, _ = O.posv(A, b)
    assert rel_err(from_dev(bd, k, n, 1), xo) < 1e-3


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_big_not_positive_definite_info(gbla_lib, cuda, dt):
    n = 300 if dt == np.float32 else 200   # global-memory variant
    A = spd_batch(np.random.default_rng(4), 2, n, shift=0.5)
    A[1, 57, 57] = -1e3                    # leading minor of order 58 is not positive definite
    Ad = to_dev(A, dt)
    info = _potrf(gbla_lib, Ad, n, 2, dt)
    assert info.cpu().tolist() == [0, 58]
