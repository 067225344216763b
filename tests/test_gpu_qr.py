"""Batched QR / least squares through the C ABI against the FP64 oracle and
the reference's golden values (leastSquaresBatched, QRFactoriser)."""
import numpy as np
import pytest

from gputils_gb300 import workloads
from oracle import oracle as O
from tests.helpers import colmajor, from_dev, goldens, ptr, rel_err, rowmajor, stream, to_dev

pytestmark = pytest.mark.gpu
G = goldens()
TOL = {np.float32: G["precision_low"], np.float64: G["precision_high"]}
PFX = {np.float32: "s", np.float64: "d"}


def _gels(lib, A, B, dt, refine=0, workspace=False):
    import torch
    k, m, n = A.shape
    nrhs = B.shape[2]
    Ad, Bd = to_dev(A, dt), to_dev(B, dt)
    info = torch.full((k,), -1, dtype=torch.int32, device="cuda")
    if dt == np.float32 and workspace:
        wsb = lib.gbla_sgels_batched_workspace_bytes(m, n, k)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        st = lib.gbla_sgels_batched_ws(m, n, nrhs, ptr(Ad), m * n, ptr(Bd), m * nrhs, ptr(info), refine, ptr(ws),
                                       wsb, k, stream())
    elif dt == np.float32:
        st = lib.gbla_sgels_batched(m, n, nrhs, ptr(Ad), m * n, ptr(Bd), m * nrhs, ptr(info), refine, k, stream())
    else:
        st = lib.gbla_dgels_batched(m, n, nrhs, ptr(Ad), m * n, ptr(Bd), m * nrhs, ptr(info), k, stream())
    assert st == 0
    return from_dev(Ad, k, m, n), from_dev(Bd, k, m, nrhs), info.cpu().numpy()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_golden_least_squares(gbla_lib, cuda, dt):
    # tensorLeastSquares1 (test/testTensor.cu:1012-1039)
    A = colmajor(G["ls1_a"], 2, 2, 3)
    b = colmajor(G["ls1_b"], 2, 1, 3)
    _, X, info = _gels(gbla_lib, A, b, dt)
    assert (info == 0).all()
    assert np.linalg.norm(A @ X[:, :2] - b) < TOL[dt]
    # qrLeastSquares (test/testTensor.cu:1496-1535): residual norm 80.003169364198072
    A = rowmajor(G["qr_ls_a_rowmajor"], 4, 3)
    b = np.array(G["qr_ls_b"]).reshape(1, 4, 1)
    _, X, _ = _gels(gbla_lib, A, b, dt)
    res = np.linalg.norm(A[0] @ X[0, :3, 0] - b[0, :, 0])
    assert abs(res - G["qr_ls_residual"]) < TOL[dt]


@pytest.mark.parametrize("shape", [(1, 1), (5, 5), (20, 3), (33, 32), (64, 17), (100, 1), (128, 32), (97, 31)])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_geqrf_ormqr_trsm_vs_oracle(gbla_lib, cuda, shape, dt):
    import torch
    m, n = shape
    rng = np.random.default_rng(m * 100 + n)
    k = 11
    A = rng.uniform(-100, 100, (k, m, n)).astype(dt)
    QRo, tauo = O.geqrf(A)
    Ad = to_dev(A, dt)
    tau = torch.zeros(k * n, dtype=Ad.dtype, device="cuda")
    p = PFX[dt]
    assert getattr(gbla_lib, f"gbla_{p}geqrf_batched")(m, n, ptr(Ad), m * n, ptr(tau), n, None, k, stream()) == 0
    QR = from_dev(Ad, k, m, n)
    tol = 5e-5 if dt == np.float32 else 1e-11
    assert rel_err(QR, QRo) < tol
    assert np.abs(tau.cpu().numpy().reshape(k, n) - tauo).max() < tol * 10
    # explicit Q (as QRFactoriser::getQR builds it, include/tensor.cuh:1929-1995), then Q R == A
    I = np.tile(np.eye(m)[:, :n], (k, 1, 1))
    Qd = to_dev(I, dt)
    assert getattr(gbla_lib, f"gbla_{p}ormqr_batched")(0, m, n, n, ptr(Ad), m * n, ptr(tau), n, ptr(Qd), m * n, k,
                                                        stream()) == 0
    Q = from_dev(Qd, k, m, n)
    assert rel_err(Q @ np.triu(QR[:, :n, :n]), A) < tol
    # least squares the QRFactoriser way: Q^T b then R^-1 (include/tensor.cuh:1891-1927)
    b = rng.standard_normal((k, m, 2)).astype(dt)
    bd = to_dev(b, dt)
    assert getattr(gbla_lib, f"gbla_{p}ormqr_batched")(1, m, 2, n, ptr(Ad), m * n, ptr(tau), n, ptr(bd), m * 2, k,
                                                        stream()) == 0
    assert getattr(gbla_lib, f"gbla_{p}trsm_upper_batched")(n, 2, ptr(Ad), m, m * n, ptr(bd), m, m * 2, k,
                                                             stream()) == 0
    x = from_dev(bd, k, m, 2)[:, :n]
    _, Xo = O.gels(A, b)
    assert rel_err(x, Xo[:, :n]) < (1e-3 if dt == np.float32 else 1e-9)


@pytest.mark.parametrize("shape", [(128, 32), (64, 64 // 2), (40, 7), (32, 32)])
def test_gels_refinement_reaches_fp64_accuracy(gbla_lib, cuda, shape):
    m, n = shape
    A, B = workloads.d2b_least_squares(k=64, m=m, n=n, nrhs=3, cond=1e3, seed=m + n)
    _, Xo = O.gels(A, B)
    _, X0, info = _gels(gbla_lib, A, B, np.float32, refine=0)
    _, X2, info2 = _gels(gbla_lib, A, B, np.float32, refine=2)
    assert (info == 0).all() and (info2 == 0).all()
    e0 = rel_err(X0[:, :n], Xo[:, :n])
    e2 = rel_err(X2[:, :n], Xo[:, :n])
    assert e2 < 1e-6, (e0, e2)
    assert e2 < e0


def test_rank_deficient_info(gbla_lib, cuda):
    A = np.zeros((2, 6, 3))
    A[0] = np.random.default_rng(0).standard_normal((6, 3))
    A[1, :, 0] = 1.0
    A[1, :, 1] = 2.0   # column 1 parallel to column 0 -> R(1,1) == 0 exactly? (not in floating point)
    A[1, :, 2] = 0.0   # zero column -> R(2,2) == 0
    _, _, info = _gels(gbla_lib, A, np.ones((2, 6, 1)), np.float64)
    assert info[0] == 0 and info[1] in (2, 3)


def test_d2b_config_full_size(gbla_lib, cuda):
    """Config D2b at full size: 8192 x (128x32), kappa = 1e3, 4 RHS, with
    refinement.  Every system: the normal-equations residual; a sample: the
    FP64 oracle at <= 1e-6."""
    A, B = workloads.d2b_least_squares()
    k, m, n = A.shape
    _, X, info = _gels(gbla_lib, A, B, np.float32, refine=1)
    assert (info == 0).all()
    x = X[:, :n].astype(np.float64)
    A64 = A.astype(np.float64)
    ne = np.linalg.norm(A64.transpose(0, 2, 1) @ (B - A64 @ x), axis=(1, 2))
    scale = np.linalg.norm(A64, axis=(1, 2)) * np.linalg.norm(B, axis=(1, 2))
    assert (ne / scale).max() < 1e-5
    idx = np.arange(0, k, 97)
    _, Xo = O.gels(A[idx], B[idx])
    assert rel_err(x[idx], Xo[:, :n]) < 1e-6


@pytest.mark.parametrize("shape", [(1, 1), (20, 3), (33, 32), (64, 17), (97, 31), (100, 32), (128, 32)])
@pytest.mark.parametrize("refine", [0, 1, 2])
@pytest.mark.parametrize("nrhs", [1, 4, 7])
def test_gels_workspace_path_is_bit_identical(gbla_lib, cuda, shape, refine, nrhs):
    """gbla_sgels_batched_ws (factor kernel + one-block-per-system solve)
    returns exactly the factors, solutions and info of gbla_sgels_batched."""
    m, n = shape
    A, B = workloads.d2b_least_squares(k=37, m=m, n=n, nrhs=nrhs, cond=1e3, seed=m * 7 + n)
    F1, X1, i1 = _gels(gbla_lib, A, B, np.float32, refine=refine)
    F2, X2, i2 = _gels(gbla_lib, A, B, np.float32, refine=refine, workspace=True)
    assert (i1 == i2).all() and (i1 == 0).all()
    assert np.array_equal(F1, F2)
    assert np.array_equal(X1, X2)


def test_gels_workspace_rank_deficient_and_too_small(gbla_lib, cuda):
    import torch
    A = np.zeros((2, 6, 3), np.float32)
    A[0] = np.random.default_rng(0).standard_normal((6, 3))
    A[1, :, 0] = 1.0
    F1, X1, i1 = _gels(gbla_lib, A, np.ones((2, 6, 2)), np.float32, refine=1)
    F2, X2, i2 = _gels(gbla_lib, A, np.ones((2, 6, 2)), np.float32, refine=1, workspace=True)
    assert (i1 == i2).all() and i2[0] == 0 and i2[1] in (2, 3)
    assert np.array_equal(F1, F2) and np.array_equal(X1, X2, equal_nan=True)
    Ad, Bd = to_dev(A, np.float32), to_dev(np.ones((2, 6, 1)), np.float32)
    wsb = gbla_lib.gbla_sgels_batched_workspace_bytes(6, 3, 2)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    assert gbla_lib.gbla_sgels_batched_ws(6, 3, 1, ptr(Ad), 18, ptr(Bd), 6, None, 1, ptr(ws), wsb - 1, 2,
                                          stream()) == 4
