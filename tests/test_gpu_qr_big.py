"""QR, Q application and least squares beyond the warp kernels' 128 x 32
(one block per matrix, any m >= n): against the FP64 oracle, f32 and f64,
with the matrix in shared memory and, for the largest shapes, worked on in
global memory (GPUtils' geqrf / ormqr / trsm / gelsBatched accept any m >= n,
include/tensor.cuh:1340-1394, 1866-1927)."""
import numpy as np
import pytest

from gputils_gb300 import workloads
from oracle import oracle as O
from tests.helpers import from_dev, ptr, rel_err, stream, to_dev

pytestmark = pytest.mark.gpu
PFX = {np.float32: "s", np.float64: "d"}
# shapes: shared-memory working copy for all but the last two of each type
# (f32 600 x 100 and f64 256 x 128 exceed 227 KB and run in global memory)
SHAPES = [(128, 64), (100, 50), (128, 128), (256, 100), (129, 1), (300, 40), (40, 33), (64, 64)]
GLOBAL_SHAPES = {np.float32: [(600, 100), (1030, 64)], np.float64: [(256, 128), (400, 90)]}


def _geqrf(lib, A, dt):
    import torch
    k, m, n = A.shape
    Ad = to_dev(A, dt)
    tau = torch.zeros(k * n, dtype=Ad.dtype, device="cuda")
    info = torch.full((k,), -1, dtype=torch.int32, device="cuda")
    assert getattr(lib, f"gbla_{PFX[dt]}geqrf_batched")(m, n, ptr(Ad), m * n, ptr(tau), n, ptr(info), k,
                                                         stream()) == 0
    return Ad, tau, info.cpu().numpy()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("which", range(len(SHAPES) + 2))
def test_geqrf_ormqr_trsm_big_vs_oracle(gbla_lib, cuda, dt, which):
    m, n = (SHAPES + GLOBAL_SHAPES[dt])[which]
    rng = np.random.default_rng(m * 1000 + n)
    k = 6
    A = rng.uniform(-1, 1, (k, m, n)).astype(dt)
    QRo, tauo = O.geqrf(A)
    Ad, tau, info = _geqrf(gbla_lib, A, dt)
    assert (info == 0).all()
    QR = from_dev(Ad, k, m, n)
    kappa = max(np.linalg.cond(A[i].astype(np.float64)) for i in range(k))
    tol = (2e-6 if dt == np.float32 else 1e-14) * kappa * np.sqrt(m)
    assert rel_err(QR, QRo) < tol
    assert np.abs(tau.cpu().numpy().reshape(k, n) - tauo).max() < tol * 10
    # explicit Q (QRFactoriser::getQR), Q R == A and Q^T Q == I
    p = PFX[dt]
    I = np.tile(np.eye(m)[:, :n], (k, 1, 1))
    Qd = to_dev(I, dt)
    assert getattr(gbla_lib, f"gbla_{p}ormqr_batched")(0, m, n, n, ptr(Ad), m * n, ptr(tau), n, ptr(Qd), m * n, k,
                                                        stream()) == 0
    Q = from_dev(Qd, k, m, n).astype(np.float64)
    eps = 1e-6 if dt == np.float32 else 1e-14
    assert rel_err(Q @ np.triu(QR[:, :n, :n]), A) < eps * np.sqrt(m) * 10
    assert np.abs(Q.transpose(0, 2, 1) @ Q - np.eye(n)).max() < eps * m
    # QRFactoriser::leastSquares: Q^T b, then R^-1 (ormqr + trsm)
    b = rng.standard_normal((k, m, 3)).astype(dt)
    bd = to_dev(b, dt)
    assert getattr(gbla_lib, f"gbla_{p}ormqr_batched")(1, m, 3, n, ptr(Ad), m * n, ptr(tau), n, ptr(bd), m * 3, k,
                                                        stream()) == 0
    assert getattr(gbla_lib, f"gbla_{p}trsm_upper_batched")(n, 3, ptr(Ad), m, m * n, ptr(bd), m, m * 3, k,
                                                             stream()) == 0
    x = from_dev(bd, k, m, 3)[:, :n]
    _, Xo = O.gels(A, b)
    assert rel_err(x, Xo[:, :n]) < tol * kappa


def _gels(lib, A, B, dt, refine):
    import torch
    k, m, n = A.shape
    nrhs = B.shape[2]
    Ad, Bd = to_dev(A, dt), to_dev(B, dt)
    info = torch.full((k,), -1, dtype=torch.int32, device="cuda")
    if dt == np.float32:
        st = lib.gbla_sgels_batched(m, n, nrhs, ptr(Ad), m * n, ptr(Bd), m * nrhs, ptr(info), refine, k, stream())
    else:
        st = lib.gbla_dgels_batched(m, n, nrhs, ptr(Ad), m * n, ptr(Bd), m * nrhs, ptr(info), k, stream())
    return st, Ad, from_dev(Bd, k, m, nrhs), info.cpu().numpy()


@pytest.mark.parametrize("shape", [(128, 64), (100, 50), (128, 128), (256, 100), (200, 33), (70, 70)])
@pytest.mark.parametrize("nrhs", [1, 4, 11])
def test_sgels_big_refined_vs_oracle(gbla_lib, cuda, shape, nrhs):
    """Single precision with refinement reaches FP64-level accuracy at
    kappa = 1e3, like the 128 x 32 path; without refinement it is FP32-level."""
    m, n = shape
    A, B = workloads.d2b_least_squares(k=8, m=m, n=n, nrhs=nrhs, cond=1e3, seed=m * 3 + n)
    _, Xo = O.gels(A, B)
    st0, _, X0, i0 = _gels(gbla_lib, A, B, np.float32, 0)
    st1, F1, X1, i1 = _gels(gbla_lib, A, B, np.float32, 1)
    st2, _, X2, i2 = _gels(gbla_lib, A, B, np.float32, 2)
    assert st0 == st1 == st2 == 0
    assert (i0 == 0).all() and (i1 == 0).all() and (i2 == 0).all()
    e0 = rel_err(X0[:, :n], Xo[:, :n])
    e1 = rel_err(X1[:, :n], Xo[:, :n])
    e2 = rel_err(X2[:, :n], Xo[:, :n])
    assert e0 < 1e-3 and e1 < 1e-6 and e2 < 1e-6, (e0, e1, e2)
    # rows >= n: (Q^T b)(n:m), whose norm is the residual norm
    if m > n:
        r = np.linalg.norm(B.astype(np.float64) - A.astype(np.float64) @ Xo[:, :n], axis=1)
        assert np.allclose(np.linalg.norm(X1[:, n:].astype(np.float64), axis=1), r, rtol=1e-4)
    # factors as geqrf leaves them
    QRo, _ = O.geqrf(A)
    assert rel_err(from_dev(F1, 8, m, n), QRo) < 1e-4


@pytest.mark.parametrize("shape", [(128, 64), (256, 100), (128, 128), (256, 128), (400, 90)])
def test_dgels_big_vs_oracle(gbla_lib, cuda, shape):
    m, n = shape
    A, B = workloads.d2b_least_squares(k=5, m=m, n=n, nrhs=3, cond=1e3, seed=m + n)
    A, B = A.astype(np.float64), B.astype(np.float64)
    _, Xo = O.gels(A, B)
    st, _, X, info = _gels(gbla_lib, A, B, np.float64, 0)
    assert st == 0 and (info == 0).all()
    assert rel_err(X[:, :n], Xo[:, :n]) < 1e-11


def test_sgels_global_memory_shapes(gbla_lib, cuda):
    """Beyond shared memory: without refinement the factorisation runs in A
    (global memory); refinement needs the original A beside the working copy
    and is refused (GBLA_NOT_SUPPORTED) there."""
    m, n = 600, 100
    A, B = workloads.d2b_least_squares(k=3, m=m, n=n, nrhs=2, cond=1e2, seed=9)
    _, Xo = O.gels(A, B)
    st, _, X, info = _gels(gbla_lib, A, B, np.float32, 0)
    assert st == 0 and (info == 0).all()
    assert rel_err(X[:, :n], Xo[:, :n]) < 1e-4
    st, _, _, _ = _gels(gbla_lib, A, B, np.float32, 1)
    assert st == 2


def test_big_rank_deficient_info(gbla_lib, cuda):
    A = np.random.default_rng(1).standard_normal((2, 150, 60))
    A[1, :, 40] = 0.0   # zero column -> R(40, 40) == 0 exactly
    A[1, :, 41:] = 0.0
    for dt in (np.float32, np.float64):
        _, _, info = _geqrf(gbla_lib, A, dt)
        assert info[0] == 0 and info[1] == 41
