"""One-sided Jacobi SVD and null space beyond the 64-column block kernel:
n <= 128 columns, any m >= n (GPUtils' Svd::factorise and Nullspace take any
m >= n, include/tensor.cuh:1624-1676, 2044-2085).  Against the FP64 oracle in
f32 and f64, with the working copy in shared memory and, where it does not
fit, in global memory."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import from_dev, ptr, rel_err, stream, to_dev
from tests.test_gpu_svd import _nullspace, _svd

pytestmark = pytest.mark.gpu

# (96, 96), (128, 128), (200, 128) as asked of the block kernels, plus odd
# sizes, a one-column case and shapes whose f32 / f64 working copy exceeds
# shared memory (global-memory variant)
SHAPES = [(96, 96), (128, 128), (200, 128), (150, 65), (129, 100), (256, 80), (300, 1), (70, 69), (400, 128)]


def _check(r, A, o, dt, compute_u):
    k, m, n = A.shape
    tol = 2e-6 if dt == np.float32 else 1e-12
    assert (r["info"] == 0).all(), r["sweeps"]
    smax = o["S"].max(axis=1, keepdims=True)
    # singular values: relative to sigma_max (the Jacobi stopping test is relative to column norms)
    assert np.abs(r["S"] - o["S"]).max() / smax.min() < tol * np.sqrt(m), np.abs(r["S"] - o["S"]).max()
    assert np.all(np.diff(r["S"], axis=1) <= 0)
    V = r["Vt"].transpose(0, 2, 1).astype(np.float64)
    orth = 1e-5 if dt == np.float32 else 1e-12
    assert np.abs(V.transpose(0, 2, 1) @ V - np.eye(n)).max() < orth * np.sqrt(n)
    # A V = U_n diag(S)
    AV = A.astype(np.float64) @ V
    assert rel_err(np.linalg.norm(AV, axis=1)[:, None, :], r["S"][:, None, :]) < tol * np.sqrt(m) * 10
    # sign rule: the largest-magnitude entry of each v_j is negative
    for b in range(k):
        for j in range(n):
            i = np.argmax(np.abs(V[b, :, j]))
            assert V[b, i, j] <= 0
    if compute_u:
        Uf = r["U"].astype(np.float64)
        assert np.abs(Uf.transpose(0, 2, 1) @ Uf - np.eye(m)).max() < orth * m
        rec = Uf[:, :, :n] @ (r["S"][:, :, None] * r["Vt"])
        assert rel_err(rec, A) < tol * np.sqrt(m) * 10


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_big_svd_vs_oracle(gbla_lib, cuda, shape, dt):
    m, n = shape
    rng = np.random.default_rng(m * 31 + n)
    k = 4
    A = rng.standard_normal((k, m, n)).astype(dt)
    compute_u = m <= 200
    r = _svd(gbla_lib, A, compute_u=compute_u, tol=1e-6 if dt == np.float32 else 1e-14, max_sweeps=60, dt=dt)
    o = O.gesvj(A.astype(np.float64))
    _check(r, A, o, dt, compute_u)


def test_big_svd_rank_deficient_u_completion(gbla_lib, cuda):
    """Rank 50 of 100 columns: the zero singular values come last and U is
    completed to a full orthonormal basis of R^180."""
    rng = np.random.default_rng(5)
    k, m, n, r = 3, 180, 100, 50
    A = (rng.standard_normal((k, m, r)) @ rng.standard_normal((k, r, n))).astype(np.float64)
    res = _svd(gbla_lib, A, compute_u=True, tol=1e-14, max_sweeps=60, dt=np.float64)
    assert (res["info"] == 0).all()
    assert (res["S"][:, r:] < 1e-10 * res["S"][:, :1]).all()
    U = res["U"]
    assert np.abs(U.transpose(0, 2, 1) @ U - np.eye(m)).max() < 1e-12
    assert rel_err(U[:, :, :n] @ (res["S"][:, :, None] * res["Vt"]), A) < 1e-12


def test_big_svd_warm_start_not_supported(gbla_lib, cuda):
    import torch
    m = n = 96
    A = torch.zeros(m * n, device="cuda")
    S = torch.zeros(n, device="cuda")
    Vt = torch.zeros(n * n, device="cuda")
    V0 = torch.eye(n, device="cuda")
    assert gbla_lib.gbla_sgesvj_batched(m, n, ptr(A), m * n, ptr(S), n, ptr(Vt), n * n, None, 0, ptr(V0), n * n,
                                        1e-6, 30, None, None, 1, stream()) == 2
    assert gbla_lib.gbla_sgesvj_batched(200, 129, ptr(A), 0, ptr(S), 0, ptr(Vt), 0, None, 0, None, 0,
                                        1e-6, 30, None, None, 0, stream()) == 0  # empty batch


@pytest.mark.parametrize("shape", [(100, 140), (70, 300), (128, 128), (65, 66)])
def test_big_nullspace(gbla_lib, cuda, shape):
    """Null space of fat m x n matrices beyond 64 rows (SVD of A^T, n x m,
    with the full n x n U)."""
    m, n = shape
    rng = np.random.default_rng(m + n)
    k = 4
    A = rng.standard_normal((k, m, n)).astype(np.float32)
    A[::2, -5:, :] = 0.0  # rank m - 5 for even matrices
    N, P, nul = _nullspace(gbla_lib, A)
    for i in range(k):
        rank = m - 5 if i % 2 == 0 else m
        assert nul[i] == n - rank
        if nul[i] == 0:
            assert np.abs(N[i]).max() == 0.0 and np.abs(P[i]).max() == 0.0
            continue
        Ni = N[i][:, :nul[i]].astype(np.float64)
        assert np.abs(A[i] @ Ni).max() < 1e-4 * np.sqrt(n)
        assert np.abs(Ni.T @ Ni - np.eye(nul[i])).max() < 1e-5 * np.sqrt(n)
        assert np.abs(P[i] - Ni @ Ni.T).max() < 1e-5 * np.sqrt(n)
        assert np.abs(N[i][:, nul[i]:]).max() == 0.0
