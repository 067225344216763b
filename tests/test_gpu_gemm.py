"""Batched GEMM (addAB) through the C ABI: FFMA path for every shape, the
tcgen05 BF16x6 split path for 64x64x64, against the FP64 oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import colmajor, from_dev, goldens, ptr, rel_err, stream, to_dev

pytestmark = pytest.mark.gpu
G = goldens()
FP32, BF16X6 = 1, 2


def _sgemm(lib, A, B, Cin=None, alpha=1.0, beta=0.0, mode=0, dt=np.float32):
    import torch
    k, m, kk = A.shape
    n = B.shape[2]
    Ad, Bd = to_dev(A, dt), to_dev(B, dt)
    Cd = to_dev(Cin, dt) if Cin is not None else torch.zeros(k * m * n, dtype=Ad.dtype, device="cuda")
    if dt == np.float32:
        st = lib.gbla_sgemm_batched(m, n, kk, alpha, ptr(Ad), m * kk, ptr(Bd), kk * n, beta, ptr(Cd), m * n, k,
                                    mode, stream())
    else:
        st = lib.gbla_dgemm_batched(m, n, kk, alpha, ptr(Ad), m * kk, ptr(Bd), kk * n, beta, ptr(Cd), m * n, k,
                                    stream())
    return st, from_dev(Cd, k, m, n)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_golden_addAB(gbla_lib, cuda, dt):
    # tensorAddAB (test/testTensor.cu:828-853): exact integer result
    A = colmajor(G["addAB_a"], 2, 3, 3)
    B = colmajor(G["addAB_b"], 3, 2, 3)
    st, Cm = _sgemm(gbla_lib, A, B, dt=dt)
    assert st == 0
    assert np.array_equal(Cm.transpose(0, 2, 1).ravel(), np.array(G["addAB_expected"]))


SHAPES = [(1, 1, 1), (2, 3, 4), (7, 5, 3), (16, 16, 16), (33, 17, 65), (64, 64, 64), (100, 70, 130), (128, 1, 64)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_ffma_vs_oracle(gbla_lib, cuda, shape, dt):
    m, n, kk = shape
    rng = np.random.default_rng(m * 1000 + n * 10 + kk)
    k = 9
    A = rng.uniform(-1, 1, (k, m, kk)); B = rng.uniform(-1, 1, (k, kk, n)); Cin = rng.uniform(-1, 1, (k, m, n))
    A, B, Cin = A.astype(dt), B.astype(dt), Cin.astype(dt)
    st, Cm = _sgemm(gbla_lib, A, B, Cin, alpha=0.75, beta=-1.5, mode=FP32, dt=dt)
    assert st == 0
    ref = O.gemm(A, B, Cin, 0.75, -1.5)
    assert rel_err(Cm, ref) < (2e-6 if dt == np.float32 else 1e-14)


@pytest.mark.parametrize("batch", [1, 2, 3, 17, 1000])
def test_tcgen05_bf16x6_vs_oracle(gbla_lib, cuda, batch):
    rng = np.random.default_rng(batch)
    A = rng.uniform(-1, 1, (batch, 64, 64)).astype(np.float32)
    B = rng.uniform(-1, 1, (batch, 64, 64)).astype(np.float32)
    st, Cm = _sgemm(gbla_lib, A, B, mode=BF16X6)
    assert st == 0
    assert gbla_lib.gbla_device_error_flags() == 0
    ref = O.gemm(A, B)
    err = rel_err(Cm, ref)
    assert err < 1e-6, err


def test_tcgen05_alpha_beta(gbla_lib, cuda):
    rng = np.random.default_rng(9)
    A = rng.uniform(-1, 1, (5, 64, 64)).astype(np.float32)
    B = rng.uniform(-1, 1, (5, 64, 64)).astype(np.float32)
    Cin = rng.uniform(-1, 1, (5, 64, 64)).astype(np.float32)
    st, Cm = _sgemm(gbla_lib, A, B, Cin, alpha=-2.0, beta=0.5, mode=BF16X6)
    assert st == 0
    assert rel_err(Cm, O.gemm(A, B, Cin, -2.0, 0.5)) < 1e-6


def test_d2a_config_full_size(gbla_lib, cuda):
    """Config D2a at full size: 16384 pairs of 64x64 fp32, U[-1,1].  Oracle on
    a sample of pairs; every pair checked by a size-independent identity
    (C e = A (B e) with e the all-ones vector, computed in FP64)."""
    import torch
    rng = np.random.default_rng(7)
    k = 16384
    A = rng.uniform(-1, 1, (k, 64, 64)).astype(np.float32)
    B = rng.uniform(-1, 1, (k, 64, 64)).astype(np.float32)
    st, Cm = _sgemm(gbla_lib, A, B)   # AUTO: tensor-core path
    assert st == 0
    e = np.ones((64, 1))
    lhs = Cm.astype(np.float64) @ e
    rhs = A.astype(np.float64) @ (B.astype(np.float64) @ e)
    assert (np.abs(lhs - rhs).max(axis=(1, 2)) / np.abs(rhs).max(axis=(1, 2))).max() < 1e-5
    idx = np.arange(0, k, 257)
    assert rel_err(Cm[idx], O.gemm(A[idx], B[idx])) < 1e-6
