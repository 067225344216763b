"""One large SPD matrix factored on the whole GPU (gbla_spotrf_large): the
diagonal blocks on one thread block, the panels below them on many, the
trailing updates on the tensor cores (BF16x3 split, FP32 accumulation).
The reference's CholeskyFactoriser calls cusolverDnSpotrf for this
(include/tensor.cuh:1703-1709 workspace, 1754-1761 factorise); checked here
against the FP64 oracle, the single-block batched path and the LAPACK info
convention."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import from_dev, ptr, rel_err, spd_batch, stream, to_dev

pytestmark = pytest.mark.gpu


def _factor_large(lib, A, lda=None):
    """A: (n, n) float64 SPD.  Returns (factored matrix as (n, n) float32, info)."""
    import torch

    n = A.shape[0]
    lda = n if lda is None else lda
    buf = np.full((n, lda), np.float32(7.5), dtype=np.float32)  # column-major storage: buf[j, i] = A(i, j)
    buf[:, :n] = A.T.astype(np.float32)
    Ad = torch.from_numpy(buf).cuda()
    ws = torch.empty(max(1, lib.gbla_spotrf_large_workspace_bytes(n)), dtype=torch.uint8, device="cuda")
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    st = lib.gbla_spotrf_large(n, ptr(Ad), lda, ptr(info), ptr(ws), ws.numel(), stream())
    assert st == 0
    out = Ad.cpu().numpy()
    assert np.all(out[:, n:] == np.float32(7.5))  # rows beyond n of each column untouched
    return out[:, :n].T.copy(), int(info.item())


@pytest.mark.parametrize("n", [1, 100, 128, 129, 200, 256, 300, 640, 1000, 1536])
def test_large_potrf_vs_oracle(gbla_lib, cuda, n):
    rng = np.random.default_rng(1000 + n)
    A = spd_batch(rng, 1, n, shift=0.5)[0]
    L, info = _factor_large(gbla_lib, A)
    assert info == 0
    Lo, oinfo = O.potrf(A[None])
    assert int(oinfo[0]) == 0
    assert rel_err(np.tril(L)[None], np.tril(Lo[0])[None]) < 4e-6 * np.sqrt(n)
    assert np.array_equal(np.triu(L, 1), np.triu(A.astype(np.float32), 1))  # strict upper triangle untouched
    # the factor reproduces A to FP32 accuracy
    Lt = np.tril(L).astype(np.float64)
    assert np.linalg.norm(Lt @ Lt.T - A) / np.linalg.norm(A) < 2e-6 * np.sqrt(n)


@pytest.mark.parametrize("n,lda", [(300, 305), (520, 640)])
def test_large_potrf_leading_dimension(gbla_lib, cuda, n, lda):
    rng = np.random.default_rng(n + lda)
    A = spd_batch(rng, 1, n, shift=0.5)[0]
    L, info = _factor_large(gbla_lib, A, lda)
    Lo, _ = O.potrf(A[None])
    assert info == 0
    assert rel_err(np.tril(L)[None], np.tril(Lo[0])[None]) < 4e-6 * np.sqrt(n)


@pytest.mark.parametrize("n", [300, 640])
def test_large_potrf_matches_single_block_path(gbla_lib, cuda, n):
    """Same factor as gbla_spotrf_batched with batch = 1, to FP32 accuracy."""
    import torch

    rng = np.random.default_rng(7 * n)
    A = spd_batch(rng, 1, n, shift=0.5)
    L, _ = _factor_large(gbla_lib, A[0])
    Ad = to_dev(A, np.float32)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert gbla_lib.gbla_spotrf_batched(n, ptr(Ad), n * n, ptr(info), 1, stream()) == 0
    Lb = from_dev(Ad, 1, n, n)[0]
    assert rel_err(np.tril(L)[None], np.tril(Lb)[None]) < 4e-6 * np.sqrt(n)


@pytest.mark.parametrize("n,bad", [(640, 300), (640, 0), (1000, 999), (300, 128)])
def test_large_potrf_info_first_failing_minor(gbla_lib, cuda, n, bad):
    """info = j when the leading minor of order j is the first that is not
    positive definite (LAPACK / cuSOLVER convention), also when the failure
    lies past the first panels."""
    rng = np.random.default_rng(n + bad)
    A = spd_batch(rng, 1, n, shift=0.5)[0]
    A[bad, bad] = -50.0
    _, info = _factor_large(gbla_lib, A)
    _, oinfo = O.potrf(A[None])
    assert info == bad + 1 == int(oinfo[0])


def test_large_potrf_bad_arguments(gbla_lib, cuda):
    import torch

    A = torch.zeros(300 * 300, dtype=torch.float32, device="cuda")
    ws = torch.empty(16, dtype=torch.uint8, device="cuda")
    assert gbla_lib.gbla_spotrf_large(300, ptr(A), 299, None, ptr(ws), 16, stream()) == 1   # lda < n
    assert gbla_lib.gbla_spotrf_large(300, ptr(A), 300, None, ptr(ws), 16, stream()) != 0   # workspace too small
    assert gbla_lib.gbla_spotrf_large(0, None, 1, None, None, 0, stream()) == 0
    assert gbla_lib.gbla_spotrf_large_workspace_bytes(128) == 0  # one panel: no trailing update
    assert gbla_lib.gbla_spotrf_large_workspace_bytes(129) >= 2 * 129 * 768 * 2


def test_large_potrf_repeat_and_graph_replay(gbla_lib, cuda):
    """The look-ahead (a side stream joined by events) gives the same bits on
    repeated calls and when the call is captured in a CUDA graph and replayed
    (the first call on the thread, made before the capture, creates the side
    stream)."""
    import torch

    n = 700
    rng = np.random.default_rng(700)
    A0 = torch.from_numpy(spd_batch(rng, 1, n, shift=0.5)[0].T.astype(np.float32).copy()).cuda()
    ws = torch.empty(gbla_lib.gbla_spotrf_large_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    side = torch.cuda.Stream()
    outs = []
    with torch.cuda.stream(side):
        for _ in range(2):
            A = A0.clone()
            assert gbla_lib.gbla_spotrf_large(n, ptr(A), n, ptr(info), ptr(ws), ws.numel(), side.cuda_stream) == 0
            outs.append(A)
    torch.cuda.synchronize()
    assert torch.equal(outs[0], outs[1])
    A = torch.empty_like(A0)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        A.copy_(A0)
        assert gbla_lib.gbla_spotrf_large(n, ptr(A), n, ptr(info), ptr(ws), ws.numel(), side.cuda_stream) == 0
    for _ in range(2):
        A.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(A, outs[0])
        assert int(info.item()) == 0


@pytest.mark.parametrize("n,nrhs", [(129, 1), (300, 3), (640, 1), (1000, 5), (1536, 2)])
def test_large_potrs_vs_oracle(gbla_lib, cuda, n, nrhs):
    """gbla_spotrs_large (blocked solve with one factor, the drop-in
    CholeskyFactoriser<float>::solve above n = 128) against the FP64 oracle,
    with the factor from gbla_spotrf_large, and against the single-block
    gbla_spotrs_batched on the same factor."""
    import torch

    rng = np.random.default_rng(3 * n + nrhs)
    A = spd_batch(rng, 1, n, shift=0.5)[0]
    L, info = _factor_large(gbla_lib, A)
    assert info == 0
    b = rng.standard_normal((n, nrhs))
    Ld = torch.from_numpy(L.T.copy()).cuda()  # column-major
    ldb = n + 3
    Bbuf = np.full((nrhs, ldb), np.float32(-2.25), dtype=np.float32)
    Bbuf[:, :n] = b.T.astype(np.float32)
    Bd = torch.from_numpy(Bbuf).cuda()
    assert gbla_lib.gbla_spotrs_large(n, nrhs, ptr(Ld), n, ptr(Bd), ldb, stream()) == 0
    out = Bd.cpu().numpy()
    assert np.all(out[:, n:] == np.float32(-2.25))  # rows beyond n untouched
    x = out[:, :n].T.astype(np.float64)
    _, xo, _ = O.posv(A[None], b[None])
    kappa = np.linalg.cond(A)
    assert rel_err(x[None], xo) < 2e-6 * kappa * np.sqrt(n)
    # the single-block path on the same factor
    B1 = torch.from_numpy(np.ascontiguousarray(b.T.astype(np.float32))).cuda()
    assert gbla_lib.gbla_spotrs_batched(n, nrhs, ptr(Ld), n * n, ptr(B1), n * nrhs, 1, stream()) == 0
    x1 = B1.cpu().numpy().T.astype(np.float64)
    assert rel_err(x[None], x1[None]) < 2e-6 * kappa * np.sqrt(n)


def test_large_potrs_bad_arguments(gbla_lib, cuda):
    assert gbla_lib.gbla_spotrs_large(300, 1, None, 299, None, 300, stream()) == 1  # lda < n
    assert gbla_lib.gbla_spotrs_large(300, 1, None, 300, None, 299, stream()) == 1  # ldb < n
    assert gbla_lib.gbla_spotrs_large(0, 1, None, 1, None, 1, stream()) == 0
    assert gbla_lib.gbla_spotrs_large(300, 0, None, 300, None, 300, stream()) == 0
