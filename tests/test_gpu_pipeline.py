"""Host-buffer calls (gbla_*_host): chunks of the batch streamed through the
device over several worker streams give exactly the results of the
device-resident calls, for any chunk size, strided host layouts, pinned and
pageable memory, and beta != 0."""
import ctypes as C

import numpy as np
import pytest

from gputils_gb300 import workloads
from tests.helpers import ptr, stream

pytestmark = pytest.mark.gpu


@pytest.fixture()
def pipe(gbla_lib, cuda):
    p = C.c_void_p()
    assert gbla_lib.gbla_pipeline_create(3, C.byref(p)) == 0
    yield p
    assert gbla_lib.gbla_pipeline_destroy(p) == 0


def _host(x, pinned):
    """A host tensor holding its own copy of x (pinned or pageable)."""
    import torch
    t = torch.from_numpy(np.array(x, copy=True, order="C"))
    return t.pin_memory() if pinned else t


@pytest.mark.parametrize("chunk", [0, 1, 7, 1000])
@pytest.mark.parametrize("pinned", [True, False])
def test_gemm_host_matches_device(gbla_lib, cuda, pipe, chunk, pinned):
    import torch
    rng = np.random.default_rng(chunk + 11)
    k = 1037
    A = rng.standard_normal((k, 64, 64)).astype(np.float32)
    B = rng.standard_normal((k, 64, 64)).astype(np.float32)
    hA, hB = _host(A, pinned), _host(B, pinned)
    hC = _host(np.zeros_like(A), pinned)
    assert gbla_lib.gbla_sgemm_batched_host(pipe, 64, 64, 64, 1.0, ptr(hA), 4096, ptr(hB), 4096, 0.0, ptr(hC),
                                            4096, k, 0, chunk, stream()) == 0
    dA, dB = hA.cuda(), hB.cuda()
    dC = torch.empty_like(dA)
    assert gbla_lib.gbla_sgemm_batched(64, 64, 64, 1.0, ptr(dA), 4096, ptr(dB), 4096, 0.0, ptr(dC), 4096, k, 0,
                                       stream()) == 0
    torch.cuda.synchronize()
    assert torch.equal(hC, dC.cpu())


def test_gemm_host_strided_and_beta(gbla_lib, cuda, pipe):
    """Host strides larger than a matrix (2-D copies) and C read back in for beta != 0."""
    import torch
    rng = np.random.default_rng(5)
    k, m, n, kk = 301, 24, 16, 40
    sA, sB, sC = m * kk + 9, kk * n + 3, m * n + 17
    hA = _host(rng.standard_normal(k * sA).astype(np.float32), True)
    hB = _host(rng.standard_normal(k * sB).astype(np.float32), True)
    C0 = rng.standard_normal(k * sC).astype(np.float32)
    hC = _host(C0, True)
    assert gbla_lib.gbla_sgemm_batched_host(pipe, m, n, kk, 0.5, ptr(hA), sA, ptr(hB), sB, -2.0, ptr(hC), sC, k,
                                            1, 50, stream()) == 0
    dA, dB, dC = hA.cuda(), hB.cuda(), torch.from_numpy(C0).cuda()
    assert gbla_lib.gbla_sgemm_batched(m, n, kk, 0.5, ptr(dA), sA, ptr(dB), sB, -2.0, ptr(dC), sC, k, 1,
                                       stream()) == 0
    torch.cuda.synchronize()
    got, want = hC.numpy().reshape(k, sC), dC.cpu().numpy().reshape(k, sC)
    assert np.array_equal(got[:, :m * n], want[:, :m * n])
    assert np.array_equal(got[:, m * n:], C0.reshape(k, sC)[:, m * n:])  # padding untouched


@pytest.mark.parametrize("chunk", [0, 3, 500])
@pytest.mark.parametrize("shape", [(128, 32), (40, 7)])
def test_gels_host_matches_workspace_path(gbla_lib, cuda, pipe, chunk, shape):
    import torch
    m, n = shape
    A, B = workloads.d2b_least_squares(k=1111, m=m, n=n, nrhs=4, cond=1e3, seed=m + n)
    k, r = A.shape[0], 4
    Acm = np.ascontiguousarray(A.transpose(0, 2, 1))
    Bcm = np.ascontiguousarray(B.transpose(0, 2, 1))
    hA, hB = _host(Acm, True), _host(Bcm, True)
    hX, hF = _host(np.zeros_like(Bcm), True), _host(np.zeros_like(Acm), True)
    hI = _host(np.full(k, -1, np.int32), True)
    assert gbla_lib.gbla_sgels_batched_host(pipe, m, n, r, ptr(hA), m * n, ptr(hF), ptr(hB), m * r, ptr(hX),
                                            ptr(hI), 1, k, chunk, stream()) == 0
    dA, dB = torch.from_numpy(Acm).cuda(), torch.from_numpy(Bcm).cuda()
    info = torch.full((k,), -1, dtype=torch.int32, device="cuda")
    wsb = gbla_lib.gbla_sgels_batched_workspace_bytes(m, n, k)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    assert gbla_lib.gbla_sgels_batched_ws(m, n, r, ptr(dA), m * n, ptr(dB), m * r, ptr(info), 1, ptr(ws), wsb, k,
                                          stream()) == 0
    torch.cuda.synchronize()
    assert torch.equal(hX, dB.cpu())
    assert torch.equal(hF, dA.cpu())
    assert torch.equal(hI, info.cpu()) and int(hI.max()) == 0
    assert torch.equal(hA, torch.from_numpy(Acm))  # inputs untouched
    assert torch.equal(hB, torch.from_numpy(Bcm))


def test_gels_host_in_place_and_invalid(gbla_lib, cuda, pipe):
    import torch
    A, B = workloads.d2b_least_squares(k=64, m=33, n=5, nrhs=2, seed=1)
    Acm = np.ascontiguousarray(A.transpose(0, 2, 1))
    Bcm = np.ascontiguousarray(B.transpose(0, 2, 1))
    hA, hB = _host(Acm, False), _host(Bcm, False)
    assert gbla_lib.gbla_sgels_batched_host(pipe, 33, 5, 2, ptr(hA), 165, ptr(hA), ptr(hB), 66, ptr(hB), None, 1,
                                            64, 0, stream()) == 0
    dA, dB = torch.from_numpy(Acm).cuda(), torch.from_numpy(Bcm).cuda()
    wsb = gbla_lib.gbla_sgels_batched_workspace_bytes(33, 5, 64)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    assert gbla_lib.gbla_sgels_batched_ws(33, 5, 2, ptr(dA), 165, ptr(dB), 66, None, 1, ptr(ws), wsb, 64,
                                          stream()) == 0
    torch.cuda.synchronize()
    assert torch.equal(hA, dA.cpu()) and torch.equal(hB, dB.cpu())
    # invalid requests are refused before anything is enqueued
    assert gbla_lib.gbla_sgels_batched_host(pipe, 4, 5, 1, ptr(hA), 20, None, ptr(hB), 4, ptr(hB), None, 1, 1, 0,
                                            stream()) == 1
    assert gbla_lib.gbla_sgels_batched_host(pipe, 33, 5, 2, ptr(hA), 165, None, ptr(hB), 66, None, None, 1, 1, 0,
                                            stream()) == 1
    assert gbla_lib.gbla_sgels_batched_host(pipe, 129, 5, 1, ptr(hA), 645, None, ptr(hB), 129, ptr(hB), None, 1,
                                            1, 0, stream()) == 2
    assert gbla_lib.gbla_sgemm_batched_host(None, 4, 4, 4, 1.0, ptr(hA), 16, ptr(hA), 16, 0.0, ptr(hB), 16, 1, 0,
                                            0, stream()) == 1
