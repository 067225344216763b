"""Ragged batched Cholesky factor + solve + refinement (gbla_{s,d}posv_ragged)
through the C ABI against the FP64 oracle's per-system potrf + potrs."""
import ctypes as C

import numpy as np
import pytest

from gputils_gb300 import workloads
from oracle import oracle as O
from tests.helpers import stream

pytestmark = pytest.mark.gpu


def _plan(lib, a_off, b_off, n, nrhs):
    p = C.c_void_p()
    a_off = np.ascontiguousarray(a_off, np.int64); b_off = np.ascontiguousarray(b_off, np.int64)
    n = np.ascontiguousarray(n, np.int32); nrhs = np.ascontiguousarray(nrhs, np.int32)
    st = lib.gbla_ragged_plan_create(a_off.ctypes.data, b_off.ctypes.data, n.ctypes.data, nrhs.ctypes.data,
                                     len(n), C.byref(p))
    return st, p


def _solve(lib, n, nrhs, a_off, b_off, A, B, dt, refine):
    import torch
    st, plan = _plan(lib, a_off, b_off, n, nrhs)
    assert st == 0
    Ad = torch.tensor(A.astype(dt)).cuda()
    Bd = torch.tensor(B.astype(dt)).cuda()
    info = torch.full((len(n),), -1, dtype=torch.int32, device="cuda")
    fn = lib.gbla_sposv_ragged if dt == np.float32 else lib.gbla_dposv_ragged
    assert fn(plan, Ad.data_ptr(), Bd.data_ptr(), info.data_ptr(), refine, stream()) == 0
    torch.cuda.synchronize()
    assert lib.gbla_ragged_plan_destroy(plan) == 0
    return Ad.cpu().numpy(), Bd.cpu().numpy(), info.cpu().numpy()


def _max_rel_err(n, nrhs, b_off, X, Xref):
    worst = 0.0
    for i in range(len(n)):
        sl = slice(b_off[i], b_off[i] + n[i] * nrhs[i])
        if nrhs[i] == 0:
            continue
        d = np.linalg.norm(X[sl].astype(np.float64) - Xref[sl]) / np.linalg.norm(Xref[sl])
        worst = max(worst, d)
    return worst


@pytest.mark.parametrize("dt,refine,tol", [(np.float32, 0, 5e-5), (np.float32, 1, 1e-6), (np.float32, 2, 1e-6),
                                           (np.float64, 0, 5e-5), (np.float64, 2, 1e-11), (np.float64, 3, 1e-13)])
def test_mixed_sizes_vs_oracle(gbla_lib, cuda, dt, refine, tol):
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(count=700, seed=21, dtype=np.float64)
    Af, Xf, info = _solve(gbla_lib, n, nrhs, a_off, b_off, A, B, dt, refine)
    Ao, Xo, info_o = O.posv_ragged(A.astype(dt), B.astype(dt), a_off, b_off, n, nrhs)
    assert (info == 0).all() and (info_o == 0).all()
    err = _max_rel_err(n, nrhs, b_off, Xf, Xo)
    assert err < tol, err
    # L in place (FP32 factor), strict upper triangle untouched
    for i in range(0, len(n), 37):
        k = n[i]
        L = Af[a_off[i]:a_off[i] + k * k].reshape(k, k).T
        Lo = Ao[a_off[i]:a_off[i] + k * k].reshape(k, k).T
        assert np.abs(np.tril(L) - np.tril(Lo)).max() < 5e-5 * np.abs(Lo).max()
        Ain = A[a_off[i]:a_off[i] + k * k].reshape(k, k).T.astype(dt)
        assert np.array_equal(np.triu(L, 1), np.triu(Ain, 1))


def test_edges_and_info(gbla_lib, cuda):
    rng = np.random.default_rng(5)
    ns = [1, 8, 9, 16, 17, 32, 33, 64, 128, 5, 40]
    rhs = [1, 0, 8, 3, 1, 2, 5, 1, 8, 2, 3]
    mats, a_off, b_off, Bs = [], [], [], []
    ao = bo = 0
    for k, (nn, r) in enumerate(zip(ns, rhs)):
        G = rng.standard_normal((nn, nn))
        M = G.T @ G / nn + 0.1 * np.eye(nn)
        if k == 9:
            M[3, 3] = -5.0      # leading minor 4 fails
        if k == 10:
            M[39, 39] = -1.0    # last minor fails (large path)
        mats.append(M.T.ravel()); a_off.append(ao); ao += nn * nn
        Bs.append(rng.standard_normal(nn * r)); b_off.append(bo); bo += nn * r
    A, B = np.concatenate(mats), np.concatenate(Bs)
    _, X, info = _solve(gbla_lib, np.array(ns), np.array(rhs), np.array(a_off), np.array(b_off), A, B,
                        np.float32, 1)
    assert list(info[:9]) == [0] * 9 and info[9] == 4 and info[10] == 40
    _, Xo, _ = O.posv_ragged(A.astype(np.float32), B.astype(np.float32), a_off, b_off, ns, rhs)
    assert _max_rel_err(ns[:9], rhs[:9], b_off[:9], X, Xo) < 1e-6


def test_invalid_plans(gbla_lib, cuda):
    st, _ = _plan(gbla_lib, [0], [0], [0], [1])
    assert st == 1
    st, _ = _plan(gbla_lib, [0], [0], [129], [1])
    assert st == 1
    st, p = _plan(gbla_lib, [], [], [], [])
    assert st == 0
    assert gbla_lib.gbla_sposv_ragged(p, None, None, None, 1, stream()) == 0   # empty plan: no-op
    assert gbla_lib.gbla_sragged_autotune(p, None, None, 1, 1, None, None, stream()) == 0
    assert gbla_lib.gbla_ragged_plan_destroy(p) == 0


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_d3_config_full_size(gbla_lib, cuda, dt):
    """Config D3 at full size: 20000 systems, n log-uniform in [4,128], nrhs 1..8.
    Every system: relative residual; a sample: the FP64 oracle at <= 1e-6."""
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(dtype=np.float64)
    refine = 1 if dt == np.float32 else 2
    _, X, info = _solve(gbla_lib, n, nrhs, a_off, b_off, A, B, dt, refine)
    assert (info == 0).all()
    idx = np.arange(0, len(n), 97)
    sub = lambda arr, off, sz: np.concatenate([arr[off[i]:off[i] + sz[i]] for i in idx])
    a_sz, b_sz = n.astype(np.int64) ** 2, n.astype(np.int64) * nrhs
    As, Bs = sub(A, a_off, a_sz), sub(B, b_off, b_sz)
    a2 = np.concatenate([[0], np.cumsum(a_sz[idx])[:-1]]); b2 = np.concatenate([[0], np.cumsum(b_sz[idx])[:-1]])
    _, Xo, _ = O.posv_ragged(As.astype(dt), Bs.astype(dt), a2, b2, n[idx], nrhs[idx])
    Xs = sub(X, b_off, b_sz)
    assert _max_rel_err(n[idx], nrhs[idx], b2, Xs, Xo) < 1e-6
    worst = 0.0
    for i in range(0, len(n), 13):
        k, r = n[i], nrhs[i]
        M = A[a_off[i]:a_off[i] + k * k].reshape(k, k).T
        b = B[b_off[i]:b_off[i] + k * r].reshape(r, k).T
        x = X[b_off[i]:b_off[i] + k * r].reshape(r, k).T.astype(np.float64)
        worst = max(worst, np.linalg.norm(M @ x - b) / np.linalg.norm(b))
    assert worst < 1e-6


class Cfg(C.Structure):
    _fields_ = [("threads", C.c_int), ("systems_per_block", C.c_int)]


CONFIGS = [(128, 1), (128, 2), (256, 1), (256, 2), (256, 4), (512, 1), (512, 2), (512, 4), (512, 8), (768, 1),
           (768, 2), (768, 4), (768, 8)]


def test_config_get_set_and_invalid(gbla_lib, cuda):
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(count=200, seed=3, dtype=np.float64)
    st, p = _plan(gbla_lib, a_off, b_off, n, nrhs)
    assert st == 0
    c = Cfg()
    assert gbla_lib.gbla_ragged_plan_get_config(p, C.byref(c)) == 0
    assert (c.threads, c.systems_per_block) == (256, 2)
    for bad in (Cfg(64, 1), Cfg(256, 3), Cfg(128, 4), Cfg(256, 8), Cfg(1024, 1), Cfg(768, 16)):
        assert gbla_lib.gbla_ragged_plan_set_config(p, C.byref(bad)) == 1
    assert gbla_lib.gbla_ragged_plan_set_config(p, C.byref(Cfg(512, 8))) == 0
    assert gbla_lib.gbla_ragged_plan_get_config(p, C.byref(c)) == 0
    assert (c.threads, c.systems_per_block) == (512, 8)
    ntasks, smem = C.c_int(), C.c_size_t()
    assert gbla_lib.gbla_ragged_plan_tasks(p, C.byref(ntasks), C.byref(smem)) == 0
    assert 0 < ntasks.value <= len(n) and 0 < smem.value <= 226 * 1024
    assert gbla_lib.gbla_ragged_plan_destroy(p) == 0


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_every_configuration_gives_identical_results_and_autotune_keeps_inputs(gbla_lib, cuda, dt):
    import torch
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(count=3000, seed=8, dtype=np.float64)
    st, p = _plan(gbla_lib, a_off, b_off, n, nrhs)
    assert st == 0
    Ah, Bh = torch.tensor(A.astype(dt)).cuda(), torch.tensor(B.astype(dt)).cuda()
    fn = gbla_lib.gbla_sposv_ragged if dt == np.float32 else gbla_lib.gbla_dposv_ragged
    tune = gbla_lib.gbla_sragged_autotune if dt == np.float32 else gbla_lib.gbla_dragged_autotune
    refine = 1 if dt == np.float32 else 2

    def run(times=1):
        for _ in range(times):  # repeated calls: the queue counter resets itself
            Ad, Bd = Ah.clone(), Bh.clone()
            info = torch.full((len(n),), -1, dtype=torch.int32, device="cuda")
            assert fn(p, Ad.data_ptr(), Bd.data_ptr(), info.data_ptr(), refine, stream()) == 0
            torch.cuda.synchronize()
            assert (info == 0).all()
        return Ad, Bd

    A0, X0 = run(3)
    for cfg in CONFIGS:
        assert gbla_lib.gbla_ragged_plan_set_config(p, C.byref(Cfg(*cfg))) == 0
        A1, X1 = run(2)
        assert torch.equal(A1, A0) and torch.equal(X1, X0), cfg
    Ak, Bk = Ah.clone(), Bh.clone()
    best, ms = Cfg(), C.c_float()
    assert tune(p, Ak.data_ptr(), Bk.data_ptr(), refine, 2, C.byref(best), C.byref(ms), stream()) == 0
    torch.cuda.synchronize()
    assert torch.equal(Ak, Ah) and torch.equal(Bk, Bh)       # inputs untouched
    assert (best.threads, best.systems_per_block) in CONFIGS and ms.value > 0
    cur = Cfg()
    assert gbla_lib.gbla_ragged_plan_get_config(p, C.byref(cur)) == 0
    assert (cur.threads, cur.systems_per_block) == (best.threads, best.systems_per_block)
    A2, X2 = run()
    assert torch.equal(A2, A0) and torch.equal(X2, X0)
    assert gbla_lib.gbla_ragged_plan_destroy(p) == 0


def test_graph_replays_of_one_launch(gbla_lib, cuda):
    """A call is one kernel; captured in a CUDA graph it replays correctly many
    times in a row (the queue counter is reset by each launch)."""
    import torch
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(count=2000, seed=9, dtype=np.float32)
    st, p = _plan(gbla_lib, a_off, b_off, n, nrhs)
    assert st == 0
    A0, B0 = torch.tensor(A).cuda(), torch.tensor(B).cuda()
    Ad, Bd = A0.clone(), B0.clone()
    info = torch.full((len(n),), -1, dtype=torch.int32, device="cuda")
    assert gbla_lib.gbla_sposv_ragged(p, Ad.data_ptr(), Bd.data_ptr(), info.data_ptr(), 1, stream()) == 0
    torch.cuda.synchronize()
    X_ref = Bd.clone()
    g = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    with torch.cuda.graph(g, stream=cap):
        cs = torch.cuda.current_stream().cuda_stream
        assert gbla_lib.gbla_sposv_ragged(p, Ad.data_ptr(), Bd.data_ptr(), info.data_ptr(), 1, cs) == 0
    for _ in range(5):
        Ad.copy_(A0)
        Bd.copy_(B0)
        info.fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        assert (info == 0).all() and torch.equal(Bd, X_ref)
    assert gbla_lib.gbla_ragged_plan_destroy(p) == 0
