"""Learned Jacobi warm start: the BF16 tensor-core GEMM against a torch FP64
reference of the same op, the network's gradients and frames against the
FP64 oracle (oracle/wsnet.py), the warm SVD's cold fallback, and what the
trained network gains over the cold start at the same tolerance."""
import ctypes as C

import numpy as np
import pytest

from gputils_gb300 import warmstart as W
from gputils_gb300 import workloads
from oracle import oracle as O
from oracle import wsnet as OW
from tests.helpers import stream

pytestmark = pytest.mark.gpu


class Epi(C.Structure):
    _fields_ = [("alpha", C.c_float), ("bias", C.c_void_p), ("relu", C.c_int), ("mask", C.c_void_p),
                ("ld_mask", C.c_int64), ("out_f32", C.c_void_p), ("ld_f32", C.c_int64), ("out_bf16", C.c_void_p),
                ("ld_bf16", C.c_int64), ("out_bf16_t", C.c_void_p), ("ld_bf16_t", C.c_int64)]


def _bf(t):
    import torch
    return t.to(torch.bfloat16)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 136), (1000, 2016, 512), (77, 40, 8),
                                   (512, 512, 4096), (2016, 512, 1000)])
def test_gemm_bf16_vs_torch(gbla_lib, cuda, M, N, K):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = _bf(torch.randn(M, K, device="cuda", generator=g))
    B = _bf(torch.randn(N, K, device="cuda", generator=g))
    bias = torch.randn(N, device="cuda", generator=g)
    ref = A.double() @ B.double().T
    out = torch.full((M, N), float("nan"), device="cuda")
    e = Epi(alpha=1.0, out_f32=out.data_ptr(), ld_f32=N)
    st = gbla_lib.gbla_gemm_bf16_tn(M, N, K, A.data_ptr(), K, B.data_ptr(), K, C.byref(e), stream())
    assert st == 0
    torch.cuda.synchronize()
    scale = ref.abs().max().item()
    assert (out.double() - ref).abs().max().item() < 2e-6 * scale * max(1.0, K / 64) ** 0.5
    # fused epilogue: 0.5 * acc + bias, ReLU, BF16 row-major and transposed
    ob = torch.zeros((M, N), device="cuda", dtype=torch.bfloat16)
    ot = torch.zeros((N, M + 8), device="cuda", dtype=torch.bfloat16)
    e = Epi(alpha=0.5, bias=bias.data_ptr(), relu=1, out_bf16=ob.data_ptr(), ld_bf16=N, out_bf16_t=ot.data_ptr(),
            ld_bf16_t=M + 8)
    assert gbla_lib.gbla_gemm_bf16_tn(M, N, K, A.data_ptr(), K, B.data_ptr(), K, C.byref(e), stream()) == 0
    torch.cuda.synchronize()
    want = torch.clamp(0.5 * ref + bias.double(), min=0.0)
    tolb = 2 ** -7 * want.abs() + 1e-5 * scale
    assert ((ob.double() - want).abs() <= tolb).all()
    assert torch.equal(ot[:, :M], ob.T)
    # ReLU-derivative mask from a stored activation
    mask = _bf(torch.randn(M, N, device="cuda", generator=g))
    out2 = torch.empty((M, N), device="cuda")
    e = Epi(alpha=1.0, mask=mask.data_ptr(), ld_mask=N, out_f32=out2.data_ptr(), ld_f32=N)
    assert gbla_lib.gbla_gemm_bf16_tn(M, N, K, A.data_ptr(), K, B.data_ptr(), K, C.byref(e), stream()) == 0
    torch.cuda.synchronize()
    assert torch.equal(out2 == 0, (mask.float() <= 0) | (out == 0))
    assert torch.equal(out2[mask.float() > 0], out[mask.float() > 0])
    assert gbla_lib.gbla_device_error_flags() == 0


def test_gemm_bf16_rejects_bad_arguments(gbla_lib, cuda):
    import torch
    A = torch.zeros((64, 64), device="cuda", dtype=torch.bfloat16)
    o = torch.zeros((64, 64), device="cuda")
    e = Epi(alpha=1.0, out_f32=o.data_ptr(), ld_f32=64)
    L = gbla_lib
    assert L.gbla_gemm_bf16_tn(64, 64, 60, A.data_ptr(), 60, A.data_ptr(), 64, C.byref(e), stream()) == 1  # ld % 8
    assert L.gbla_gemm_bf16_tn(64, 64, 64, A.data_ptr() + 2, 64, A.data_ptr(), 64, C.byref(e), stream()) == 1
    assert L.gbla_gemm_bf16_tn(64, 64, 64, A.data_ptr(), 64, A.data_ptr(), 64, None, stream()) == 1
    e0 = Epi(alpha=1.0)
    assert L.gbla_gemm_bf16_tn(64, 64, 64, A.data_ptr(), 64, A.data_ptr(), 64, C.byref(e0), stream()) == 1
    assert L.gbla_gemm_bf16_tn(0, 64, 64, None, 64, None, 64, C.byref(e), stream()) == 0


def _family(k, n=64, seed=6, theta_seed=99):
    basis = W.family_basis(n, seed)
    return W.family_batch(basis, k, theta_seed), basis


def _random_params(net, seed, w3_scale=0.02):
    import torch
    off, sizes = OW.layout(net.n, net.hidden)
    g = torch.Generator(device="cuda").manual_seed(seed)
    p = torch.empty(net.param_count, device="cuda")
    for b, (o, s) in enumerate(zip(off[:-1], sizes)):
        fan = net.n * net.n if b < 2 else net.hidden
        scale = (6.0 / fan) ** 0.5 if b in (0, 2) else (w3_scale if b == 4 else 0.05)
        p[o:o + s] = (torch.rand(s, device="cuda", generator=g) * 2 - 1) * scale
    net.set_params(p)
    return p


def test_gradients_match_oracle(gbla_lib, cuda):
    import torch
    n, hidden, k = 64, 512, 24
    A, _ = _family(k)
    _, V, _, _ = W.jacobi(A)
    net = W.WarmStartNet(n, hidden, max_batch=64, seed=3)
    p = _random_params(net, 11)
    Vb, _ = np.linalg.qr(np.random.default_rng(2).standard_normal((n, n)))
    net.set_base(torch.tensor(Vb.T.copy(), dtype=torch.float32))  # column-major
    loss, g, asg = net.gradients(A, V)
    torch.cuda.synchronize()
    p_np, A_np, V_np = p.cpu().numpy(), A.reshape(k, -1).cpu().numpy(), V.reshape(k, -1).cpu().numpy()
    Vb_cm = Vb.T.ravel()
    lo, go, used = OW.gradients(p_np, A_np, V_np, Vb_cm, n, hidden, assign=asg.cpu().numpy())
    assert abs(loss.item() - lo) < 1e-4 * lo
    off, _ = OW.layout(n, hidden)
    g_np = g.cpu().numpy().astype(np.float64)
    for b in range(6):
        gb, ob = g_np[off[b]:off[b + 1]], go[off[b]:off[b + 1]]
        err = np.linalg.norm(gb - ob) / np.linalg.norm(ob)
        assert err < 5e-3, (b, err)
    # the GPU's greedy matching is the oracle's on (almost) every matrix
    _, _, own = OW.gradients(p_np, A_np, V_np, Vb_cm, n, hidden)
    agree = (own == asg.cpu().numpy()).all(axis=1).mean()
    assert agree >= 0.9, agree
    net.close()


def test_frames_orthogonal_and_match_oracle(gbla_lib, cuda):
    import torch
    n, hidden, k = 64, 512, 40
    A, _ = _family(k, theta_seed=5)
    net = W.WarmStartNet(n, hidden, max_batch=16, seed=1)  # predict runs in chunks of 16
    eye = np.eye(n)
    # Cayley frame alone: W3 = 0 makes the outputs exactly b3 (FP32)
    p = _random_params(net, 4, w3_scale=0.0)
    off, _ = OW.layout(n, hidden)
    p[off[5]:off[6]] = 0.5 * torch.randn(off[6] - off[5], device="cuda")
    net.set_params(p)
    Vb, _ = np.linalg.qr(np.random.default_rng(8).standard_normal((n, n)))
    net.set_base(torch.tensor(Vb.T.copy(), dtype=torch.float32))
    V0n = net.predict(A).cpu().numpy().astype(np.float64).transpose(0, 2, 1)  # (row, col)
    assert np.abs(V0n.transpose(0, 2, 1) @ V0n - eye).max() < 2e-5
    b3 = p[off[5]:off[6]].cpu().numpy().astype(np.float64)
    _, V0o = OW.cayley(b3[None], Vb, n)
    assert np.abs(V0n - V0o).max() < 2e-5
    # whole network: BF16 activations may round differently under FP32 and
    # FP64 accumulation, so the frames agree to the BF16 level only
    p = _random_params(net, 4, w3_scale=0.05)
    net.set_base(torch.eye(n))
    V0n = net.predict(A).cpu().numpy().astype(np.float64).transpose(0, 2, 1)
    assert np.abs(V0n.transpose(0, 2, 1) @ V0n - eye).max() < 2e-5
    _, _, _, O_ = OW.forward(p.cpu().numpy(), A.reshape(k, -1).cpu().numpy(), n, hidden)
    _, V0o = OW.cayley(O_, eye, n)
    d = np.abs(V0n - V0o)
    assert d.max() < 5e-3 and d.mean() < 5e-5, (d.max(), d.mean())
    net.close()


def test_warm_svd_fallback_and_exact_start(gbla_lib, cuda):
    import torch
    n, k = 64, 128
    A, _ = _family(k, theta_seed=17)
    S_cold, V, sw_cold, info = W.jacobi(A)
    assert (info == 0).all()
    # converged FP32 frames: done in a few sweeps, no fallback
    S, Vt, sw, info, fb = W.warm_jacobi(A, V, warm_budget=4)
    assert (info == 0).all() and (fb == 0).all() and sw.max().item() <= 4
    assert ((S - S_cold).abs() / S_cold[:, :1]).max().item() < 2e-6
    # random frames with a budget of 1 sweep: the cold restart runs and agrees
    Q, _ = torch.linalg.qr(torch.randn(k, n, n, device="cuda", dtype=torch.float64))
    S, Vt, sw, info, fb = W.warm_jacobi(A, Q.float().contiguous(), warm_budget=1)
    assert (info == 0).all() and fb.sum().item() == k
    assert torch.equal(sw, sw_cold + 1)
    assert ((S - S_cold).abs() / S_cold[:, :1]).max().item() < 2e-6
    o = O.gesvj(A[:16].double().cpu().numpy().transpose(0, 2, 1))
    assert np.abs(S[:16].cpu().numpy() - o["S"]).max() / o["S"][:, 0].max() < 1e-6


def test_trained_network_reduces_sweeps(gbla_lib, cuda):
    """Train on 60k family pairs (a short schedule) and compare warm against
    cold Jacobi at the same tolerance on held-out members of the 64 x 64
    family: fewer sweeps, same singular values (<= 1e-6 vs FP64)."""
    import torch
    net, stats = W.train_family_model(n=64, pairs=60_000, epochs=6, batch=512, seed=0)
    assert stats["loss"][-1] < stats["loss"][0]
    A = torch.tensor(workloads.svd_family(2048, 64, seed=6)[0].transpose(0, 2, 1).copy(), device="cuda")
    S_c, _, sw_c, info_c = W.jacobi(A)
    V0 = net.predict(A)
    S_w, _, sw_w, info_w, fb = W.warm_jacobi(A, V0, warm_budget=net.warm_budget)
    assert (info_c == 0).all() and (info_w == 0).all()
    cold, warm = sw_c.float().mean().item(), sw_w.float().mean().item()
    assert warm * 1.3 <= cold, (warm, cold)
    assert fb.float().mean().item() < 0.02
    idx = np.arange(0, 2048, 64)
    o = O.gesvj(A[idx].double().cpu().numpy().transpose(0, 2, 1))
    for S in (S_c, S_w):
        err = np.abs(S[idx].cpu().numpy() - o["S"]).max(axis=1) / np.linalg.norm(o["S"], axis=1)
        assert err.max() < 1e-6
    net.close()
