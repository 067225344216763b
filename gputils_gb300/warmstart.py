"""Learned warm start for the batched one-sided Jacobi SVD.

Host side of the gbla_wsnet_* entry points (``gputils_gb300/csrc/wsnet.cu``):
a network maps each n x n matrix to a skew matrix S whose Cayley transform
about a base frame Vb gives an orthogonal warm start V0 = Vb (I - S)^{-1}
(I + S) for Jacobi; the warm run falls back to a cold start
(gbla_sgesvj_warm_batched) when it has not converged within the cold sweep
count.  Training data are (A, V) pairs produced by the plain cold Jacobi SVD
(gbla_sgesvj_batched) on the GPU; training runs entirely in the library's
own BF16 tensor-core forward / backward kernels and an FP32 Adam.

Matrices cross this module as torch CUDA tensors of shape (k, n, n) holding
column-major matrices (element (i, j) of matrix b at [b, j, i]), i.e. the
flat layout of the C ABI.  PyTorch supplies device memory and streams only.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib

_lib_call = _lib.call


def _torch():
    import torch
    return torch


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def family_basis(n: int, seed: int, params: int = 4) -> np.ndarray:
    """The parametric family's fixed matrices A0, A1..A_params ~ N(0, 1)/sqrt(n),
    drawn exactly as ``workloads.svd_family`` draws them (row, col indexing)."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal((params + 1, n, n)) / np.sqrt(n)


def family_batch(basis: np.ndarray, count: int, theta_seed: int, device="cuda"):
    """count members A(theta) = A0 + sum_j theta_j A_j, theta ~ U[-1, 1]^p from
    its own seed, generated on the device in FP64 and rounded to FP32.
    Returns a (count, n, n) column-major FP32 tensor."""
    torch = _torch()
    p = basis.shape[0] - 1
    g = torch.Generator(device=device).manual_seed(theta_seed)
    theta = torch.rand((count, p), generator=g, device=device, dtype=torch.float64) * 2.0 - 1.0
    B = torch.tensor(basis.transpose(0, 2, 1).copy(), device=device, dtype=torch.float64)  # column-major
    A = B[0].unsqueeze(0) + torch.einsum("kp,pij->kij", theta, B[1:])
    return A.to(torch.float32).contiguous()


def jacobi(A, tol: float = 1e-6, max_sweeps: int = 60, V0=None):
    """Cold (or plain warm, no fallback) batched Jacobi SVD of column-major
    (k, n, n) A.  Returns S (k, n), V (k, n, n) column-major, sweeps, info."""
    torch = _torch()
    k, n, _ = A.shape
    S = torch.empty((k, n), device=A.device, dtype=torch.float32)
    Vt = torch.empty((k, n, n), device=A.device, dtype=torch.float32)
    sweeps = torch.empty(k, device=A.device, dtype=torch.int32)
    info = torch.empty(k, device=A.device, dtype=torch.int32)
    _lib_call("gbla_sgesvj_batched", n, n, _ptr(A), n * n, _ptr(S), n, _ptr(Vt), n * n, None, n * n,
              _ptr(V0), n * n, tol, max_sweeps, _ptr(info), _ptr(sweeps), k, _stream())
    # Vt column-major holds V^T, whose column-major layout is V row-major
    V = Vt.transpose(1, 2).contiguous()
    return S, V, sweeps, info


def warm_jacobi(A, V0, warm_budget: int, tol: float = 1e-6, max_sweeps: int = 60):
    """Jacobi from V0 with cold fallback after warm_budget sweeps.
    Returns S, Vt (column-major V^T), sweeps, info, fallback."""
    torch = _torch()
    k, n, _ = A.shape
    S = torch.empty((k, n), device=A.device, dtype=torch.float32)
    Vt = torch.empty((k, n, n), device=A.device, dtype=torch.float32)
    sweeps = torch.empty(k, device=A.device, dtype=torch.int32)
    info = torch.empty(k, device=A.device, dtype=torch.int32)
    fb = torch.empty(k, device=A.device, dtype=torch.int32)
    _lib_call("gbla_sgesvj_warm_batched", n, n, _ptr(A), n * n, _ptr(S), n, _ptr(Vt), n * n, None, n * n,
              _ptr(V0), n * n, warm_budget, tol, max_sweeps, _ptr(info), _ptr(sweeps), _ptr(fb), k, _stream())
    return S, Vt, sweeps, info, fb


class WarmStartNet:
    """Owner of a gbla_wsnet (network weights, Adam state, base frame)."""

    def __init__(self, n: int = 64, hidden: int = 512, max_batch: int = 4096, seed: int = 0):
        self.n, self.hidden, self.max_batch = n, hidden, max_batch
        self.P = n * (n - 1) // 2
        h = C.c_void_p()
        _lib_call("gbla_wsnet_create", n, hidden, max_batch, seed, C.byref(h))
        self._h = h
        self.warm_budget = None

    def close(self):
        if self._h:
            _lib.lib().gbla_wsnet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def param_count(self) -> int:
        return int(_lib.lib().gbla_wsnet_param_count(self._h))

    def params(self):
        torch = _torch()
        p = torch.empty(self.param_count, device="cuda", dtype=torch.float32)
        _lib_call("gbla_wsnet_get_params", self._h, _ptr(p), _stream())
        return p

    def set_params(self, p):
        torch = _torch()
        p = p.to(device="cuda", dtype=torch.float32).contiguous()
        _lib_call("gbla_wsnet_set_params", self._h, _ptr(p), _stream())

    def base(self):
        torch = _torch()
        b = torch.empty((self.n, self.n), device="cuda", dtype=torch.float32)
        _lib_call("gbla_wsnet_get_base", self._h, _ptr(b), _stream())
        return b

    def set_base(self, Vb):
        torch = _torch()
        Vb = Vb.to(device="cuda", dtype=torch.float32).contiguous()
        _lib_call("gbla_wsnet_set_base", self._h, _ptr(Vb), _stream())

    def gradients(self, A, V, idx=None):
        """(mean loss, flat gradient, assignment) for one batch without updating."""
        torch = _torch()
        b = A.shape[0] if idx is None else idx.shape[0]
        g = torch.empty(self.param_count, device="cuda", dtype=torch.float32)
        loss = torch.empty(1, device="cuda", dtype=torch.float32)
        asg = torch.empty((b, self.n), device="cuda", dtype=torch.int32)
        _lib_call("gbla_wsnet_gradients", self._h, _ptr(A), self.n * self.n, _ptr(V), self.n * self.n, _ptr(idx),
                  b, _ptr(g), _ptr(loss), _ptr(asg), _stream())
        return loss, g, asg

    def train_step(self, A, V, idx, lr: float, loss_out=None):
        _lib_call("gbla_wsnet_train_step", self._h, _ptr(A), self.n * self.n, _ptr(V), self.n * self.n, _ptr(idx),
                  idx.shape[0], lr, _ptr(loss_out), _stream())

    def fit(self, A, V, epochs: int = 20, batch: int = 512, lr: float = 1e-3, lr_min: float = 1e-5,
            seed: int = 0, log=None):
        """Adam with a cosine learning-rate decay over shuffled mini-batches of
        the (A, V) pairs (both (k, n, n) column-major on the device).
        Returns the per-epoch mean training loss."""
        torch = _torch()
        k = A.shape[0]
        batch = min(batch, self.max_batch)
        steps_per_epoch = k // batch
        total = max(1, epochs * steps_per_epoch)
        losses = torch.zeros(steps_per_epoch, device="cuda", dtype=torch.float32)
        g = torch.Generator(device="cuda").manual_seed(seed)
        hist = []
        step = 0
        for ep in range(epochs):
            perm = torch.randperm(k, generator=g, device="cuda").to(torch.int32)
            for s in range(steps_per_epoch):
                rate = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * step / total))
                self.train_step(A, V, perm[s * batch:(s + 1) * batch], rate, losses[s:s + 1])
                step += 1
            hist.append(float(losses.mean()))
            if log:
                log(ep, hist[-1])
        return hist

    def predict(self, A, out=None):
        """Warm-start frames V0 (k, n, n) column-major for column-major A."""
        torch = _torch()
        k = A.shape[0]
        if out is None:
            out = torch.empty((k, self.n, self.n), device="cuda", dtype=torch.float32)
        _lib_call("gbla_wsnet_predict", self._h, _ptr(A), self.n * self.n, _ptr(out), self.n * self.n, k,
                  _stream())
        return out

    def save(self, path: str):
        np.savez(path, n=self.n, hidden=self.hidden, params=self.params().cpu().numpy(),
                 base=self.base().cpu().numpy(), warm_budget=-1 if self.warm_budget is None else self.warm_budget)

    def load(self, path: str):
        torch = _torch()
        z = np.load(path)
        if int(z["n"]) != self.n or int(z["hidden"]) != self.hidden:
            raise ValueError("checkpoint shape does not match this network")
        self.set_params(torch.tensor(z["params"]))
        self.set_base(torch.tensor(z["base"]))
        wb = int(z["warm_budget"])
        self.warm_budget = None if wb < 0 else wb


def train_family_model(n: int = 64, family_seed: int = 6, pairs: int = 200_000, epochs: int = 20,
                       hidden: int = 512, batch: int = 256, lr: float = 1e-3, tol: float = 1e-6,
                       theta_seed: int = 1234, seed: int = 0, infer_batch: int = 32768, log=None):
    """Generate `pairs` (A, V) pairs of the parametric family with the cold
    Jacobi SVD, set the base frame to the family's A0 frame, train, and set
    the warm budget to the median cold sweep count.  Returns (net, stats)."""
    torch = _torch()
    basis = family_basis(n, family_seed)
    A = family_batch(basis, pairs, theta_seed)
    chunks, sweeps = [], []
    for c0 in range(0, pairs, 32768):
        _, V, sw, info = jacobi(A[c0:c0 + 32768], tol=tol)
        chunks.append(V)
        sweeps.append(sw)
    V = torch.cat(chunks)
    sweeps = torch.cat(sweeps)
    A0 = torch.tensor(basis[0].T.copy(), device="cuda", dtype=torch.float32).reshape(1, n, n).contiguous()
    _, Vb, _, _ = jacobi(A0, tol=tol)
    # buffers sized for inference on a whole benchmark batch in one pass
    net = WarmStartNet(n, hidden, max_batch=max(batch, infer_batch), seed=seed)
    net.set_base(Vb[0])
    hist = net.fit(A, V, epochs=epochs, batch=batch, lr=lr, seed=seed, log=log)
    net.warm_budget = int(sweeps.float().median().item())
    stats = {"pairs": pairs, "epochs": epochs, "loss": hist, "cold_sweeps_mean": float(sweeps.float().mean()),
             "warm_budget": net.warm_budget}
    del A, V
    return net, stats
