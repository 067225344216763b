"""FP64 restatement of the learned Jacobi warm start (network, Cayley frame,
greedy column matching, frame-matching loss and its gradient).

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` to check the GPU kernels
(libgbla's gbla_wsnet_* entry points); never by the product.

The reference has no such component (its Svd always starts Jacobi from the
identity), so there is no reference output to pin against: this module is the
definition the GPU path is checked against, and its own gradient is checked
by finite differences in ``tests/test_oracle.py``.

Layouts follow the C ABI: an n x n matrix is a flat column-major vector
(element (i, j) at j n + i); network activations are row-major
[batch][features].  BF16 rounding (round to nearest even) is applied at the
points where the GPU path stores BF16: the packed input, the weights, the
hidden activations, dL/dO and the hidden-layer gradients.  Products are
accumulated in FP64 here and in FP32 on the GPU.
"""
from __future__ import annotations

import numpy as np


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even); returns float64."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def layout(n: int, hidden: int):
    """Offsets of W1, b1, W2, b2, W3, b3 in the flat parameter vector."""
    P, nn = n * (n - 1) // 2, n * n
    sizes = [hidden * nn, hidden, hidden * hidden, hidden, P * hidden, P]
    off = np.concatenate([[0], np.cumsum(sizes)])
    return off, sizes


def unpack(params, n: int, hidden: int):
    off, _ = layout(n, hidden)
    P, nn = n * (n - 1) // 2, n * n
    p = np.asarray(params, dtype=np.float64)
    W1 = p[off[0]:off[1]].reshape(hidden, nn)
    b1 = p[off[1]:off[2]]
    W2 = p[off[2]:off[3]].reshape(hidden, hidden)
    b2 = p[off[3]:off[4]]
    W3 = p[off[4]:off[5]].reshape(P, hidden)
    b3 = p[off[5]:off[6]]
    return W1, b1, W2, b2, W3, b3


def upper_pairs(n: int):
    """(i, j), i < j, in output order: row-major upper triangle."""
    return np.triu_indices(n, 1)


def skew(o, n: int) -> np.ndarray:
    """S (k, n, n) from output rows o (k, P): S[i, j] = o_p, S[j, i] = -o_p."""
    o = np.atleast_2d(o)
    iu, ju = upper_pairs(n)
    S = np.zeros((o.shape[0], n, n))
    S[:, iu, ju] = o
    S[:, ju, iu] = -o
    return S


def cayley(o, Vb, n: int):
    """X = (I - S)^{-1} and V0 = Vb (2 X - I), both (k, n, n) (row, col indexing)."""
    S = skew(o, n)
    eye = np.eye(n)
    X = np.linalg.solve(eye[None] - S, np.broadcast_to(eye, S.shape))
    V0 = np.einsum("ij,kjl->kil", Vb, 2.0 * X - eye[None])
    return X, V0


def greedy_match(C) -> tuple[np.ndarray, np.ndarray]:
    """Greedy matching of predicted columns (rows of C) to true columns: the
    largest |C[i, j]| among unmatched rows and columns first, ties to the
    smallest row-major position.  Returns perm (n,) and signs (n,)."""
    n = C.shape[0]
    a = np.abs(C).copy()
    perm = np.zeros(n, dtype=np.int64)
    sgn = np.zeros(n)
    for _ in range(n):
        f = int(np.argmax(a))
        i, j = divmod(f, n)
        perm[i] = j
        sgn[i] = -1.0 if C[i, j] < 0 else 1.0
        a[i, :] = -1.0
        a[:, j] = -1.0
    return perm, sgn


def frame_loss(o, V, Vb, n: int, assign=None):
    """Loss per matrix ||V0 - V Pi D||_F^2 and dL_b/do (k, P).

    o: (k, P) network outputs; V: (k, n, n) true frames (row, col indexing);
    Vb: (n, n).  assign (optional, (k, n) ints sign * (1 + index)) fixes the
    matching instead of recomputing it.  Returns (loss (k,), dO (k, P),
    assign (k, n))."""
    o = np.atleast_2d(np.asarray(o, dtype=np.float64))
    k = o.shape[0]
    X, V0 = cayley(o, Vb, n)
    iu, ju = upper_pairs(n)
    loss = np.zeros(k)
    dO = np.zeros_like(o)
    out_assign = np.zeros((k, n), dtype=np.int64)
    for b in range(k):
        if assign is None:
            perm, sgn = greedy_match(V0[b].T @ V[b])
        else:
            a = np.asarray(assign[b])
            perm, sgn = np.abs(a) - 1, np.sign(a).astype(np.float64)
        out_assign[b] = (sgn * (perm + 1)).astype(np.int64)
        T = V[b][:, perm] * sgn[None, :]
        R = V0[b] - T
        loss[b] = np.sum(R * R)
        dCay = Vb.T @ (2.0 * R)
        dS = 2.0 * X[b].T @ dCay @ X[b].T
        dO[b] = dS[iu, ju] - dS[ju, iu]
    return loss, dO, out_assign


def forward(params, A_cm, n: int, hidden: int):
    """A_cm: (k, n*n) column-major vecs.  Returns X, H1, H2 (BF16-rounded) and O."""
    W1, b1, W2, b2, W3, b3 = unpack(params, n, hidden)
    X = bf16(A_cm)
    H1 = bf16(np.maximum(X @ bf16(W1).T + b1, 0.0))
    H2 = bf16(np.maximum(H1 @ bf16(W2).T + b2, 0.0))
    O = (H2 @ bf16(W3).T + b3).astype(np.float32).astype(np.float64)
    return X, H1, H2, O


def gradients(params, A_cm, V_cm, Vb_cm, n: int, hidden: int, assign=None):
    """Mean loss over the batch and its gradient w.r.t. the flat parameters,
    with the GPU path's BF16 rounding points.  V_cm, Vb_cm column-major."""
    k = A_cm.shape[0]
    W1, b1, W2, b2, W3, b3 = unpack(params, n, hidden)
    X, H1, H2, O = forward(params, A_cm, n, hidden)
    V = np.asarray(V_cm, dtype=np.float64).reshape(k, n, n).transpose(0, 2, 1)
    Vb = np.asarray(Vb_cm, dtype=np.float64).reshape(n, n).T
    loss, dO, used = frame_loss(O, V, Vb, n, assign)
    dO = bf16(dO / k)
    g3 = dO.T @ H2
    gb3 = dO.sum(0)
    dH2 = bf16((dO @ bf16(W3)) * (H2 > 0))
    g2 = dH2.T @ H1
    gb2 = dH2.sum(0)
    dH1 = bf16((dH2 @ bf16(W2)) * (H1 > 0))
    g1 = dH1.T @ X
    gb1 = dH1.sum(0)
    grad = np.concatenate([g1.ravel(), gb1, g2.ravel(), gb2, g3.ravel(), gb3])
    return loss.mean(), grad, used
