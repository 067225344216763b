"""The warm-start oracle (oracle/wsnet.py) on the CPU: BF16 rounding against
torch's conversion, the Cayley frame, the greedy matching, and the analytic
gradient of the frame-matching loss against central finite differences."""
import numpy as np

from oracle import wsnet as OW


def test_bf16_rounding_matches_torch():
    import torch
    x = np.random.default_rng(0).standard_normal(10000).astype(np.float32) * 10.0
    x[:4] = [1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -(1.0 + 2 ** -8), 0.0]  # ties to even
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(OW.bf16(x), ref)


def test_cayley_frame_is_orthogonal():
    n = 12
    rng = np.random.default_rng(1)
    o = rng.standard_normal((3, n * (n - 1) // 2))
    Vb, _ = np.linalg.qr(rng.standard_normal((n, n)))
    X, V0 = OW.cayley(o, Vb, n)
    assert np.abs(V0.transpose(0, 2, 1) @ V0 - np.eye(n)).max() < 1e-12
    S = OW.skew(o, n)
    assert np.allclose(S, -S.transpose(0, 2, 1))
    _, V00 = OW.cayley(np.zeros((1, n * (n - 1) // 2)), Vb, n)
    assert np.allclose(V00[0], Vb)


def test_greedy_match_finds_permutation_and_signs():
    n = 10
    rng = np.random.default_rng(2)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    perm = rng.permutation(n)
    sgn = rng.choice([-1.0, 1.0], n)
    V = Q[:, perm] * sgn          # V[:, i] = sgn_i Q[:, perm_i]
    C = Q.T @ V                   # rows: predicted columns (Q), cols: true columns (V)
    p, s = OW.greedy_match(C)
    # predicted column i of Q is true column j with Q[:, i] = s V[:, j]
    assert np.allclose(V[:, p] * s[None, :], Q)


def test_loss_gradient_matches_finite_differences():
    n = 6
    P = n * (n - 1) // 2
    rng = np.random.default_rng(3)
    o = 0.3 * rng.standard_normal((2, P))
    V = np.stack([np.linalg.qr(rng.standard_normal((n, n)))[0] for _ in range(2)])
    Vb, _ = np.linalg.qr(rng.standard_normal((n, n)))
    loss, dO, asg = OW.frame_loss(o, V, Vb, n)
    h = 1e-6
    num = np.zeros_like(o)
    for b in range(2):
        for p in range(P):
            op, om = o.copy(), o.copy()
            op[b, p] += h
            om[b, p] -= h
            lp, _, _ = OW.frame_loss(op, V, Vb, n, assign=asg)
            lm, _, _ = OW.frame_loss(om, V, Vb, n, assign=asg)
            num[b, p] = (lp[b] - lm[b]) / (2 * h)
    assert np.abs(num - dO).max() < 1e-6 * max(1.0, np.abs(dO).max())


def test_network_gradient_matches_finite_differences_without_rounding(monkeypatch):
    """The backward pass of oracle.gradients is the derivative of its forward
    pass (BF16 rounding switched off so the loss is smooth)."""
    monkeypatch.setattr(OW, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    n, hidden, k = 4, 8, 3
    off, sizes = OW.layout(n, hidden)
    rng = np.random.default_rng(4)
    p = 0.3 * rng.standard_normal(off[-1])
    A = rng.standard_normal((k, n * n))
    V = np.stack([np.linalg.qr(rng.standard_normal((n, n)))[0].T.ravel() for _ in range(k)])
    Vb = np.linalg.qr(rng.standard_normal((n, n)))[0].T.ravel()
    # forward() rounds O through float32; compare in a float64 copy of it
    monkeypatch.setattr(OW, "forward", _forward64)
    loss, grad, asg = OW.gradients(p, A, V, Vb, n, hidden)
    h = 1e-6
    idx = rng.choice(off[-1], 40, replace=False)
    for e in idx:
        pp, pm = p.copy(), p.copy()
        pp[e] += h
        pm[e] -= h
        lp, _, _ = OW.gradients(pp, A, V, Vb, n, hidden, assign=asg)
        lm, _, _ = OW.gradients(pm, A, V, Vb, n, hidden, assign=asg)
        assert abs((lp - lm) / (2 * h) - grad[e]) < 1e-5 * max(1.0, abs(grad[e]))


def _forward64(params, A_cm, n, hidden):
    W1, b1, W2, b2, W3, b3 = OW.unpack(params, n, hidden)
    X = np.asarray(A_cm, dtype=np.float64)
    H1 = np.maximum(X @ W1.T + b1, 0.0)
    H2 = np.maximum(H1 @ W2.T + b2, 0.0)
    return X, H1, H2, H2 @ W3.T + b3
