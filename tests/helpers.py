"""Shared helpers for the GPU parity tests: column-major device batches,
error metrics and the golden values read from tests/golden/."""
from __future__ import annotations

import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def goldens():
    with open(os.path.join(GOLDEN_DIR, "reference_goldens.json")) as f:
        return json.load(f)["values"]


def to_dev(x, dtype):
    """(k, m, n) numpy batch -> contiguous CUDA tensor in DTensor layout
    (column-major matrices back to back)."""
    import torch

    x = np.asarray(x)
    if x.ndim == 2:
        x = x[None]
    cm = np.ascontiguousarray(x.transpose(0, 2, 1)).astype(dtype)
    return torch.from_numpy(cm).cuda()


def from_dev(t, k, m, n):
    return t.detach().cpu().numpy().reshape(k, n, m).transpose(0, 2, 1)


def colmajor(values, m, n, k=1):
    """Flat column-major values (DTensor upload order) -> (k, m, n)."""
    return np.asarray(values, dtype=np.float64).reshape(k, n, m).transpose(0, 2, 1)


def rowmajor(values, m, n, k=1):
    """Flat row-major values (StorageMode::rowMajor, per matrix) -> (k, m, n)."""
    return np.asarray(values, dtype=np.float64).reshape(k, m, n)


def stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def ptr(t):
    return t.data_ptr()


def rel_err(x, ref, axis=(1, 2)):
    """max over the batch of ||x - ref|| / ||ref|| (Frobenius per matrix)."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    num = np.sqrt(((x - ref) ** 2).sum(axis=axis))
    den = np.sqrt((ref ** 2).sum(axis=axis))
    den = np.where(den == 0, 1.0, den)
    return float((num / den).max())


def spd_batch(rng, k, n, shift=1.0, scale=None):
    G = rng.standard_normal((k, n, n))
    s = float(n) if scale is None else scale
    return G.transpose(0, 2, 1) @ G / s + shift * np.eye(n)
