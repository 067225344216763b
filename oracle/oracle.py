"""ctypes front end of the FP64 CPU oracle (``oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``; never by the product.

Batches are numpy arrays of shape ``(k, m, n)`` (k matrices of m x n).  They
are widened to float64 and laid out column-major, matrix after matrix (the
reference's DTensor (m, n, k) layout, include/tensor.cuh:264-281), before the
C routines run.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_int64)


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile next to this file."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "all"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_max_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_gemm_batched.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_double, _dp, C.c_int]
        L.orc_potrf_batched.argtypes = [C.c_int, _dp, _ip, C.c_int]
        L.orc_potrs_batched.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.orc_posv_ragged.argtypes = [C.c_int, _lp, _lp, _ip, _ip, _dp, _dp, _ip]
        L.orc_geqrf_batched.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.orc_ormqr_batched.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp, C.c_int]
        L.orc_trsm_upper_batched.argtypes = [C.c_int, C.c_int, _dp, C.c_int, C.c_int64, _dp, C.c_int, C.c_int64, C.c_int]
        L.orc_gels_batched.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.orc_gesvj_batched.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_int, _ip, _ip, C.c_int]
        _lib = L
    return _lib


def set_threads(t: int) -> None:
    lib().orc_set_threads(int(t))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def to_cm(x) -> np.ndarray:
    """(k, m, n) array -> contiguous float64 buffer, column-major per matrix."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 2:
        x = x[None]
    # always a fresh buffer: the C routines work in place
    return np.array(x.transpose(0, 2, 1), dtype=np.float64, order="C", copy=True)


def from_cm(buf, k: int, m: int, n: int) -> np.ndarray:
    """Inverse of :func:`to_cm`: column-major buffer -> (k, m, n) array."""
    return np.asarray(buf).reshape(k, n, m).transpose(0, 2, 1)


def gemm(A, B, C=None, alpha: float = 1.0, beta: float = 0.0) -> np.ndarray:
    """C_i <- alpha A_i B_i + beta C_i for (k,m,kk) A and (k,kk,n) B."""
    A = np.asarray(A); B = np.asarray(B)
    k, m, kk = A.shape
    n = B.shape[2]
    a, b = to_cm(A), to_cm(B)
    c = to_cm(C) if C is not None else np.zeros((k, n, m))
    lib().orc_gemm_batched(m, n, kk, alpha, _p(a), _p(b), beta if C is not None else 0.0, _p(c), k)
    return from_cm(c, k, m, n)


def potrf(A):
    """Lower Cholesky of each (n,n) matrix.  Returns (A with L in the lower
    triangle and the original strict upper triangle, info)."""
    A = np.asarray(A)
    k, n, _ = A.shape
    a = to_cm(A)
    info = np.zeros(k, dtype=np.int32)
    lib().orc_potrf_batched(n, _p(a), _p(info, _ip), k)
    return from_cm(a, k, n, n), info


def potrs(L, B):
    L = np.asarray(L); B = np.asarray(B)
    k, n, _ = L.shape
    nrhs = B.shape[2]
    l, b = to_cm(L), to_cm(B)
    lib().orc_potrs_batched(n, nrhs, _p(l), _p(b), k)
    return from_cm(b, k, n, nrhs)


def posv(A, B):
    """Factor + solve; returns (L-in-place A, X, info)."""
    Af, info = potrf(A)
    X = potrs(Af, B)
    return Af, X, info


def posv_ragged(A_arena, B_arena, a_off, b_off, n, nrhs):
    """Ragged factor+solve on flat float64 arenas (column-major per system)."""
    A = np.array(A_arena, dtype=np.float64, copy=True)
    B = np.array(B_arena, dtype=np.float64, copy=True)
    a_off = np.ascontiguousarray(a_off, dtype=np.int64)
    b_off = np.ascontiguousarray(b_off, dtype=np.int64)
    n = np.ascontiguousarray(n, dtype=np.int32)
    nrhs = np.ascontiguousarray(nrhs, dtype=np.int32)
    info = np.zeros(len(n), dtype=np.int32)
    lib().orc_posv_ragged(len(n), _p(a_off, _lp), _p(b_off, _lp), _p(n, _ip), _p(nrhs, _ip),
                          _p(A), _p(B), _p(info, _ip))
    return A, B, info


def geqrf(A):
    A = np.asarray(A)
    k, m, n = A.shape
    a = to_cm(A)
    tau = np.zeros((k, min(m, n)))
    lib().orc_geqrf_batched(m, n, _p(a), _p(tau), k)
    return from_cm(a, k, m, n), tau


def ormqr(QR, tau, Cm, trans: bool = True):
    QR = np.asarray(QR); Cm = np.asarray(Cm)
    k, m, n = QR.shape
    nrhs = Cm.shape[2]
    kk = tau.shape[1]
    qr, c, t = to_cm(QR), to_cm(Cm), np.ascontiguousarray(tau, dtype=np.float64)
    lib().orc_ormqr_batched(1 if trans else 0, m, nrhs, kk, _p(qr), n, _p(t), _p(c), k)
    return from_cm(c, k, m, nrhs)


def gels(A, B):
    """QR least squares.  Returns (QR factors, B with X in rows [0, n))."""
    A = np.asarray(A); B = np.asarray(B)
    k, m, n = A.shape
    nrhs = B.shape[2]
    a, b = to_cm(A), to_cm(B)
    lib().orc_gels_batched(m, n, nrhs, _p(a), _p(b), k)
    return from_cm(a, k, m, n), from_cm(b, k, m, nrhs)


def gesvj(A, tol: float = 1e-15, max_sweeps: int = 60, compute_u: bool = False):
    """One-sided Jacobi SVD.  Returns dict with S (k, n) sorted descending,
    V (k, n, n), U (k, m, m) or None, sweeps, info."""
    A = np.asarray(A)
    k, m, n = A.shape
    a = to_cm(A)
    S = np.zeros((k, n)); V = np.zeros((k, n, n))
    U = np.zeros((k, m, m)) if compute_u else None
    sweeps = np.zeros(k, dtype=np.int32); info = np.zeros(k, dtype=np.int32)
    up = _p(U) if compute_u else C.cast(None, _dp)
    lib().orc_gesvj_batched(m, n, _p(a), _p(S), _p(V), up, tol, max_sweeps, _p(sweeps, _ip), _p(info, _ip), k)
    return {
        "S": S,
        "V": from_cm(V, k, n, n),
        "U": from_cm(U, k, m, m) if compute_u else None,
        "sweeps": sweeps,
        "info": info,
    }
