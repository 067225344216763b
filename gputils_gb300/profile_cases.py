"""Small, self-checking cases of the hot kernels, sized for ncu captures.

    python -m gputils_gb300.profile_cases ragged [--count 4000] [--dtype f32]
    python -m gputils_gb300.profile_cases svd64 [--count 4096] [--warm]
    python -m gputils_gb300.profile_cases gels [--count 8192] [--two-kernel]

Each case runs one call of the library on seeded inputs of the benchmark's
distributions (a few hundred MB on the device at most), checks the status
outputs and prints a one-line summary; with --repeat N it runs the call N times
(the ragged case also times each size bucket of its plan separately).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np

from . import _lib, warmstart, workloads


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def ragged(count: int, dtype: str, repeat: int, nmin: int = 4, rhs_max: int = 8, refine: int = -1) -> dict:
    import torch
    L = _lib.lib()
    dt = np.float32 if dtype == "f32" else np.float64
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(count=count, nmin=nmin, rhs_max=rhs_max, dtype=dt)
    p = C.c_void_p()
    _lib.check(L.gbla_ragged_plan_create(np.ascontiguousarray(a_off).ctypes.data,
                                         np.ascontiguousarray(b_off).ctypes.data,
                                         np.ascontiguousarray(n, np.int32).ctypes.data,
                                         np.ascontiguousarray(nrhs, np.int32).ctypes.data, len(n), C.byref(p)),
               "plan")
    fn = L.gbla_sposv_ragged if dt == np.float32 else L.gbla_dposv_ragged
    if refine < 0:
        refine = 1 if dt == np.float32 else 2
    A0, B0 = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    info = torch.empty(len(n), dtype=torch.int32, device="cuda")
    times = []
    for _ in range(repeat):
        Ad, Bd = A0.clone(), B0.clone()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(fn(p, Ad.data_ptr(), Bd.data_ptr(), info.data_ptr(), refine, _stream()), "posv_ragged")
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    assert int(info.max()) == 0
    _lib.check(L.gbla_ragged_plan_destroy(p), "plan destroy")
    return {"case": "ragged", "systems": count, "dtype": dtype, "nmin": nmin, "rhs_max": rhs_max, "refine": refine,
            "ms": min(times), "large_systems": int((n > 32).sum())}


def svd64(count: int, warm: bool, repeat: int) -> dict:
    import torch
    A = warmstart.family_batch(warmstart.family_basis(64, 6), count, 77)
    times = []
    for _ in range(repeat):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if warm:
            net = warmstart.WarmStartNet(64, 512, max_batch=count, seed=0)
            e0.record()
            V0 = net.predict(A)
            S, Vt, sw, info, fb = warmstart.warm_jacobi(A, V0, 9)
            e1.record()
        else:
            e0.record()
            S, V, sw, info = warmstart.jacobi(A)
            e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    assert int(info.max()) == 0
    return {"case": "svd64", "matrices": count, "warm": warm, "ms": min(times),
            "sweeps": float(sw.float().mean())}


def gels(count: int, repeat: int, two_kernel: bool = False) -> dict:
    import torch
    L = _lib.lib()
    A, B = workloads.d2b_least_squares(k=count)
    k, m, nn = A.shape
    r = B.shape[2]
    Ah = torch.from_numpy(np.ascontiguousarray(A.transpose(0, 2, 1))).cuda()
    Bh = torch.from_numpy(np.ascontiguousarray(B.transpose(0, 2, 1))).cuda()
    info = torch.empty(k, dtype=torch.int32, device="cuda")
    wsb = L.gbla_sgels_batched_workspace_bytes(m, nn, k)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    times = []
    for _ in range(repeat):
        Ad, Bd = Ah.clone(), Bh.clone()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        if not two_kernel:
            _lib.check(L.gbla_sgels_batched(m, nn, r, Ad.data_ptr(), m * nn, Bd.data_ptr(), m * r, info.data_ptr(),
                                            1, k, _stream()), "sgels")
        else:
            _lib.check(L.gbla_sgels_batched_ws(m, nn, r, Ad.data_ptr(), m * nn, Bd.data_ptr(), m * r,
                                               info.data_ptr(), 1, ws.data_ptr(), wsb, k, _stream()), "sgels_ws")
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    assert int(info.max()) == 0
    return {"case": "gels", "systems": k, "two_kernel": two_kernel, "ms": min(times)}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("case", choices=["ragged", "svd64", "gels"])
    ap.add_argument("--count", type=int, default=0)
    ap.add_argument("--dtype", choices=["f32", "f64"], default="f32")
    ap.add_argument("--warm", action="store_true")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--nmin", type=int, default=4, help="ragged: smallest n")
    ap.add_argument("--rhs-max", type=int, default=8, help="ragged: largest nrhs")
    ap.add_argument("--refine", type=int, default=-1, help="ragged: refinement steps (default 1 f32, 2 f64)")
    ap.add_argument("--two-kernel", action="store_true",
                    help="gels: the workspace entry point (warp factorisation + block solve)")
    a = ap.parse_args(argv)
    if a.case == "ragged":
        out = ragged(a.count or 4000, a.dtype, a.repeat, a.nmin, a.rhs_max, a.refine)
    elif a.case == "svd64":
        out = svd64(a.count or 4096, a.warm, a.repeat)
    else:
        out = gels(a.count or 8192, a.repeat, a.two_kernel)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
