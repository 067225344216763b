#!/usr/bin/env python
"""Benchmark of the batched-matrix hot path on GB300.

Default workload (one "step"): the precision configuration of the headline
metric --
  * DTensor::addAB on 16384 pairs of 64x64 fp32 matrices (entries U[-1,1]),
    tcgen05 tensor cores with a three-way BF16 split (6 products, FP32
    accumulation), and
  * leastSquaresBatched on 8192 tall 128x32 fp32 matrices (U diag(s) V^T,
    Haar U, V, s log-spaced 1..1e3) with 4 right-hand sides, FP32 Householder
    QR plus one step of augmented-system refinement with double-FP32
    residuals.
value = (16384 + 8192) matrices per step / device time per step, inputs
resident in HBM (each step has its own copy of the least-squares inputs,
which the solver overwrites; every step's inputs exceed the 129 MB L2).

Other workloads (--workload d1 ...) time the other configurations.

Arms: --impl ours (default) runs this library; --impl reference times the
reference's path on the host cores.  GPUtils has no CPU implementation (every
numeric call is cuBLAS/cuSOLVER), so the reference arm runs the FP64 CPU
restatement of those library algorithms (oracle/), all host threads, on a
bounded sample of the same workload.  The reference's own cuBLAS/cuSOLVER
call sequence on the same GPU is reported inside the ours line as
"reference_library".
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "traffic.json")
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
# FP32 FFMA rate of this GPU, measured by the FMA probe (baseline/peak_probe.cu) at
# start-up while the SM clock is sampled (fp32_peak()); the denominator of the
# CUDA-core rooflines
FP32_PEAK = {"tflops": None, "sm_mhz": None, "source": None}

# algorithmic work per unit (each input read once, each output written once)
GEMM_BYTES_PER_PAIR = 3 * 64 * 64 * 4                       # A, B in; C out
GEMM_FLOPS_PER_PAIR = 2 * 64 ** 3
LS_M, LS_N, LS_RHS = 128, 32, 4
# per-system algorithmic bytes: A and B in, x out (the factors written back over A
# and the rows of B below n are not counted)
LS_BYTES_PER_MATRIX = 4 * (LS_M * LS_N + LS_M * LS_RHS + LS_N * LS_RHS)
LS_FLOPS_PER_MATRIX = (2 * LS_M * LS_N ** 2 - 2 * LS_N ** 3 // 3
                       + LS_RHS * (4 * LS_M * LS_N - 2 * LS_N ** 2 + LS_N ** 2))


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["d2", "d1", "d3", "d4", "d5", "large"], default="d2",
                    help="large: one --large-n matrix through CholeskyFactoriser<float> (part of the d2 line's workloads)")
    ap.add_argument("--dtype", choices=["f32", "f64"], default="f32", help="data type of the ragged workload d3")
    ap.add_argument("--ref-sample", type=int, default=0,
                    help="matrices the reference SVD host loop runs on (d4/d5; scaled to the batch)")
    ap.add_argument("--refine", type=int, default=1, help="least-squares refinement steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-library", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="budget of the CPU baseline sample")
    ap.add_argument("--peaks", action="store_true", help="print the measured FFMA / DFMA rates and exit")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="fraction of the workload's batch to run (small cases for ncu captures)")
    ap.add_argument("--no-workloads", action="store_true",
                    help="d2: skip the other configurations' results in the default line")
    ap.add_argument("--no-autotune", action="store_true", help="d3: keep the plan's default launch configuration")
    ap.add_argument("--ragged-config", default=None,
                    help="d3: threads,systems_per_block of the plan instead of autotuning (e.g. 768,8)")
    ap.add_argument("--ws-pairs", type=int, default=200_000, help="d5: (A, V) training pairs of the warm-start net")
    ap.add_argument("--ws-epochs", type=int, default=20, help="d5: training epochs of the warm-start net")
    ap.add_argument("--large-n", type=int, default=4096, help="order of the one-matrix Cholesky in the workloads")
    return ap.parse_args(argv)


# ------------------------------------------------------------- distributed
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def dist_init(world: int, backend: str):
    import torch.distributed as dist

    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist


def aggregate(elapsed_s: float, units_this_rank: float, world: int, dist=None, device=None):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time (max over ranks)."""
    if world > 1:
        import torch

        t = torch.tensor([elapsed_s, units_this_rank], dtype=torch.float64, device=device)
        tmax = t[:1].clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
        return float(tmax.item()), float(t[1].item())
    return elapsed_s, units_this_rank


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"gbla_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9 and parts[1].isdigit():
                rows.append(parts)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        maxmhz = max(int(r[2]) for r in rows)
        loaded = [int(r[1]) for r in rows if float(r[3] or 0) > 0] or [int(r[1]) for r in rows]
        busy = [int(r[1]) for r in rows if int(r[1]) > 0.3 * maxmhz] or loaded
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": maxmhz, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3] or 0) for r in rows)}


# ------------------------------------------------------------- helpers
def peaks():
    if os.path.exists(PEAKS_FILE):
        d = json.load(open(PEAKS_FILE))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops", FALLBACK_PEAKS["bf16_tflops"]),
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": FALLBACK_PEAKS["hbm_gbs"], "bf16_tflops": FALLBACK_PEAKS["bf16_tflops"],
            "bf16_tflops_sustained": None, "source": "fallback"}


def traffic_for(kernel: str):
    if os.path.exists(TRAFFIC_FILE):
        return json.load(open(TRAFFIC_FILE)).get(kernel)
    return None


def to_dev(x, dev):
    import torch

    x = np.asarray(x)
    return torch.from_numpy(np.ascontiguousarray(x.transpose(0, 2, 1))).to(dev)


def from_dev(t, k, m, n):
    return t.detach().cpu().numpy().reshape(k, n, m).transpose(0, 2, 1)


def rel_err(x, ref):
    x = np.asarray(x, np.float64); ref = np.asarray(ref, np.float64)
    num = np.sqrt(((x - ref) ** 2).sum(axis=(1, 2)))
    den = np.sqrt((ref ** 2).sum(axis=(1, 2)))
    return float((num / np.where(den == 0, 1, den)).max())


def rel_err_t(x, ref, k):
    """max over k matrices of ||x_i - ref_i|| / ||ref_i|| (FP64, on the device);
    x and ref hold k equally sized matrices back to back."""
    xd = x.reshape(k, -1).double()
    rd = ref.reshape(k, -1).double()
    num = (xd - rd).norm(dim=1)
    den = rd.norm(dim=1)
    den = den.where(den > 0, den.new_ones(()))
    return float((num / den).max())


# ------------------------------------------------------------ CPU baseline
def _repeat_timed(fn, seconds: float):
    """Run fn() until `seconds` have passed (at least once); returns (calls, total seconds)."""
    calls, t0 = 0, time.perf_counter()
    while True:
        fn()
        calls += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            return calls, el


def cpu_baseline_d2(seconds: float):
    """FP64 oracle (OpenMP over matrices, all host threads) on a fixed sample
    of the d2 workload, repeated for about `seconds`; matrices/s."""
    from gputils_gb300 import workloads
    from oracle import oracle as O

    O.set_threads(os.cpu_count() or 1)
    ng, nl = 2048, 1024
    A, B = workloads.d2a_gemm(k=ng, seed=12)
    LA, LB = workloads.d2b_least_squares(k=nl, seed=13)
    cg, tg = _repeat_timed(lambda: O.gemm(A, B), seconds * 0.5)
    cl, tl = _repeat_timed(lambda: O.gels(LA, LB), seconds * 0.5)
    g_rate, l_rate = cg * ng / tg, cl * nl / tl
    # one step = 16384 GEMM pairs + 8192 least-squares systems
    t_step = 16384 / g_rate + 8192 / l_rate
    return {"value": (16384 + 8192) / t_step, "unit": "matrices/s", "cores": O.max_threads(), "kind": "port",
            "sample": f"{cg} x {ng} GEMM pairs + {cl} x {nl} least-squares systems in {tg + tl:.1f} s "
                      f"(FP64, OpenMP over matrices), combined in the 16384 : 8192 ratio of a step",
            "gemm_pairs_per_s": g_rate, "ls_systems_per_s": l_rate}


def cpu_baseline_d1(seconds: float):
    from gputils_gb300 import workloads
    from oracle import oracle as O

    O.set_threads(os.cpu_count() or 1)
    M, b = workloads.d1_cholesky(k=4096, seed=11)
    calls, t = _repeat_timed(lambda: O.posv(M, b), seconds)
    return {"value": 4096 * calls / t, "unit": "matrices/s", "cores": O.max_threads(), "kind": "port",
            "sample": f"{calls} x 4096 16x16 Cholesky factor+solve in {t:.1f} s (FP64, OpenMP over matrices)"}


def _ragged_subset(count, seed, dtype):
    from gputils_gb300 import workloads
    return workloads.d3_ragged(count=count, seed=seed, dtype=dtype)


def cpu_baseline_d3(seconds: float, dtype=np.float32):
    """FP64 potrf + potrs per system (OpenMP over systems) on a 2000-system
    sample of the ragged distribution; systems/s."""
    from oracle import oracle as O

    O.set_threads(os.cpu_count() or 1)
    n, nrhs, a_off, b_off, A, B = _ragged_subset(2000, 31, np.float64)
    calls, t = _repeat_timed(lambda: O.posv_ragged(A, B, a_off, b_off, n, nrhs), seconds)
    return {"value": 2000 * calls / t, "unit": "matrices/s", "cores": O.max_threads(), "kind": "port",
            "sample": f"{calls} x 2000 ragged SPD systems (n 4..128, nrhs 1..8) in {t:.1f} s "
                      f"(FP64 potrf + potrs per system, OpenMP over systems)"}


def cpu_baseline_svd(seconds: float, n: int):
    """FP64 one-sided Jacobi SVD per matrix (OpenMP over matrices) on a
    sample of the parametric family; matrices/s."""
    from gputils_gb300 import workloads
    from oracle import oracle as O

    O.set_threads(os.cpu_count() or 1)
    k = 256 if n <= 32 else 64
    A = workloads.svd_family(k, n, seed=41)[0]
    calls, t = _repeat_timed(lambda: O.gesvj(A, tol=1e-6), seconds)
    return {"value": k * calls / t, "unit": "matrices/s", "cores": O.max_threads(), "kind": "port",
            "sample": f"{calls} x {k} {n}x{n} one-sided Jacobi SVDs (FP64, tol 1e-6) in {t:.1f} s "
                      f"(OpenMP over matrices)"}


CPU_BASELINES = {
    "d1": lambda sec, args: cpu_baseline_d1(sec),
    "d2": lambda sec, args: cpu_baseline_d2(sec),
    "d3": lambda sec, args: cpu_baseline_d3(sec),
    "d4": lambda sec, args: cpu_baseline_svd(sec, 32),
    "d5": lambda sec, args: cpu_baseline_svd(sec, 64),
}


# ------------------------------------------------------------ reference arm
def run_reference_arm(args):
    rank, world, _ = dist_env()
    if world > 1:
        dist = dist_init(world, "gloo")
        if rank != 0:
            dist.barrier()
            return
    if args.workload not in CPU_BASELINES:
        print(json.dumps({"impl": "reference", "unavailable": f"no CPU sample for workload {args.workload}; its "
                          "reference is the cuSOLVER call on the GPU, reported in our line"}), flush=True)
        return
    # each step is a bounded sample: about cpu_seconds, and the whole run a few minutes at most
    budget = max(0.5, min(args.cpu_seconds, 120.0 / max(1, args.steps + args.warmup)))
    fn = CPU_BASELINES[args.workload]
    for _ in range(args.warmup):
        fn(min(budget, 2.0), args)
    vals = [fn(budget, args) for _ in range(args.steps)]
    v = statistics.median([x["value"] for x in vals])
    first = vals[0]
    line = {
        "impl": "reference", "metric": metric_name(args.workload), "value": v, "unit": "matrices/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(args.workload, args),
        "cpu_baseline": {"value": v, "unit": "matrices/s", "cores": first["cores"], "kind": first["kind"],
                         "sample": first["sample"]},
        "e2e": {"value": v, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()


def metric_name(workload):
    return "matrices/s on 1 GB300 (Chol/QR/SVD batched) vs ref cuSOLVER build at equal FP64 err"


def _k(count, args):
    """Batch count of a workload at the --scale fraction (at least 1)."""
    scale = getattr(args, "scale", 1.0) if args is not None else 1.0
    return max(1, int(round(count * scale)))


def workload_config(workload, args=None):
    """The configuration dict of a workload; both arms print the same one."""
    refine = getattr(args, "refine", 1) if args is not None else 1
    scale = getattr(args, "scale", 1.0) if args is not None else 1.0
    extra = {} if scale == 1.0 else {"scale": scale}
    if workload == "d2":
        return dict({"workload": "precision: addAB 16384 x 64x64x64 fp32 (BF16x6 tcgen05) + leastSquaresBatched "
                                 "8192 x 128x32 fp32, 4 RHS, kappa 1e3 (FP32 QR + double-FP32 refinement)",
                     "gemm_pairs": _k(16384, args), "ls_systems": _k(8192, args), "refine_steps": refine,
                     "parallelism": "replicas",
                     "l2": "inputs larger than L2 every step (per-step copies of the least-squares inputs)"}, **extra)
    if workload == "d1":
        return dict({"workload": "Cholesky factor+solve 4096 x 16x16 fp32, 1 RHS (CholeskyBatchFactoriser API: "
                                 "potrf + potrs)",
                     "matrices": _k(4096, args), "parallelism": "replicas",
                     "l2": "L2 flushed between timed steps (the 4.5 MB working set fits in L2)"}, **extra)
    if workload == "d3":
        dt = getattr(args, "dtype", "f32") if args is not None else "f32"
        return dict({"workload": f"ragged Cholesky factor+solve, 20000 SPD systems, n log-uniform in [4,128], "
                                 f"nrhs 1..8, {dt}, one call (plan + CUDA graph), FP32 factor + refinement",
                     "systems": _k(20000, args), "dtype": dt, "refine_steps": 1 if dt == "f32" else 2,
                     "parallelism": "replicas",
                     "l2": "inputs larger than L2 every step (per-step copies of the arenas)"}, **extra)
    if workload == "d5":
        pairs = getattr(args, "ws_pairs", 200_000) if args is not None else 200_000
        return dict({"workload": "learned warm start: one-sided Jacobi SVD (S and V^T) of 32768 64x64 fp32 matrices "
                                 "of the parametric family A0 + sum theta_j A_j, tol 1e-6; each step = network "
                                 "(4096->512->512->2016, BF16 tcgen05) + Cayley frame + warm Jacobi with cold fallback",
                     "matrices": _k(32768, args), "n": 64, "train_pairs": pairs, "parallelism": "replicas",
                     "l2": "inputs (537 MB) larger than L2"}, **extra)
    return dict({"workload": "one-sided Jacobi SVD (Svd::factorise, S and V^T) of 8192 32x32 fp32 matrices of the "
                             "parametric family A0 + sum theta_j A_j, tol 1e-6, cold start",
                 "matrices": _k(8192, args), "n": 32, "parallelism": "replicas",
                 "l2": "per-step copies of the input (the SVD destroys it)"}, **extra)


# ------------------------------------------------------------- ours: d2
class RefLib:
    def __init__(self, stream):
        from gputils_gb300 import build

        path = build.BASELINE_LIB
        if not os.path.exists(path):
            build.build_baseline()
        self.L = C.CDLL(path)
        vp, ip = C.c_void_p, C.c_int
        self.L.refp_init.argtypes = [vp]
        self.L.refp_sgemm_batched.argtypes = [ip, ip, ip, C.c_float, vp, vp, C.c_float, vp, ip]
        self.L.refp_sgels_batched.argtypes = [ip, ip, vp, vp, ip, vp]
        self.L.refp_spotrf_batched.argtypes = [ip, vp, vp, ip]
        self.L.refp_spotrs_batched.argtypes = [ip, vp, vp, vp, ip]
        self.L.refp_dpotrf_batched.argtypes = [ip, vp, vp, ip]
        self.L.refp_dpotrs_batched.argtypes = [ip, vp, vp, vp, ip]
        self.L.refp_sgesvd_lwork.argtypes = [ip, ip]
        self.L.refp_sgesvd_loop.argtypes = [ip, ip, vp, vp, vp, vp, vp, ip, vp, ip, ip]
        self.L.refp_spotrf_bufsize.argtypes = [ip, vp]
        self.L.refp_spotrf.argtypes = [ip, vp, vp, ip, vp]
        self.L.refp_spotrs.argtypes = [ip, vp, vp, vp]
        assert self.L.refp_init(stream) == 0


def ptr_array(t, count, stride_elems, dev):
    import torch

    base = t.data_ptr()
    return (torch.arange(count, dtype=torch.int64, device=dev) * (stride_elems * t.element_size()) + base)


def run_ours_d2(args, dev, st, L, rank, world, dist):
    import torch
    from gputils_gb300 import workloads, _lib
    from oracle import oracle as O

    A, B = workloads.d2a_gemm(k=_k(16384, args))
    LA, LB = workloads.d2b_least_squares(k=_k(8192, args))
    kg, kl = A.shape[0], LA.shape[0]
    Ag, Bg = to_dev(A, dev), to_dev(B, dev)
    Cg = torch.empty_like(Ag)
    LA0, LB0 = to_dev(LA, dev), to_dev(LB, dev)
    nsteps = args.warmup + args.steps
    LAs = [LA0.clone() for _ in range(nsteps)]
    LBs = [LB0.clone() for _ in range(nsteps)]
    info = torch.empty(kl, dtype=torch.int32, device=dev)
    m, n, r = LS_M, LS_N, LS_RHS

    def step(i, evs=None):
        if evs: evs[0].record()
        _lib.check(L.gbla_sgemm_batched(64, 64, 64, 1.0, Ag.data_ptr(), 4096, Bg.data_ptr(), 4096, 0.0,
                                        Cg.data_ptr(), 4096, kg, 0, st), "sgemm")
        if evs: evs[1].record()
        _lib.check(L.gbla_sgels_batched(m, n, r, LAs[i].data_ptr(), m * n, LBs[i].data_ptr(), m * r,
                                        info.data_ptr(), args.refine, kl, st), "sgels")
        if evs: evs[2].record()

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        e0.record()
        for i in range(args.steps):
            step(args.warmup + i, evs[i])
        e1.record()
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    elapsed = e0.elapsed_time(e1) / 1e3
    t_gemm = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps / 1e3
    t_ls = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps / 1e3
    units = (kg + kl) * args.steps
    elapsed_max, units_all = aggregate(elapsed, units, world, dist, dev)
    assert gbla_device_flags_ok(L)

    # accuracy vs the FP64 oracle on a sample
    idx_g = np.arange(0, kg, 128)
    err_gemm = rel_err(from_dev(Cg, kg, 64, 64)[idx_g], O.gemm(A[idx_g], B[idx_g]))
    idx_l = np.arange(0, kl, 64)
    X = from_dev(LBs[args.warmup], kl, m, r)[idx_l, :n]
    _, Xo = O.gels(LA[idx_l], LB[idx_l])
    err_ls = rel_err(X, Xo[:, :n])
    info_ok = bool((info.cpu().numpy() == 0).all())

    # ---- end to end through the C ABI with host buffers (pinned), copies timed
    hA, hB = torch.from_numpy(np.ascontiguousarray(A.transpose(0, 2, 1))).pin_memory(), \
        torch.from_numpy(np.ascontiguousarray(B.transpose(0, 2, 1))).pin_memory()
    hLA, hLB = torch.from_numpy(np.ascontiguousarray(LA.transpose(0, 2, 1))).pin_memory(), \
        torch.from_numpy(np.ascontiguousarray(LB.transpose(0, 2, 1))).pin_memory()
    hC = torch.empty_like(hA).pin_memory()
    hX = torch.empty_like(hLB).pin_memory()
    # host-buffer calls: chunks rotate over three worker streams, so copies in,
    # kernels and copies out of consecutive chunks overlap
    pipe = C.c_void_p()
    _lib.check(L.gbla_pipeline_create(3, C.byref(pipe)), "pipeline")

    def e2e_step():
        _lib.check(L.gbla_sgemm_batched_host(pipe, 64, 64, 64, 1.0, hA.data_ptr(), 4096, hB.data_ptr(), 4096, 0.0,
                                             hC.data_ptr(), 4096, kg, 0, 0, st), "sgemm_host")
        _lib.check(L.gbla_sgels_batched_host(pipe, m, n, r, hLA.data_ptr(), m * n, None, hLB.data_ptr(), m * r,
                                             hX.data_ptr(), None, args.refine, kl, 0, st), "sgels_host")

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    # the host results agree with the device-resident path
    e2e_ok = bool(torch.equal(hX, LBs[0].cpu())) and bool(torch.equal(hC, Cg.cpu()))
    esteps = max(3, min(args.steps, 10))
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(esteps):
        e2e_step()
    f1.record()
    torch.cuda.synchronize()
    e2e_t = f0.elapsed_time(f1) / 1e3 / esteps
    e2e_max, _ = aggregate(e2e_t, 0.0, world, dist, dev)
    h2d = (hA.numel() + hB.numel() + hLA.numel() + hLB.numel()) * 4
    d2h = (hC.numel() + hX.numel()) * 4
    _lib.check(L.gbla_pipeline_destroy(pipe), "pipeline destroy")

    # ---- reference library path (cuBLAS / cuSOLVER calls of tensor.cuh) on the same GPU
    reflib = None
    if not args.no_reference_library:
        try:
            reflib = reference_library_d2(dev, st, Ag, Bg, Cg, LA0, LB0, A, B, LA, LB, LBs[args.warmup])
        except Exception as exc:  # reported, never fatal for our own numbers
            reflib = {"unavailable": f"{type(exc).__name__}: {exc}"}

    pk = peaks()
    rl = {}
    for name, t, bytes_, flops_, units_k in (("gemm", t_gemm, GEMM_BYTES_PER_PAIR, GEMM_FLOPS_PER_PAIR, kg),
                                             ("gels", t_ls, LS_BYTES_PER_MATRIX, LS_FLOPS_PER_MATRIX, kl)):
        ach = bytes_ * units_k / t / 1e9
        tr = traffic_for(name + "_d2")
        rl[name] = {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                    "frac": ach / pk["hbm_gbs"], "traffic": tr, "ms": t * 1e3,
                    "algorithmic_bytes_per_launch": bytes_ * units_k, "peak_source": pk["source"] + " hbm_gbs",
                    # the same launch against the FP32 FFMA rate (algorithmic flops, LAPACK counts)
                    "fp32_tflops": flops_ * units_k / t / 1e12,
                    "fp32_frac": flops_ * units_k / t / 1e12 / FP32_PEAK["tflops"]}
    dom = "gemm" if t_gemm >= t_ls else "gels"
    value = units_all / elapsed_max
    line = {
        "metric": metric_name("d2"), "value": value, "unit": "matrices/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_max / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy generators, configuration distributions)",
        "config": workload_config("d2", args),
        "roofline": dict(rl[dom], kernel=dom),
        "roofline_all": rl,
        "max_rel_err_vs_fp64": {"gemm": err_gemm, "least_squares_x": err_ls},
        "info_all_zero": info_ok,
        "e2e": {"value": (kg + kl) * world / e2e_max, "unit": "matrices/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_max * 1e3,
                "path": "C ABI host-buffer calls (gbla_sgemm_batched_host + gbla_sgels_batched_host, chunks "
                        "over 3 streams) on pinned host buffers: H2D of A, B, A_ls, B_ls and D2H of C, X inside "
                        "the timed region", "matches_device_path": e2e_ok},
        "gpu_launches": 2 * args.steps,  # device-resident step: GEMM + fused least squares
        "clocks": clk.summary(),
        "reference_library": reflib,
    }
    return line


def gbla_device_flags_ok(L):
    return L.gbla_device_error_flags() == 0


def reference_library_d2(dev, st, Ag, Bg, Cg, LA0, LB0, A, B, LA, LB, X_ours):
    """The reference's calls on the same inputs: cublasSgemmBatched with
    pointer arrays (addAB) and cublasSgelsBatched (nrhs = 1, so the 4 RHS run
    as one call on a 4x-replicated batch; replication not timed)."""
    import torch
    from oracle import oracle as O

    R = RefLib(st)
    kg, kl = Ag.shape[0], LA0.shape[0]
    m, n, r = LS_M, LS_N, LS_RHS
    Cr = torch.empty_like(Cg)
    pa, pb, pc = ptr_array(Ag, kg, 4096, dev), ptr_array(Bg, kg, 4096, dev), ptr_array(Cr, kg, 4096, dev)
    # replicated least-squares batch: system (i, c) = (A_i, column c of B_i)
    LAr = LA0.repeat_interleave(r, dim=0).contiguous()                      # (4k, n, m)
    LBr = LB0.reshape(kl, r, m).reshape(kl * r, 1, m).contiguous()          # (4k, 1, m)
    LAr0, LBr0 = LAr.clone(), LBr.clone()
    pla, plb = ptr_array(LAr, kl * r, m * n, dev), ptr_array(LBr, kl * r, m, dev)
    hinfo = C.c_int(0)

    def gemm():
        assert R.L.refp_sgemm_batched(64, 64, 64, 1.0, pa.data_ptr(), pb.data_ptr(), 0.0, pc.data_ptr(), kg) == 0

    def gels():
        assert R.L.refp_sgels_batched(m, n, pla.data_ptr(), plb.data_ptr(), kl * r, C.byref(hinfo)) == 0

    gemm(); LAr.copy_(LAr0); LBr.copy_(LBr0); gels()
    torch.cuda.synchronize()
    reps = 5
    tg = tl = 0.0
    for _ in range(reps):
        LAr.copy_(LAr0); LBr.copy_(LBr0)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record(); gemm(); e[1].record(); gels(); e[2].record()
        torch.cuda.synchronize()
        tg += e[0].elapsed_time(e[1]) / 1e3
        tl += e[1].elapsed_time(e[2]) / 1e3
    tg /= reps; tl /= reps
    idx = np.arange(0, kg, 128)
    err_g = rel_err(from_dev(Cr, kg, 64, 64)[idx], O.gemm(A[idx], B[idx]))
    X = LBr.reshape(kl, r, m).cpu().numpy().transpose(0, 2, 1)[:, :n]
    idl = np.arange(0, kl, 64)
    _, Xo = O.gels(LA[idl], LB[idl])
    err_l = rel_err(X[idl], Xo[:, :n])
    # ours against the reference library's own output, every matrix
    Xr = LBr.reshape(kl, r, m)[:, :, :n]
    Xu = X_ours.reshape(kl, r, m)[:, :, :n]
    vs_ref = {"gemm": rel_err_t(Cg, Cr, kg), "least_squares_x": rel_err_t(Xu, Xr, kl)}
    return {"value": (kg + kl) / (tg + tl), "unit": "matrices/s", "gemm_ms": tg * 1e3, "gels_ms": tl * 1e3,
            "max_rel_err_vs_fp64": {"gemm": err_g, "least_squares_x": err_l},
            "ours_max_rel_err_vs_reference_output": vs_ref,
            "calls": "cublasSgemmBatched (pointer arrays) + cublasSgelsBatched on the 4x-replicated batch "
                     "(one call; nrhs = 1 in the reference API)"}


# ------------------------------------------------------------- ours: d3
def _ragged_bytes(n, nrhs, elem):
    n = n.astype(np.int64)
    return int((elem * (n * n + n * (n + 1) // 2 + 2 * n * nrhs)).sum())


class RaggedCfg(C.Structure):
    _fields_ = [("threads", C.c_int), ("systems_per_block", C.c_int)]

    def as_dict(self):
        return {"threads": self.threads, "systems_per_block": self.systems_per_block}


def run_ours_d3(args, dev, st, L, rank, world, dist):
    """One gbla_{s,d}posv_ragged call per step on 20000 mixed systems,
    captured once per step buffer in a CUDA graph and replayed."""
    import torch
    from gputils_gb300 import workloads, _lib
    from oracle import oracle as O

    dt = np.float32 if args.dtype == "f32" else np.float64
    tdt = torch.float32 if dt == np.float32 else torch.float64
    n, nrhs, a_off, b_off, A, B = workloads.d3_ragged(count=_k(20000, args), dtype=dt)
    count = len(n)
    plan = C.c_void_p()
    _lib.check(L.gbla_ragged_plan_create(np.ascontiguousarray(a_off).ctypes.data,
                                         np.ascontiguousarray(b_off).ctypes.data,
                                         np.ascontiguousarray(n, np.int32).ctypes.data,
                                         np.ascontiguousarray(nrhs, np.int32).ctypes.data, count, C.byref(plan)),
               "plan")
    refine = 1 if dt == np.float32 else 2
    fn = L.gbla_sposv_ragged if dt == np.float32 else L.gbla_dposv_ragged
    A0 = torch.from_numpy(A).to(dev)
    B0 = torch.from_numpy(B).to(dev)
    # launch configuration: the plan's autotuner on this batch (set-up, untimed)
    cfg = RaggedCfg()
    _lib.check(L.gbla_ragged_plan_get_config(plan, C.byref(cfg)), "get config")
    tuning = {"default": cfg.as_dict()}
    if args.ragged_config:
        t, g = (int(v) for v in args.ragged_config.split(","))
        cfg = RaggedCfg(t, g)
        _lib.check(L.gbla_ragged_plan_set_config(plan, C.byref(cfg)), "set config")
        tuning["set"] = cfg.as_dict()
    elif not args.no_autotune:
        best, best_ms = RaggedCfg(), C.c_float()
        tune = L.gbla_sragged_autotune if dt == np.float32 else L.gbla_dragged_autotune
        _lib.check(tune(plan, A0.data_ptr(), B0.data_ptr(), refine, 3, C.byref(best), C.byref(best_ms), st),
                   "autotune")
        tuning.update({"chosen": best.as_dict(), "chosen_ms": best_ms.value, "candidates": 13})
        cfg = best
    nsteps = args.warmup + args.steps
    As = [A0.clone() for _ in range(nsteps)]
    Bs = [B0.clone() for _ in range(nsteps)]
    info = torch.empty(count, dtype=torch.int32, device=dev)
    # one CUDA graph per step buffer (each replay is the whole ragged solve)
    graphs = []
    cap = torch.cuda.Stream()
    for i in range(nsteps):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=cap):
            cs = torch.cuda.current_stream().cuda_stream
            _lib.check(fn(plan, As[i].data_ptr(), Bs[i].data_ptr(), info.data_ptr(), refine, cs), "posv_ragged")
        graphs.append(g)
    torch.cuda.synchronize()
    # graph capture recorded the work but did not run it: restore pristine inputs
    for i in range(nsteps):
        As[i].copy_(A0); Bs[i].copy_(B0)
    torch.cuda.synchronize()
    for i in range(args.warmup):
        graphs[i].replay()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        e0.record()
        for i in range(args.steps):
            graphs[args.warmup + i].replay()
        e1.record()
        torch.cuda.synchronize()
    elapsed = e0.elapsed_time(e1) / 1e3
    elapsed_max, units_all = aggregate(elapsed, count * args.steps, world, dist, dev)
    assert (info.cpu().numpy() == 0).all()
    # accuracy vs FP64 on a sample of systems
    X = Bs[args.warmup].cpu().numpy()
    idx = np.arange(0, count, 41)
    a_sz, b_sz = n.astype(np.int64) ** 2, n.astype(np.int64) * nrhs
    As_ = np.concatenate([A[a_off[i]:a_off[i] + a_sz[i]] for i in idx])
    Bs_ = np.concatenate([B[b_off[i]:b_off[i] + b_sz[i]] for i in idx])
    a2 = np.concatenate([[0], np.cumsum(a_sz[idx])[:-1]]); b2 = np.concatenate([[0], np.cumsum(b_sz[idx])[:-1]])
    _, Xo, _ = O.posv_ragged(As_, Bs_, a2, b2, n[idx], nrhs[idx])
    err = 0.0
    for j, i in enumerate(idx):
        x = X[b_off[i]:b_off[i] + b_sz[i]].astype(np.float64)
        xo = Xo[b2[j]:b2[j] + b_sz[i]]
        err = max(err, float(np.linalg.norm(x - xo) / np.linalg.norm(xo)))

    # e2e: pinned host arenas, H2D of A and B, the solve, D2H of X, per step
    hA, hB = torch.from_numpy(A).pin_memory(), torch.from_numpy(B).pin_memory()
    hX = torch.empty_like(hB).pin_memory()
    dA, dB = torch.empty_like(A0), torch.empty_like(B0)

    def e2e_step():
        dA.copy_(hA, non_blocking=True); dB.copy_(hB, non_blocking=True)
        _lib.check(fn(plan, dA.data_ptr(), dB.data_ptr(), info.data_ptr(), refine, st), "posv_ragged")
        hX.copy_(dB, non_blocking=True)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    esteps = max(3, min(args.steps, 10))
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(esteps):
        e2e_step()
    f1.record()
    torch.cuda.synchronize()
    e2e_t, _ = aggregate(f0.elapsed_time(f1) / 1e3 / esteps, 0.0, world, dist, dev)

    reflib = None
    if not args.no_reference_library:
        try:
            reflib = reference_library_d3(dev, st, n, nrhs, a_off, b_off, A0, B0, dt, Bs[args.warmup])
        except Exception as exc:
            reflib = {"unavailable": f"{type(exc).__name__}: {exc}"}
    pk = peaks()
    t = elapsed_max / args.steps
    bytes_ = _ragged_bytes(n, nrhs, np.dtype(dt).itemsize)
    ach = bytes_ / t / 1e9
    ntasks, smem = C.c_int(), C.c_size_t()
    _lib.check(L.gbla_ragged_plan_tasks(plan, C.byref(ntasks), C.byref(smem)), "plan tasks")
    tuning.update({"tasks": ntasks.value, "smem_bytes_per_block": smem.value})
    _lib.check(L.gbla_ragged_plan_destroy(plan), "plan destroy")
    launches = 1  # one persistent kernel per call
    return {
        "metric": metric_name("d3"), "value": units_all / elapsed_max, "unit": "matrices/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded)",
        "config": workload_config("d3", args), "launch_config": tuning,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": traffic_for("ragged_d3_" + args.dtype),
                     "kernel": "k_ragged_persistent (the one kernel of a call)", "algorithmic_bytes_per_launch": bytes_},
        "max_rel_err_vs_fp64": {"x": err},
        "e2e": {"value": count * world / e2e_t, "unit": "matrices/s",
                "h2d_bytes_per_step": int(hA.numel() + hB.numel()) * hA.element_size(),
                "d2h_bytes_per_step": int(hX.numel()) * hX.element_size(), "ms_per_step": e2e_t * 1e3},
        "gpu_launches": launches * args.steps, "clocks": clk.summary(), "reference_library": reflib,
    }


def reference_library_d3(dev, st, n, nrhs, a_off, b_off, A0, B0, dt, X_ours):
    """The reference's way to solve a ragged batch: for each distinct n one
    potrfBatched over that size group (CholeskyBatchFactoriser::factorise),
    then one potrsBatched per right-hand-side column (solve takes nrhs = 1),
    over the systems that have that column.  Pointer arrays address the
    matrices in place (no gathers)."""
    import torch
    from oracle import oracle as O

    R = RefLib(st)
    elem = np.dtype(dt).itemsize
    calls = []
    for nn in np.unique(n):
        ids = np.nonzero(n == nn)[0]
        pa = torch.tensor(A0.data_ptr() + a_off[ids] * elem, dtype=torch.int64, device=dev)
        info = torch.zeros(len(ids), dtype=torch.int32, device=dev)
        calls.append(("f", int(nn), pa, None, info, len(ids)))
        for c in range(int(nrhs[ids].max())):
            sel = ids[nrhs[ids] > c]
            pl = torch.tensor(A0.data_ptr() + a_off[sel] * elem, dtype=torch.int64, device=dev)
            pb = torch.tensor(B0.data_ptr() + (b_off[sel] + c * nn) * elem, dtype=torch.int64, device=dev)
            calls.append(("s", int(nn), pl, pb, info, len(sel)))
    potrf = R.L.refp_spotrf_batched if dt == np.float32 else R.L.refp_dpotrf_batched
    potrs = R.L.refp_spotrs_batched if dt == np.float32 else R.L.refp_dpotrs_batched
    Ac, Bc = A0.clone(), B0.clone()

    def run():
        for kind, nn, p1, p2, info, k in calls:
            if kind == "f":
                assert potrf(nn, p1.data_ptr(), info.data_ptr(), k) == 0
            else:
                assert potrs(nn, p1.data_ptr(), p2.data_ptr(), info.data_ptr(), k) == 0

    run()
    torch.cuda.synchronize()
    reps, tot = 3, 0.0
    for _ in range(reps):
        A0.copy_(Ac); B0.copy_(Bc)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        e[0].record(); run(); e[1].record()
        torch.cuda.synchronize()
        tot += e[0].elapsed_time(e[1]) / 1e3
    t = tot / reps
    X = B0.cpu().numpy()
    Xu = X_ours.cpu().numpy()
    A0.copy_(Ac); B0.copy_(Bc)
    idx = np.arange(0, len(n), 41)
    err = 0.0
    Ah, Bh = Ac.cpu().numpy(), Bc.cpu().numpy()
    for i in idx:
        k, r = int(n[i]), int(nrhs[i])
        M = Ah[a_off[i]:a_off[i] + k * k].reshape(k, k).T.astype(np.float64)
        b = Bh[b_off[i]:b_off[i] + k * r].reshape(r, k).T.astype(np.float64)
        xo = np.linalg.solve(M, b)
        x = X[b_off[i]:b_off[i] + k * r].reshape(r, k).T
        err = max(err, float(np.linalg.norm(x - xo) / np.linalg.norm(xo)))
    # ours against the reference library's output, every system
    b_sz = n.astype(np.int64) * nrhs
    ends = b_off + b_sz
    vs_ref = 0.0
    for i in range(len(n)):
        xr = X[b_off[i]:ends[i]].astype(np.float64)
        xu = Xu[b_off[i]:ends[i]].astype(np.float64)
        d = np.linalg.norm(xr)
        vs_ref = max(vs_ref, float(np.linalg.norm(xu - xr) / (d if d > 0 else 1.0)))
    return {"value": len(n) / t, "unit": "matrices/s", "ms": t * 1e3, "library_calls": len(calls),
            "max_rel_err_vs_fp64": {"x": err}, "ours_max_rel_err_vs_reference_output": {"x": vs_ref},
            "calls": "per size n: cusolverDn<t>potrfBatched, then per RHS column cusolverDn<t>potrsBatched "
                     "(nrhs = 1) over the systems having that column"}


# ------------------------------------------------------------- ours: d4 / d5
def run_ours_svd(args, dev, st, L, rank, world, dist):
    import torch
    from gputils_gb300 import workloads, _lib
    from oracle import oracle as O

    nmat = 32 if args.workload == "d4" else 64
    Ah = workloads.d4_svd32(k=_k(8192, args)) if args.workload == "d4" else workloads.d5_svd64(k=_k(32768, args))
    k = Ah.shape[0]
    A0 = to_dev(Ah, dev)
    nsteps = args.warmup + args.steps
    As = [A0.clone() for _ in range(nsteps)]
    S = torch.empty(k * nmat, dtype=torch.float32, device=dev)
    Vt = torch.empty(k * nmat * nmat, dtype=torch.float32, device=dev)
    info = torch.empty(k, dtype=torch.int32, device=dev)
    sweeps = torch.empty(k, dtype=torch.int32, device=dev)

    def step(i):
        _lib.check(L.gbla_sgesvj_batched(nmat, nmat, As[i].data_ptr(), nmat * nmat, S.data_ptr(), nmat,
                                         Vt.data_ptr(), nmat * nmat, None, 0, None, 0, 1e-6, 60,
                                         info.data_ptr(), sweeps.data_ptr(), k, st), "gesvj")

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        e0.record()
        for i in range(args.steps):
            step(args.warmup + i)
        e1.record()
        torch.cuda.synchronize()
    elapsed = e0.elapsed_time(e1) / 1e3
    elapsed_max, units_all = aggregate(elapsed, k * args.steps, world, dist, dev)
    assert (info.cpu().numpy() == 0).all()
    sw = sweeps.cpu().numpy()
    idx = np.arange(0, k, 64 if nmat == 32 else 512)
    Sh = S.cpu().numpy().reshape(k, nmat)
    So = O.gesvj(Ah[idx], tol=1e-12)["S"]
    err = rel_err(Sh[idx][:, None, :], So[:, None, :])
    e2e = _e2e_leg([np.ascontiguousarray(Ah.transpose(0, 2, 1))],
                   lambda ins: (L.gbla_sgesvj_batched(nmat, nmat, ins[0].data_ptr(), nmat * nmat, S.data_ptr(), nmat,
                                                      Vt.data_ptr(), nmat * nmat, None, 0, None, 0, 1e-6, 60,
                                                      info.data_ptr(), sweeps.data_ptr(), k, st),),
                   lambda ins: [S, Vt], k, args, world, dist, dev)
    reflib = None
    if not args.no_reference_library:
        try:
            reflib = reference_library_svd(dev, st, A0, Ah, nmat, args.ref_sample or (512 if nmat == 32 else 128),
                                           S.reshape(k, nmat))
        except Exception as exc:
            reflib = {"unavailable": f"{type(exc).__name__}: {exc}"}
    pk = peaks()
    t = elapsed_max / args.steps
    flops = (4 * nmat ** 3 + 8 * nmat ** 3) * k
    return {
        "metric": metric_name(args.workload), "value": units_all / elapsed_max, "unit": "matrices/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded parametric family)", "config": workload_config(args.workload, args),
        "roofline": {"bound": "fp32 cuda cores", "achieved": flops / t / 1e12, "peak": FP32_PEAK["tflops"],
                     "unit": "TFLOP/s", "frac": flops / t / 1e12 / FP32_PEAK["tflops"],
                     "traffic": traffic_for("svd_d4"), "kernel": "gesvj", "algorithmic_flops_per_launch": flops,
                     "peak_source": FP32_PEAK["source"]},
        "max_rel_err_vs_fp64": {"sigma": err}, "sweeps": {"mean": float(sw.mean()), "max": int(sw.max())},
        "gpu_launches": args.steps, "clocks": clk.summary(), "reference_library": reflib, "e2e": e2e,
    }


def run_ours_d5(args, dev, st, L, rank, world, dist):
    """Learned warm start on the 64 x 64 family: train the network on
    --ws-pairs (A, V) pairs from the cold Jacobi SVD (setup, untimed), then
    time network + Cayley frame + warm Jacobi with cold fallback on the
    32768-matrix batch, next to the cold Jacobi on the same batch."""
    import torch
    from gputils_gb300 import workloads, warmstart as W
    from oracle import oracle as O

    n = 64
    t0 = time.time()
    net, stats = W.train_family_model(n=n, family_seed=6, pairs=args.ws_pairs, epochs=args.ws_epochs,
                                      theta_seed=1234 + rank, seed=rank)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    Ah = workloads.d5_svd64(k=_k(32768, args))
    k = Ah.shape[0]
    A = torch.from_numpy(np.ascontiguousarray(Ah.transpose(0, 2, 1))).to(dev)
    V0 = torch.empty_like(A)
    S = torch.empty((k, n), dtype=torch.float32, device=dev)
    Vt = torch.empty_like(A)
    info = torch.empty(k, dtype=torch.int32, device=dev)
    sweeps = torch.empty(k, dtype=torch.int32, device=dev)
    fb = torch.empty(k, dtype=torch.int32, device=dev)
    budget = net.warm_budget

    def warm_step(Ad):
        net.predict(Ad, out=V0)
        _lib_check(L.gbla_sgesvj_warm_batched(n, n, Ad.data_ptr(), n * n, S.data_ptr(), n, Vt.data_ptr(), n * n,
                                              None, 0, V0.data_ptr(), n * n, budget, 1e-6, 60, info.data_ptr(),
                                              sweeps.data_ptr(), fb.data_ptr(), k, st), "gesvj_warm")

    def cold_step(Ad):
        _lib_check(L.gbla_sgesvj_batched(n, n, Ad.data_ptr(), n * n, S.data_ptr(), n, Vt.data_ptr(), n * n, None,
                                         0, None, 0, 1e-6, 60, info.data_ptr(), sweeps.data_ptr(), k, st), "gesvj")

    def timed(fn, steps, clocks=False):
        for _ in range(args.warmup):
            fn(A)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clk = ClockSampler(torch.cuda.current_device()) if clocks else None
        if clk:
            clk.__enter__()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            fn(A)
        e1.record()
        torch.cuda.synchronize()
        if clk:
            clk.__exit__(None, None, None)
        return e0.elapsed_time(e1) / 1e3, (clk.summary() if clk else None)

    idx = np.arange(0, k, 512)
    So = O.gesvj(Ah[idx], tol=1e-12)["S"]
    # cold, for the comparison
    cold_t, _ = timed(cold_step, max(2, args.steps // 2))
    cold_steps = max(2, args.steps // 2)
    assert (info.cpu().numpy() == 0).all()
    sw_cold = sweeps.cpu().numpy().copy()
    err_cold = rel_err(S.cpu().numpy()[idx][:, None, :], So[:, None, :])
    # warm (the measured path)
    elapsed, clocks = timed(warm_step, args.steps, clocks=True)
    elapsed_max, units_all = aggregate(elapsed, k * args.steps, world, dist, dev)
    assert (info.cpu().numpy() == 0).all()
    sw = sweeps.cpu().numpy()
    fbk = fb.cpu().numpy()
    err = rel_err(S.cpu().numpy()[idx][:, None, :], So[:, None, :])
    # kernel split of one warm step: network + frame, then Jacobi
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record()
    net.predict(A, out=V0)
    e[1].record()
    _lib_check(L.gbla_sgesvj_warm_batched(n, n, A.data_ptr(), n * n, S.data_ptr(), n, Vt.data_ptr(), n * n, None, 0,
                                          V0.data_ptr(), n * n, budget, 1e-6, 60, info.data_ptr(), sweeps.data_ptr(),
                                          fb.data_ptr(), k, st), "gesvj_warm")
    e[2].record()
    torch.cuda.synchronize()
    t_net, t_jac = e[0].elapsed_time(e[1]) / 1e3, e[1].elapsed_time(e[2]) / 1e3

    # end to end: pinned host A in, S and V^T out, every step
    hA = torch.from_numpy(np.ascontiguousarray(Ah.transpose(0, 2, 1))).pin_memory()
    hS = torch.empty((k, n), dtype=torch.float32).pin_memory()
    hVt = torch.empty((k, n, n), dtype=torch.float32).pin_memory()
    Ad = torch.empty_like(A)

    def e2e_step():
        Ad.copy_(hA, non_blocking=True)
        warm_step(Ad)
        hS.copy_(S, non_blocking=True)
        hVt.copy_(Vt, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    esteps = max(3, min(args.steps, 5))
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(esteps):
        e2e_step()
    f1.record()
    torch.cuda.synchronize()
    e2e_t = f0.elapsed_time(f1) / 1e3 / esteps
    e2e_max, _ = aggregate(e2e_t, 0.0, world, dist, dev)

    reflib = None
    if not args.no_reference_library:
        try:
            reflib = reference_library_svd(dev, st, A, Ah, n, args.ref_sample or 128, S)
        except Exception as exc:
            reflib = {"unavailable": f"{type(exc).__name__}: {exc}"}
    t = elapsed_max / args.steps
    flops = (4 * n ** 3 + 8 * n ** 3) * k
    mlp_flops = 2 * (4096 * 512 + 512 * 512 + 512 * 2016) * k
    pk = peaks()
    net.close()
    return {
        "metric": metric_name(args.workload), "value": units_all / elapsed_max, "unit": "matrices/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (network: bf16)",
        "data": "synthetic (seeded parametric family; training pairs from a separate theta stream)",
        "config": workload_config(args.workload, args),
        "roofline": {"bound": "fp32 cuda cores", "achieved": flops / t_jac / 1e12, "peak": FP32_PEAK["tflops"],
                     "unit": "TFLOP/s", "frac": flops / t_jac / 1e12 / FP32_PEAK["tflops"],
                     "traffic": traffic_for("svd_d5_warm"), "kernel": "gesvj (warm), its own launch time",
                     "algorithmic_flops_per_launch": flops,
                     "peak_source": FP32_PEAK["source"]},
        "roofline_network": {"bound": "tensor", "achieved": mlp_flops / t_net / 1e12,
                             "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                             "frac": mlp_flops / t_net / 1e12 / pk["bf16_tflops"],
                             "note": "network GEMMs' flops over the whole predict (GEMMs + Cayley frame) time"},
        "split_ms": {"network_and_frame": t_net * 1e3, "jacobi": t_jac * 1e3},
        "max_rel_err_vs_fp64": {"sigma": err},
        "sweeps": {"mean": float(sw.mean()), "max": int(sw.max()), "fallback_fraction": float(fbk.mean()),
                   "warm_budget": budget},
        "cold": {"value": k * cold_steps / cold_t, "ms_per_step": cold_t / cold_steps * 1e3,
                 "sweeps_mean": float(sw_cold.mean()), "sweeps_max": int(sw_cold.max()),
                 "max_rel_err_vs_fp64": {"sigma": err_cold}},
        "warm_over_cold": (cold_t / cold_steps) / t,
        "training": {"pairs": stats["pairs"], "epochs": stats["epochs"], "seconds": train_s,
                     "loss_first_last": [stats["loss"][0], stats["loss"][-1]],
                     "cold_sweeps_mean_on_training_pairs": stats["cold_sweeps_mean"]},
        "gpu_launches": 6 * args.steps, "clocks": clocks, "reference_library": reflib,
        "e2e": {"value": k / e2e_max, "unit": "matrices/s", "h2d_bytes_per_step": hA.numel() * 4,
                "d2h_bytes_per_step": (hS.numel() + hVt.numel()) * 4},
    }


def _lib_check(status, what):
    from gputils_gb300 import _lib
    _lib.check(status, what)


def reference_library_svd(dev, st, A0, Ah, nmat, sample, S_ours):
    """Svd<float>::factorise: a host loop of cusolverDnSgesvd('N', 'A') over the
    matrices; timed on the first `sample` matrices and scaled (the loop's cost
    is linear in the matrix count)."""
    import torch
    from oracle import oracle as O

    R = RefLib(st)
    sample = min(sample, A0.shape[0])
    lwork = R.L.refp_sgesvd_lwork(nmat, nmat)
    assert lwork >= 0
    work = torch.empty(max(lwork, 1), dtype=torch.float32, device=dev)
    Ac = A0[:sample].clone()
    S = torch.empty(sample * nmat, dtype=torch.float32, device=dev)
    Vt = torch.empty(sample * nmat * nmat, dtype=torch.float32, device=dev)
    info = torch.empty(sample, dtype=torch.int32, device=dev)

    def run():
        assert R.L.refp_sgesvd_loop(nmat, nmat, Ac.data_ptr(), S.data_ptr(), None, Vt.data_ptr(), work.data_ptr(),
                                    lwork, info.data_ptr(), sample, 0) == 0

    Ac.copy_(A0[:sample]); run(); torch.cuda.synchronize()
    Ac.copy_(A0[:sample])
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    e[0].record(); run(); e[1].record()
    torch.cuda.synchronize()
    t = e[0].elapsed_time(e[1]) / 1e3
    So = O.gesvj(Ah[:min(sample, 64)], tol=1e-12)["S"]
    err = rel_err(S.cpu().numpy().reshape(sample, nmat)[:len(So)][:, None, :], So[:, None, :])
    vs_ref = rel_err_t(S_ours[:sample], S.reshape(sample, nmat), sample)
    return {"value": sample / t, "unit": "matrices/s", "sample": sample, "ms_for_sample": t * 1e3,
            "max_rel_err_vs_fp64": {"sigma": err},
            "ours_max_rel_err_vs_reference_output": {"sigma": vs_ref},
            "calls": f"host loop of cusolverDnSgesvd('N','A'), {sample} calls timed, scaled linearly"}


def _e2e_leg(host_inputs, call, outputs, units, args, world, dist, dev):
    """The step through the C ABI with host buffers: every step copies the
    inputs from pinned host memory, runs `call` on the device copies and copies
    `outputs(device inputs)` back to pinned host memory; timed with CUDA events
    over max(3, min(steps, 10)) steps after two untimed ones."""
    import torch
    from gputils_gb300 import _lib

    hin = [torch.from_numpy(np.ascontiguousarray(h)).pin_memory() for h in host_inputs]
    din = [torch.empty(h.shape, dtype=h.dtype, device=dev) for h in hin]
    hout = None

    def one():
        nonlocal hout
        for d, h in zip(din, hin):
            d.copy_(h, non_blocking=True)
        for status in call(din):
            _lib.check(status, "e2e")
        outs = outputs(din)
        if hout is None:
            hout = [torch.empty(o.shape, dtype=o.dtype).pin_memory() for o in outs]
        for h, o in zip(hout, outs):
            h.copy_(o, non_blocking=True)

    for _ in range(2):
        one()
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 10))
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(steps):
        one()
    f1.record()
    torch.cuda.synchronize()
    t, _ = aggregate(f0.elapsed_time(f1) / 1e3 / steps, 0.0, world, dist, dev)
    return {"value": units * world / t, "unit": "matrices/s",
            "h2d_bytes_per_step": int(sum(h.numel() * h.element_size() for h in hin)),
            "d2h_bytes_per_step": int(sum(h.numel() * h.element_size() for h in hout)), "ms_per_step": t * 1e3}


def run_ours_d1(args, dev, st, L, rank, world, dist):
    """CholeskyBatchFactoriser factorise() + solve() on 4096 16x16: the
    reference API path (2 launches: potrf, potrs)."""
    import torch
    from gputils_gb300 import workloads, _lib
    from oracle import oracle as O

    M, b = workloads.d1_cholesky(k=_k(4096, args))
    k, n = M.shape[0], M.shape[1]
    nsteps = args.warmup + args.steps
    Ms = [to_dev(M, dev) for _ in range(nsteps)]
    bs = [to_dev(b, dev) for _ in range(nsteps)]
    info = torch.empty(k, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step(i):
        _lib.check(L.gbla_spotrf_batched(n, Ms[i].data_ptr(), n * n, info.data_ptr(), k, st), "spotrf")
        _lib.check(L.gbla_spotrs_batched(n, 1, Ms[i].data_ptr(), n * n, bs[i].data_ptr(), n, k, st), "spotrs")

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    times = []
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record(); step(args.warmup + i); e[1].record()
            torch.cuda.synchronize()
            times.append(e[0].elapsed_time(e[1]) / 1e3)
    elapsed = sum(times)
    elapsed_max, units_all = aggregate(elapsed, k * args.steps, world, dist, dev)
    x = from_dev(bs[args.warmup], k, n, 1)
    idx = np.arange(0, k, 16)
    _, xo, _ = O.posv(M[idx], b[idx])
    err = rel_err(x[idx], xo)
    e2e = _e2e_leg([np.ascontiguousarray(M.transpose(0, 2, 1)), np.ascontiguousarray(b.transpose(0, 2, 1))],
                   lambda ins: (L.gbla_spotrf_batched(n, ins[0].data_ptr(), n * n, info.data_ptr(), k, st),
                                L.gbla_spotrs_batched(n, 1, ins[0].data_ptr(), n * n, ins[1].data_ptr(), n, k, st)),
                   lambda ins: [ins[1]], k, args, world, dist, dev)
    reflib = None
    if not args.no_reference_library:
        try:
            R = RefLib(st)
            Mr, br = to_dev(M, dev), to_dev(b, dev)
            pa, pb = ptr_array(Mr, k, n * n, dev), ptr_array(br, k, n, dev)
            rinfo = torch.empty(k, dtype=torch.int32, device=dev)
            M0, b0 = Mr.clone(), br.clone()
            tt = []
            for rep in range(args.warmup + args.steps):
                Mr.copy_(M0); br.copy_(b0); flush.zero_()
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                torch.cuda.synchronize()
                e[0].record()
                assert R.L.refp_spotrf_batched(n, pa.data_ptr(), rinfo.data_ptr(), k) == 0
                assert R.L.refp_spotrs_batched(n, pa.data_ptr(), pb.data_ptr(), rinfo.data_ptr(), k) == 0
                e[1].record()
                torch.cuda.synchronize()
                if rep >= args.warmup:
                    tt.append(e[0].elapsed_time(e[1]) / 1e3)
            xr = from_dev(br, k, n, 1)
            reflib = {"value": k / (sum(tt) / len(tt)), "unit": "matrices/s", "ms": sum(tt) / len(tt) * 1e3,
                      "max_rel_err_vs_fp64": {"x": rel_err(xr[idx], xo)},
                      "ours_max_rel_err_vs_reference_output": {"x": rel_err_t(bs[args.warmup], br, k)},
                      "calls": "cusolverDnSpotrfBatched + cusolverDnSpotrsBatched (nrhs = 1)"}
        except Exception as exc:
            reflib = {"unavailable": f"{type(exc).__name__}: {exc}"}
    pk = peaks()
    bytes_ = 4 * (n * n + n * (n + 1) // 2 + 2 * n) * k
    t = elapsed / args.steps
    ach = bytes_ / t / 1e9
    return {
        "metric": metric_name("d1"), "value": units_all / elapsed_max, "unit": "matrices/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_max / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": workload_config("d1", args),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": traffic_for("chol_d1"), "kernel": "potrf+potrs"},
        "max_rel_err_vs_fp64": {"x": err}, "gpu_launches": 2 * args.steps, "clocks": clk.summary(),
        "e2e": e2e, "reference_library": reflib,
    }


def run_chol_large(args, dev, st, L):
    """CholeskyFactoriser<float>::factorise on one large SPD matrix (n = 4096,
    M = G^T G / n + 0.5 I): the blocked whole-GPU path (diagonal blocks on one
    CTA, panel solves on n/64 CTAs, trailing updates on the tensor cores)
    against the reference's cusolverDnSpotrf on the same GPU and input.  The
    factors are checked in FP64 on the GPU: ||L L^T - A|| / ||A||."""
    import torch

    n = args.large_n
    g = torch.Generator(device=dev).manual_seed(4096)
    G = torch.randn(n, n, device=dev, generator=g, dtype=torch.float64) / n ** 0.5
    A64 = G.T @ G + 0.5 * torch.eye(n, device=dev, dtype=torch.float64)
    A0 = A64.float().contiguous()  # symmetric: the same storage in either order
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = torch.empty(max(1, L.gbla_spotrf_large_workspace_bytes(n)), dtype=torch.uint8, device=dev)
    reps = max(3, min(args.steps, 5))

    def timed(call):
        A = A0.clone()
        ts = []
        for rep in range(2 + reps):
            A.copy_(A0)
            torch.cuda.synchronize()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record()
            call(A)
            e[1].record()
            torch.cuda.synchronize()
            if rep >= 2:
                ts.append(e[0].elapsed_time(e[1]))
        return float(np.median(ts)), A

    def resid(A):
        Lf = torch.tril(A.T.double())  # column-major storage read row-major is the transpose
        return float(torch.linalg.matrix_norm(Lf @ Lf.T - A64) / torch.linalg.matrix_norm(A64))

    ms, A = timed(lambda A: _lib_check(L.gbla_spotrf_large(n, A.data_ptr(), n, info.data_ptr(), ws.data_ptr(),
                                                           ws.numel(), st), "spotrf_large"))
    def solve_ms(call, Lf):
        """Median time of one solve with one right-hand side (b ~ N(0,1)), and its solution."""
        b0 = torch.randn(n, device=dev, generator=g)
        b = b0.clone()
        ts = []
        for rep in range(2 + reps):
            b.copy_(b0)
            torch.cuda.synchronize()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record()
            call(Lf, b)
            e[1].record()
            torch.cuda.synchronize()
            if rep >= 2:
                ts.append(e[0].elapsed_time(e[1]))
        return float(np.median(ts)), b0, b

    def solve_err(b0, x):
        r = A64 @ x.double() - b0.double()
        return float(torch.linalg.vector_norm(r) / torch.linalg.vector_norm(b0.double()))

    out = {"config": {"workload": f"CholeskyFactoriser<float>::factorise, one {n}x{n} SPD matrix (G^T G / n + 0.5 I)",
                      "n": n},
           "value": 1e3 / ms, "unit": "matrices/s", "ms": ms, "tflops": n ** 3 / 3 / ms / 1e9,
           "info": int(info.item()), "max_rel_err_vs_fp64": {"LLt_minus_A": resid(A)},
           # per call: a diagonal block per panel, a solve and a partial update for every panel but the last,
           # and a side-stream update while more than 128 columns remain past the panel
           "gpu_launches": (n + 127) // 128 + 2 * ((n + 127) // 128 - 1) + max(0, -(-(n - 256) // 128)),
           "kernels": "k_potrf_diag + k_trsm_panel + k_gemm_bf16_tn (tcgen05, two per panel: next panel's columns "
                      "and the rest, look-ahead on a side stream)"}
    sms, sb0, sx = solve_ms(lambda Lf, b: _lib_check(L.gbla_spotrs_large(n, 1, Lf.data_ptr(), n, b.data_ptr(), n, st),
                                                     "spotrs_large"), A)
    out["solve"] = {"ms": sms, "what": "CholeskyFactoriser<float>::solve, one right-hand side (gbla_spotrs_large)",
                    "residual": solve_err(sb0, sx)}
    if not args.no_reference_library:
        try:
            R = RefLib(st)
            lw = C.c_int(0)
            assert R.L.refp_spotrf_bufsize(n, C.addressof(lw)) == 0
            work = torch.empty(max(1, lw.value), dtype=torch.float32, device=dev)
            rinfo = torch.zeros(1, dtype=torch.int32, device=dev)
            rms, Ar = timed(lambda A: R.L.refp_spotrf(n, C.c_void_p(A.data_ptr()), C.c_void_p(work.data_ptr()),
                                                      lw.value, C.c_void_p(rinfo.data_ptr())))
            lo, lr = torch.tril(A.T.double()), torch.tril(Ar.T.double())
            out["reference_library"] = {
                "value": 1e3 / rms, "unit": "matrices/s", "ms": rms, "info": int(rinfo.item()),
                "max_rel_err_vs_fp64": {"LLt_minus_A": resid(Ar)},
                "ours_max_rel_err_vs_reference_output": {
                    "L": float(torch.linalg.matrix_norm(lo - lr) / torch.linalg.matrix_norm(lr))},
                "calls": "cusolverDnSpotrf(LOWER) with its workspace sized once (CholeskyFactoriser)"}
            out["vs_reference_library"] = rms / ms
            rsms, rb0, rx = solve_ms(lambda Lf, b: R.L.refp_spotrs(n, C.c_void_p(Lf.data_ptr()), C.c_void_p(b.data_ptr()),
                                                                   C.c_void_p(rinfo.data_ptr())), Ar)
            out["reference_library"]["solve"] = {"ms": rsms, "residual": solve_err(rb0, rx),
                                                 "calls": "cusolverDnSpotrs(LOWER, nrhs = 1)"}
        except Exception as exc:
            out["reference_library"] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    return out


def run_ours_large(args, dev, st, L, rank, world, dist):
    """The one-matrix Cholesky as a line of its own (for profile captures)."""
    r = run_chol_large(args, dev, st, L)
    return {"metric": "matrices/s, one large SPD matrix (CholeskyFactoriser<float>::factorise)", "value": r["value"],
            "unit": "matrices/s", "n_gpus": world, "steps": max(3, min(args.steps, 5)), "warmup": 2,
            "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": r["config"], "max_rel_err_vs_fp64": r["max_rel_err_vs_fp64"],
            "gpu_launches": r["gpu_launches"], "reference_library": r.get("reference_library"),
            "tflops": r["tflops"], "solve": r.get("solve")}


def _probe_lib():
    from gputils_gb300 import build

    if not os.path.exists(build.PROBE_LIB):
        build.build_probe()
    L = C.CDLL(build.PROBE_LIB)
    L.peak_fma_throughput.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    return L


def fp32_peak():
    """Measure the FP32 FFMA rate once (about 0.1 s of FMA chains on every SM,
    best of three) while sampling the SM clock; sets FP32_PEAK."""
    import torch

    L = _probe_lib()
    rates = []
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(3):
            g, ms = C.c_double(), C.c_double()
            assert L.peak_fma_throughput(32, 20000, C.byref(g), C.byref(ms)) == 0
            rates.append(g.value / 1e3)
    ck = clk.summary()
    FP32_PEAK.update(tflops=max(rates), sm_mhz=ck.get("sm_mhz"),
                     source=f"FMA probe measured at bench start ({max(rates):.2f} TFLOP/s at "
                            f"{ck.get('sm_mhz')} MHz SM clock)")
    return FP32_PEAK


def print_peaks():
    import torch

    torch.cuda.init()
    L = _probe_lib()
    out = {}
    for prec, iters in ((32, 20000), (64, 200)):
        g, ms = C.c_double(), C.c_double()
        assert L.peak_fma_throughput(prec, iters, C.byref(g), C.byref(ms)) == 0
        out[f"fp{prec}_fma_tflops"] = g.value / 1e3
    print(json.dumps(out), flush=True)


SUMMARY_KEYS = ("value", "unit", "ms_per_step", "config", "launch_config", "roofline", "roofline_network",
                "split_ms", "max_rel_err_vs_fp64", "sweeps", "cold", "warm_over_cold", "training", "e2e",
                "gpu_launches", "clocks", "reference_library", "cpu_baseline")


def workload_summary(line):
    """The fields of one workload's line kept in the default line's `workloads`
    object, plus the ratio to the reference library path on the same GPU."""
    out = {k: line[k] for k in SUMMARY_KEYS if k in line}
    ref = line.get("reference_library") or {}
    if isinstance(ref, dict) and ref.get("value"):
        out["vs_reference_library"] = line["value"] / ref["value"]
        if isinstance(line.get("cold"), dict):
            out["cold"]["vs_reference_library"] = line["cold"]["value"] / ref["value"]
    return out


# the other configurations, run after the headline one in the default line
OTHER_WORKLOADS = (("d1", "f32"), ("d3_f32", "f32"), ("d3_f64", "f64"), ("d4", "f32"), ("d5", "f32"))


def main(argv=None):
    args = parse_args(argv)
    if args.peaks:
        print_peaks()
        return
    if args.impl == "reference":
        run_reference_arm(args)
        return
    import torch
    from gputils_gb300 import build, _lib

    rank, world, local = dist_env()
    dist = dist_init(world, "nccl") if world > 1 else None
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if rank == 0:
        build.build_lib()
        build.build_probe()
    if world > 1:
        dist.barrier()
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    fp32_peak()
    runners = {"d1": run_ours_d1, "d2": run_ours_d2, "d3": run_ours_d3, "d4": run_ours_svd, "d5": run_ours_d5,
               "large": run_ours_large}
    line = runners[args.workload](args, dev, st, L, rank, world, dist)
    cpu = None if args.no_cpu_baseline or rank != 0 or args.workload == "large" else \
        CPU_BASELINES[args.workload](args.cpu_seconds, args)
    line["cpu_baseline"] = cpu
    line["fp32_peak"] = dict(FP32_PEAK)
    if args.workload == "d2" and not args.no_workloads:
        # every other configuration of the metric, measured in the same run
        subs = {}
        for name, dt in OTHER_WORKLOADS:
            sub = argparse.Namespace(**vars(args))
            sub.workload, sub.dtype = name.split("_")[0], dt
            sub.cpu_seconds = min(args.cpu_seconds, 3.0)
            r = runners[sub.workload](sub, dev, st, L, rank, world, dist)
            r["cpu_baseline"] = None if args.no_cpu_baseline or rank != 0 else \
                CPU_BASELINES[sub.workload](sub.cpu_seconds, sub)
            subs[name] = workload_summary(r)
            torch.cuda.empty_cache()
        subs["chol_large_f32"] = run_chol_large(args, dev, st, L)
        line["workloads"] = subs
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
