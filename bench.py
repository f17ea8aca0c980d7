#!/usr/bin/env python
"""Benchmark of the dense factor-and-solve hot path on GB300.

Workload (one step): solve A X = B for one n = 8192 FP64 matrix with entries
iid N(0,1) and 16 right-hand sides iid N(0,1) -- PartialPivLU<MatrixXd> n=8192
with 16 RHS, the configuration the headline metric is quoted on.  A step counts
only if its normwise backward error max_j ||b_j - A x_j||_inf /
(||A||_inf ||x_j||_inf + ||b_j||_inf) is <= 1e-13, recomputed on the GPU in
FP64 after the timed region.

  value        solves/s of the headline path (default: 3xTF32 tensor-core LU +
               FP64 iterative refinement, FP64 fallback built in) with A and B
               resident in HBM (device-buffer C ABI gbs_dgesv_mixed_device)
  plain_fp64   the plain GPU FP64 path (PartialPivLU compute + solve, pivots
               identical to the reference) timed in the same run; the metric
               compares the two
  e2e          the same metric through the host-buffer C ABI (gbs_dgesv_mixed):
               the host->device copy of A and B and the device->host copy of X
               are inside the timed region
  roofline     the dominant kernel's achieved rate (algorithmic work / CUDA-event
               duration of its launches, measured live in the timed region)
               against the peak of its unit
  cpu_baseline the CPU oracle (oracle/, the reference algorithm restated in C,
               OpenMP GEMM) on the host cores: one full factor + 16-RHS solve

--impl reference runs the reference's algorithm on the host cores for the
same workload (the C restatement: the reference is header-only C++ that is not
present on the GPU host) and prints the same JSON line.

Replicas only across GPUs: under torchrun every rank solves its own system;
value is the sum over ranks, time the max over ranks.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Solves/s and TFLOP/s at ≤1e-13 backward err: mixed/batched vs plain FP64"
BE_BAR = 1e-13
# measured DRAM traffic / algorithmic bytes of a kernel (ncu captures, profiles/)
# DRAM traffic / algorithmic bytes of one launch, from the ncu captures summarised in profiles/
TRAFFIC_OVER_ALGORITHMIC = {"gemm": 533.6 / 588.4, "tc_gemm": 237.2 / 289.5}


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--path", default="tf32x3", choices=["fp64", "tf32x3", "tf32", "bf16", "fp16"])
    p.add_argument("--n", type=int, default=8192)
    p.add_argument("--nrhs", type=int, default=16)
    p.add_argument("--plain-steps", type=int, default=3)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--factor-once", action="store_true",
                   help="factor one seeded n x n system on the chosen path and exit (small ncu captures)")
    p.add_argument("--config", default="lu8192", choices=["lu8192", "llt512", "llt16384", "batched", "router", "mbatch"],
                   help="lu8192 is the headline workload; the others are the LLT kappa sweep, the batched "
                        "small systems and the learned router")
    p.add_argument("--train-labels", type=int, default=1000000, help="router: training systems (rcond labels)")
    p.add_argument("--save-router", default="", help="router: write the trained network here (JSON)")
    p.add_argument("--count", type=int, default=20000, help="mbatch: systems of the router workload (n 32..512)")
    return p.parse_args()


def lu_flops(n, nrhs):
    return 2.0 * n ** 3 / 3.0 + 2.0 * n * n * nrhs


# ----------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------- helpers
def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(local)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_hbm_gbs() -> float:
    """HBM copy bandwidth of this machine's GB300 (MEASURED_PEAKS.json, written by the pool's own probe)."""
    try:
        with open(Path(__file__).resolve().parent / "MEASURED_PEAKS.json") as f:
            return float(json.load(f)["hbm_gbs"])
    except Exception:
        return 6800.0


def backward_error_gpu(A, X, B) -> float:
    """max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf), FP64 on the GPU."""
    R = B - A @ X
    an = A.abs().sum(dim=1).max()
    num = R.abs().amax(dim=0)
    den = an * X.abs().amax(dim=0) + B.abs().amax(dim=0)
    return float((num / den).max().item())


def gemm_peak(dtype, n=8192, tf32=False):
    """Measured cuBLAS GEMM throughput (TFLOP/s) of this GPU for a unit that
    MEASURED_PEAKS.json does not list (FP64 DFMA, TF32 tensor)."""
    import torch
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = tf32
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    torch.backends.cuda.matmul.allow_tf32 = old
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def collect_phases(L, steps):
    from eigen_gb300 import _lib
    prof = {}
    for name, ph in _lib.PHASES.items():
        ms = C.c_double(); cnt = C.c_int64(); fl = C.c_double(); by = C.c_double()
        L.gbs_profile_collect(ph, C.byref(ms), C.byref(cnt), C.byref(fl), C.byref(by))
        if cnt.value:
            prof[name] = {"ms": ms.value / steps, "launches": cnt.value / steps,
                          "flops": fl.value / steps, "bytes": by.value / steps}
    L.gbs_profile_reset()
    return prof


# ----------------------------------------------------------------- CPU oracle
def cpu_oracle_solve(a_np, b_np):
    import oracle as O
    t0 = time.perf_counter()
    f, tr, _, _ = O.lu(a_np)
    x = O.lu_solve(f, tr, b_np)
    return x, time.perf_counter() - t0


def cpu_baseline(args, A_host, B_host):
    import oracle as O
    x, dt = cpu_oracle_solve(A_host, B_host)
    be = O.backward_error(A_host, x[:, :1], B_host[:, :1])
    return {"value": 1.0 / dt, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"one full PartialPivLU n={args.n} FP64 factor + {args.nrhs}-RHS solve "
                      f"(oracle/ C restatement, OpenMP GEMM), {dt:.2f} s, backward error {be:.1e}",
            "seconds": dt}


# ----------------------------------------------------------------- reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle as O
    n, nrhs = args.n, args.nrhs
    a = O.gauss(1, n, n)
    b = O.gauss(2, n, nrhs)
    times = []
    for i in range(args.warmup + args.steps):
        _, dt = cpu_oracle_solve(a, b)
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    v = args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: A, B from the seeded generator of oracle/ (Irwin-Hall(12) ~ N(0,1))",
            "config": {"workload": f"PartialPivLU<MatrixXd> n={n} + solve {nrhs} RHS", "n": n, "nrhs": nrhs,
                       "path": "reference algorithm on host cores (C restatement of Eigen's blocked LU)"},
            "tflops": lu_flops(n, nrhs) * v / 1e12,
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
                             "sample": f"full factor + {nrhs}-RHS solve per step"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- our arm
def run_ours(args):
    import numpy as np
    import torch

    import eigen_gb300 as gb
    from eigen_gb300 import _lib
    from eigen_gb300.mixed import RefineInfo, TIERS, options
    world, rank, local = dist_setup(args)
    L = gb.lib()
    n, nrhs = args.n, args.nrhs
    stream = torch.cuda.current_stream()
    g = torch.Generator(device="cuda").manual_seed(1000 + rank)
    A = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g).t()      # column-major view
    B = torch.randn(nrhs, n, dtype=torch.float64, device="cuda", generator=g).t()
    X = torch.empty(nrhs, n, dtype=torch.float64, device="cuda").t()
    tier = TIERS[args.path]
    opt = options(args.path, tol=BE_BAR)
    info = RefineInfo()
    lu = gb.PartialPivLU(dtype=np.float64)
    L.gbs_lu_set_stream(lu._h, C.c_void_p(stream.cuda_stream))

    def step_mixed():
        _lib.check(L.gbs_dgesv_mixed_device(n, nrhs, C.c_void_p(A.data_ptr()), n, C.c_void_p(B.data_ptr()), n,
                                            C.c_void_p(X.data_ptr()), n, C.byref(opt), C.byref(info),
                                            C.c_void_p(stream.cuda_stream)), "gbs_dgesv_mixed_device")

    def step_plain():
        lu.compute(A)
        X.copy_(lu.solve(B))

    step = step_plain if args.path == "fp64" else step_mixed

    def timed(fn, steps, profile):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        barrier(world)
        if profile:
            L.gbs_profile_reset()
            L.gbs_profile_enable(1)
        l0 = L.gbs_kernel_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        launches = L.gbs_kernel_launch_count() - l0
        if profile:
            L.gbs_profile_enable(0)
        return e0.elapsed_time(e1) / 1e3, launches

    clocks = ClockSampler(local)
    clocks.start()
    dt, launches = timed(step, args.steps, True)
    clk = clocks.stop()
    prof = collect_phases(L, args.steps)
    dt_max = max_over_ranks(world, dt)
    be = backward_error_gpu(A, X, B)
    ok = be <= BE_BAR
    value = world * args.steps / dt_max if ok else 0.0
    refine = info.as_dict()

    plain = None
    if args.path != "fp64" and args.plain_steps > 0:
        pdt, _ = timed(step_plain, args.plain_steps, False)
        pbe = backward_error_gpu(A, X, B)
        pdt = max_over_ranks(world, pdt)
        plain = {"value": world * args.plain_steps / pdt, "unit": "solves/s",
                 "ms_per_step": 1e3 * pdt / args.plain_steps, "backward_error": pbe,
                 "tflops": lu_flops(n, nrhs) * world * args.plain_steps / pdt / 1e12}

    # roofline of every phase, the dominant one first
    hbm_peak = measured_hbm_gbs()
    peaks = {}

    def entry(name, ph):
        t = ph["ms"] / 1e3
        if name == "tc_gemm":
            if "tf32" not in peaks:
                peaks["tf32"] = gemm_peak(torch.float32, tf32=True)
            e = {"bound": "tensor", "kernel": "tc_gemm_kernel (tcgen05 kind::tf32, 3xTF32 split)",
                 "achieved": ph["flops"] / t / 1e12 if t else 0.0, "peak": peaks["tf32"], "unit": "TFLOP/s",
                 "peak_source": "of measured: cuBLAS TF32 GEMM 8192^3 timed in this run"}
        elif name in ("gemm", "syrk", "residual"):
            if "fp64" not in peaks:
                peaks["fp64"] = gemm_peak(torch.float64)
            e = {"bound": "fp64", "kernel": {"gemm": "gemm_sub_kernel<double> (trailing update)",
                                             "syrk": "gemm_sub_kernel<double> lower (SYRK)",
                                             "residual": "mv_partial_kernel (FP64 r = b - A x)"}[name],
                 "achieved": ph["flops"] / t / 1e12 if t else 0.0, "peak": peaks["fp64"], "unit": "TFLOP/s",
                 "peak_source": "of measured: cuBLAS DGEMM 8192^3 timed in this run (FP64 has no entry in "
                                "MEASURED_PEAKS.json)"}
        else:
            e = {"bound": "hbm", "kernel": name, "achieved": ph["bytes"] / t / 1e9 if t else 0.0, "peak": hbm_peak,
                 "unit": "GB/s", "peak_source": "of measured: MEASURED_PEAKS.json hbm_gbs",
                 "note": "latency-bound (barrier or dependency chain per column / block): the fraction shows "
                         "the distance from the memory roof"}
        e["frac"] = e["achieved"] / e["peak"] if e["peak"] else None
        ratio = TRAFFIC_OVER_ALGORITHMIC.get(name)
        e["traffic"] = (ratio * ph["bytes"] / max(ph["launches"], 1)) if ratio else None
        e.update({"phase": name, "share_of_step": ph["ms"] / (1e3 * dt / args.steps),
                  "launches_per_step": ph["launches"], "algorithmic_bytes_per_launch": ph["bytes"] / max(ph["launches"], 1),
                  "algorithmic_flops_per_launch": ph["flops"] / max(ph["launches"], 1)})
        return e

    order = sorted(prof.items(), key=lambda kv: -kv[1]["ms"])
    roofline = entry(*order[0]) if order else None
    roofline_phases = [entry(k, v) for k, v in order[1:]]

    # end to end through the host-buffer C ABI
    e2e = None
    if not args.no_e2e:
        Ah = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
        Ah.copy_(A.t())                    # row-major A^T == column-major A
        Bh = torch.empty((nrhs, n), dtype=torch.float64, pin_memory=True)
        Bh.copy_(B.t())
        Xh = torch.empty((nrhs, n), dtype=torch.float64, pin_memory=True)
        pa, pb, px = C.c_void_p(Ah.data_ptr()), C.c_void_p(Bh.data_ptr()), C.c_void_p(Xh.data_ptr())
        einfo = RefineInfo()
        h = lu._h

        def e2e_step():
            if args.path == "fp64":
                _lib.check(L.gbs_lu_compute(h, n, pa, n), "compute")
                _lib.check(L.gbs_lu_solve(h, nrhs, pb, n, px, n, 0), "solve")
            else:
                _lib.check(L.gbs_dgesv_mixed(n, nrhs, pa, n, pb, n, px, n, C.byref(opt), C.byref(einfo)),
                           "gbs_dgesv_mixed")

        for _ in range(max(1, args.warmup)):
            e2e_step()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        t_e2e = max_over_ranks(world, time.perf_counter() - t0)
        be2 = backward_error_gpu(A, Xh.to("cuda").t(), B)
        e2e = {"value": (world * args.steps / t_e2e) if be2 <= BE_BAR else 0.0, "unit": "solves/s",
               "h2d_bytes_per_step": 8 * (n * n + n * nrhs), "d2h_bytes_per_step": 8 * n * nrhs,
               "backward_error": be2,
               "api": ("gbs_dgesv_mixed" if args.path != "fp64" else "gbs_lu_compute + gbs_lu_solve") +
                      " on pinned host buffers"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args, np.asfortranarray(A.cpu().numpy()), np.asfortranarray(B.cpu().numpy()))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * dt_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic: A iid N(0,1), B iid N(0,1) (torch.randn on the GPU, seeded)",
                "config": {"workload": f"PartialPivLU<MatrixXd> n={n} FP64 + solve {nrhs} RHS", "n": n,
                           "nrhs": nrhs, "path": args.path, "parallelism": f"replicas x{world}",
                           "l2": "inputs (512 MB) larger than L2 (129 MB); no flush needed"},
                "tflops": lu_flops(n, nrhs) * value / 1e12, "backward_error": be, "refinement": refine,
                "plain_fp64": plain, "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
                "e2e": e2e, "roofline": roofline, "roofline_other_phases": roofline_phases, "cpu_baseline": cpu,
                "clocks": clk,
                "gpu_launches": int(launches), "phases_ms_per_step": {k: round(v["ms"], 3) for k, v in prof.items()}}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def factor_once(args):
    import numpy as np
    import torch

    import eigen_gb300 as gb
    n = args.n
    a = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(3)).t()
    b = torch.randn(1, n, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(4)).t()
    torch.cuda.synchronize()
    if args.path == "fp64":
        lu = gb.PartialPivLU(a)
        torch.cuda.synchronize()
        ok = lu.first_zero_pivot() < 0
        out = {"first_zero_pivot": lu.first_zero_pivot()}
    else:
        x, info = gb.solve_mixed(a, b, tier=args.path)
        torch.cuda.synchronize()
        ok = info["backward_error"] <= BE_BAR
        out = info
    print(json.dumps({"factor_once": n, "path": args.path, **out}))
    return 0 if ok else 1


def _event_time(fn, reps=1):
    import torch
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    out = None
    for _ in range(reps):
        out = fn()
    e1.record(s)
    torch.cuda.synchronize()
    return out, e0.elapsed_time(e1) / 1e3 / reps


def run_llt512(args):
    """LLT<MatrixXd> n = 512: A = G G^T / 512 + I (G iid N(0,1)), one RHS,
    plain FP64 through the LLT object on device buffers (and end to end from
    host buffers), parity against the oracle on the same input, the oracle
    port timed beside it on the host cores."""
    import numpy as np
    import torch

    import oracle as O
    import eigen_gb300 as gb
    n = 512
    G = O.gauss(42, n, n)
    a = np.asfortranarray(G @ G.T / n + np.eye(n))
    b = O.gauss(43, n, 1)
    A = torch.from_numpy(a).cuda().t().contiguous().t()
    Bd = torch.from_numpy(b).cuda().t().contiguous().t()
    llt = gb.LLT(dtype=np.float64)
    L = gb.lib()
    stream = torch.cuda.current_stream()
    L.gbs_llt_set_stream(llt._h, C.c_void_p(stream.cuda_stream))

    def step():
        llt.compute(A)
        return llt.solve(Bd)
    for _ in range(args.warmup):
        step()
    l0 = L.gbs_kernel_launch_count()
    X, dt = _event_time(step, reps=args.steps)
    launches = (L.gbs_kernel_launch_count() - l0) // args.steps
    L.gbs_profile_reset()
    L.gbs_profile_enable(1)
    step()
    torch.cuda.synchronize()
    phases = {k: round(v["ms"], 4) for k, v in collect_phases(L, 1).items()}
    L.gbs_profile_enable(0)
    x = X.cpu().numpy()
    f_o, _ = O.llt(a)
    x_o = O.llt_solve(f_o, b)
    fwd = float(np.linalg.norm(x - x_o) / np.linalg.norm(x_o))
    be = O.backward_error(a, x, b)
    # end to end: host buffers through the same object (copies inside the timed region)
    llt_h = gb.LLT(dtype=np.float64)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        llt_h.compute(a)
        llt_h.solve(b)
    e2e = args.steps / (time.perf_counter() - t0)
    # CPU oracle (the reference algorithm, same input)
    t0 = time.perf_counter()
    reps = 20
    for _ in range(reps):
        f_c, _ = O.llt(a)
        O.llt_solve(f_c, b)
    cpu = reps / (time.perf_counter() - t0)
    flops = n ** 3 / 3 + 2 * n * n
    line = {"metric": METRIC, "value": 1.0 / dt, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic: A = G G^T / 512 + I, G iid N(0,1) (seed 42), b (seed 43)",
            "config": {"workload": "LLT<MatrixXd> n=512 + solve 1 RHS, plain FP64", "n": n, "nrhs": 1},
            "tflops": flops / dt / 1e12, "backward_error": be, "forward_diff_vs_oracle": fwd,
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": 8 * (n * n + n),
                    "d2h_bytes_per_step": 8 * n, "api": "gbs_llt_compute / gbs_llt_solve on host buffers"},
            "cpu_baseline": {"value": cpu, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
                             "sample": f"{reps} factor + solve of the same system"},
            "gpu_launches": int(launches), "phases_ms_per_step": phases,
            "roofline": {"bound": "latency", "note": "n = 512: 4.5e7 flop per solve, far below any roofline"}}
    print(json.dumps(line), flush=True)
    return 0


def run_llt16384(args):
    """LLT n = 16384, A = Q diag(sigma) Q^T (Haar Q, sigma log-spaced 1..kappa),
    4 right-hand sides, kappa in {1e2, 1e6, 1e10}: every tier's solves/s at
    backward error <= 1e-13 and its forward error against the FP64 solution."""
    import numpy as np
    import torch

    import eigen_gb300 as gb
    n, nrhs = 16384 if args.n == 8192 else args.n, 4
    g = torch.Generator(device="cuda").manual_seed(7)
    G = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    Q, Rq = torch.linalg.qr(G)
    Q = Q * torch.sign(torch.diagonal(Rq))
    del G, Rq
    B = torch.randn(nrhs, n, dtype=torch.float64, device="cuda", generator=g).t()
    flops = n ** 3 / 3.0 + 2.0 * n * n * nrhs
    per_kappa = {}
    best = None
    for kappa in (1e2, 1e6, 1e10):
        s = torch.logspace(0, float(np.log10(kappa)), n, dtype=torch.float64, device="cuda")
        A = (Q * s) @ Q.t()
        A = ((A + A.t()) / 2).contiguous().t()
        x64, _ = gb.solve_spd_mixed(A, B, tier="fp64")
        rows = {}
        Lb = gb.lib()
        for tier in ("fp64", "tf32x3", "fp16", "bf16"):
            gb.solve_spd_mixed(A, B, tier=tier)
            (X, info), dt = _event_time(lambda: gb.solve_spd_mixed(A, B, tier=tier))
            Lb.gbs_profile_reset()
            Lb.gbs_profile_enable(1)
            gb.solve_spd_mixed(A, B, tier=tier)
            torch.cuda.synchronize()
            phases = {k: round(v["ms"], 3) for k, v in collect_phases(Lb, 1).items()}
            Lb.gbs_profile_enable(0)
            be = backward_error_gpu(A, X, B)
            fe = float(((X - x64).abs().amax(0) / x64.abs().amax(0)).max().item())
            rows[tier] = {"solves_per_s": 1.0 / dt if be <= BE_BAR else 0.0, "ms": 1e3 * dt,
                          "tflops": flops / dt / 1e12, "backward_error": be, "forward_error_vs_fp64": fe,
                          "refine": info, "phases_ms": phases}
        fastest = max(rows, key=lambda t: rows[t]["solves_per_s"])
        per_kappa[f"{kappa:.0e}"] = {"tiers": rows, "fastest": fastest,
                                     "speedup_vs_fp64": rows[fastest]["solves_per_s"] / rows["fp64"]["solves_per_s"]}
        if kappa == 1e2:
            best = rows[fastest]
        del A
    line = {"metric": METRIC, "value": best["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": best["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: A = Q diag(sigma) Q^T, Q Haar (QR of seeded Gaussian), B iid N(0,1)",
            "config": {"workload": f"LLT<MatrixXd> n={n}, {nrhs} RHS, kappa sweep (value: kappa=1e2, fastest tier)",
                       "n": n, "nrhs": nrhs}, "per_kappa": per_kappa}
    print(json.dumps(line), flush=True)
    return 0


def run_batched(args):
    """100,000 SPD systems n ~ U{3..24} (G G^T + 0.1 I) and 20,000 general n ~
    U{4..64} (iid N(0,1)), one RHS each, FP64 and FP32: one graph launch per
    batch; per-matrix plain GPU (sampled) and the CPU oracle beside it."""
    import numpy as np
    import torch

    import oracle as O
    import eigen_gb300 as gb
    from eigen_gb300.batched import BatchedSolver
    rng = np.random.default_rng(0)
    sizes = np.concatenate([rng.integers(3, 25, 100000), rng.integers(4, 65, 20000)]).astype(np.int32)
    kinds = np.concatenate([np.zeros(100000), np.ones(20000)]).astype(np.int32)
    out = {}
    for dtype, tdt, name in ((np.float64, torch.float64, "f64"), (np.float32, torch.float32, "f32")):
        bs = BatchedSolver(sizes, kinds, dtype=dtype)
        g = torch.Generator(device="cuda").manual_seed(1)
        ah = np.empty(bs.a_elems, dtype=np.float64)
        for i, n in enumerate(sizes):
            m = rng.standard_normal((n, n))
            if kinds[i] == 0:
                m = m @ m.T + 0.1 * np.eye(n)
            ah[bs.a_off[i]:bs.a_off[i] + n * n] = m.reshape(-1, order="F")
        A0 = torch.from_numpy(ah).to(tdt).cuda()
        B0 = torch.randn(bs.b_elems, dtype=tdt, device="cuda", generator=g)
        A, B = A0.clone(), B0.clone()
        info = torch.empty(len(sizes), dtype=torch.int32, device="cuda")
        piv = torch.empty(bs.b_elems, dtype=torch.int32, device="cuda")
        dflt = []                                  # the plan's default variants, before autotuning
        for _ in range(max(args.warmup, 3) + 3):
            A.copy_(A0); B.copy_(B0)
            dflt.append(_event_time(lambda: bs.solve(A, B, info, piv))[1])
        dflt = min(dflt[-3:])
        cfg = bs.autotune(A.clone(), B.clone(), info, piv)
        times = []
        for _ in range(args.warmup + args.steps):
            A.copy_(A0); B.copy_(B0)
            _, dt = _event_time(lambda: bs.solve(A, B, info, piv))
            times.append(dt)
        dt = min(times[args.warmup:])
        failures = int((info >= 0).sum().item())
        # per-matrix plain GPU path on a sample of 200 items
        idx = rng.choice(len(sizes), 200, replace=False)
        t0 = time.perf_counter()
        for i in idx:
            n = int(sizes[i])
            m = ah[bs.a_off[i]:bs.a_off[i] + n * n].reshape((n, n), order="F").astype(dtype)
            bvec = B0[bs.b_off[i]:bs.b_off[i] + n].cpu().numpy()
            (gb.LLT(m, dtype=dtype) if kinds[i] == 0 else gb.PartialPivLU(m, dtype=dtype)).solve(bvec)
        per_matrix = 200 / (time.perf_counter() - t0)
        # CPU oracle
        a_np = ah.astype(dtype)
        b_np = B0.cpu().numpy().copy()
        lib = O.port()
        sfx = "d" if dtype == np.float64 else "s"
        t0 = time.perf_counter()
        getattr(lib, f"oracle_batched_llt_solve_{sfx}")(
            100000, np.ascontiguousarray(sizes[:100000]), np.ascontiguousarray(bs.a_off[:100000]),
            a_np.ctypes.data_as(C.c_void_p), np.ascontiguousarray(bs.b_off[:100000]), b_np.ctypes.data_as(C.c_void_p),
            np.zeros(100000, dtype=np.int32))
        getattr(lib, f"oracle_batched_lu_solve_{sfx}")(
            20000, np.ascontiguousarray(sizes[100000:]), np.ascontiguousarray(bs.a_off[100000:120000]),
            a_np.ctypes.data_as(C.c_void_p), np.ascontiguousarray(bs.b_off[100000:120000]),
            b_np.ctypes.data_as(C.c_void_p), np.zeros(bs.b_elems, dtype=np.int32), np.zeros(20000, dtype=np.int32))
        cpu = len(sizes) / (time.perf_counter() - t0)
        flops = float(np.sum(np.where(kinds == 0, sizes ** 3 / 3 + 2 * sizes ** 2, 2 * sizes ** 3 / 3 + 2 * sizes ** 2)))
        byts = float(np.sum(2 * sizes.astype(np.float64) ** 2 + 3 * sizes)) * np.dtype(dtype).itemsize
        out[name] = {"solves_per_s": len(sizes) / dt, "ms": 1e3 * dt, "tflops": flops / dt / 1e12,
                     "hbm_gbs": byts / dt / 1e9, "failures": failures, "autotuned": cfg,
                     "default_variants_ms": 1e3 * dflt,
                     "per_matrix_plain_gpu_solves_per_s": per_matrix, "cpu_oracle_solves_per_s": cpu,
                     "cpu_cores": O.num_threads()}
    fp64_peak = gemm_peak(torch.float64)
    tf = out["f64"]["tflops"]
    line = {"metric": METRIC, "value": out["f64"]["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["f64"]["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: SPD G G^T + 0.1 I (n 3..24), general iid N(0,1) (n 4..64), seeded",
            "config": {"workload": "batched: 100,000 LLT + 20,000 PartialPivLU, 1 RHS each, one CUDA-graph launch",
                       "count": int(len(sizes))},
            "gpu_launches": len(out["f64"]["autotuned"]["buckets"]),
            "roofline": {"bound": "fp64", "achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s", "frac": tf / fp64_peak,
                         "traffic": None,
                         "peak_source": "cuBLAS DGEMM measured in this run (MEASURED_PEAKS.json lists no FP64 unit)",
                         "note": "algorithmic flops per item: n^3/3 + 2n^2 (LLT), 2n^3/3 + 2n^2 (LU); one kernel "
                                 "per size group, all in one graph"},
            "batched": out}
    print(json.dumps(line), flush=True)
    return 0


def run_router(args):
    """20,000 general systems n ~ U{32..512}, A = U diag(s) V^T, log10 kappa ~
    U[1, 12]; the router (trained on rcond labels the method produces) against
    always-FP64 and try-lowest-then-fallback, all at backward error <= 1e-13."""
    import numpy as np
    import torch

    from eigen_gb300 import router as R
    ntrain = args.train_labels
    feats, labs = [], []
    t_gen = t_lab = t_feat = 0.0
    chunk = 20000
    pool = R.HaarPool(16, torch.Generator(device="cuda").manual_seed(99))
    for c0 in range(0, ntrain, chunk):
        (mb, A, _, _), dt = R.timed(lambda: R.generate(min(chunk, ntrain - c0), seed=1000 + c0, nmin=32, nmax=512,
                                                       pool=pool))
        t_gen += dt
        y, dt = R.timed(lambda: R.labels(mb, A))
        labs.append(y)
        t_lab += dt
        f, dt = R.timed(lambda: R.features(mb, A))
        feats.append(f)
        t_feat += dt
        del A, mb
    Ftr = torch.cat(feats).contiguous()
    Ytr = torch.cat(labs).contiguous()
    del pool
    r = R.Router(seed=1)
    (loss, t_fit) = R.timed(lambda: r.fit(Ftr, Ytr, epochs=12, batch=2048, lr=2e-3))
    if args.save_router:
        r.save(args.save_router)
    mt, At, Bt, logk = R.generate(20000, seed=7, nmin=32, nmax=512)
    from eigen_gb300 import _lib
    Lb = _lib.lib()
    # always FP64 (the batched FP64 kernel; the plain GPU FP64 path per matrix is sampled below)
    R.solve_fp64(mt, At, Bt)
    X64, t64 = R.timed(lambda: R.solve_fp64(mt, At, Bt))
    # try-lowest-then-fallback: FP32 + IR on everything, GMRES-IR on the same
    # factors for what it leaves, FP64 for the rest
    R.solve_cascade(mt, At, Bt)
    (Xtry, st_try), t_try = R.timed(lambda: R.solve_cascade(mt, At, Bt))
    # kernel phases of the FP64 and FP32 tiers on everything (separate, profiled runs)
    Lb.gbs_profile_reset()
    Lb.gbs_profile_enable(1)
    R.solve_fp64(mt, At, Bt)
    torch.cuda.synchronize()
    ph64 = collect_phases(Lb, 1)
    ws = R.Fp32Work(mt)
    R.solve_fp32_ir(mt, At, Bt, ws=ws)
    torch.cuda.synchronize()
    ph32 = collect_phases(Lb, 1)
    st_ir = ws.status.cpu().numpy().copy()
    R.solve_fp32_gmres(mt, At, Bt, items=torch.nonzero(ws.status == -1).flatten().to(torch.int32), ws=ws,
                       factored=True)
    torch.cuda.synchronize()
    phgm = collect_phases(Lb, 1)
    Lb.gbs_profile_enable(0)
    st_gm = ws.status.cpu().numpy()
    inner = ws.inner.cpu().numpy()
    by_kappa = {}
    for lo in range(1, 12):
        sel = (logk >= lo) & (logk < lo + 1)
        fail_ir = sel & (st_ir < 0)
        by_kappa[f"{lo}-{lo + 1}"] = {
            "ir_converged": float((st_ir[sel] >= 0).mean()),
            "gmres_converged_of_ir_failures": float((st_gm[fail_ir] >= 0).mean()) if fail_ir.any() else None,
            "gmres_mean_inner": float(inner[fail_ir].mean()) if fail_ir.any() else None}
    # routed: features + network + tier choice on the GPU, then each tier
    R.route_and_solve(r, mt, At, Bt)
    (Xr, st_r), t_r = R.timed(lambda: R.route_and_solve(r, mt, At, Bt))
    _, t_features = R.timed(lambda: R.features(mt, At))
    import eigen_gb300 as gb
    psample = np.random.default_rng(1).choice(mt.count, 100, replace=False)
    t0 = time.perf_counter()
    for i in psample:
        gb.PartialPivLU(mt.matrix(At, i).contiguous().t()).solve(mt.vector(Bt, i).reshape(-1, 1).contiguous())
    torch.cuda.synchronize()
    per_matrix = len(psample) / (time.perf_counter() - t0)
    sample = np.random.default_rng(0).choice(mt.count, 500, replace=False)
    def worst(X):
        errs = np.array([float(((mt.vector(Bt, i) - mt.matrix(At, i) @ mt.vector(X, i)).abs().max() /
                                (mt.matrix(At, i).abs().sum(1).max() * mt.vector(X, i).abs().max() +
                                 mt.vector(Bt, i).abs().max())).item()) for i in sample])
        return float(errs.max())
    pred = r.predict(R.features(mt, At))
    ytest = R.labels(mt, At)
    res = {"always_fp64": {"solves_per_s": mt.count / t64, "s": t64, "worst_backward_error_sample": worst(X64)},
           "try_lowest_then_fallback": {"solves_per_s": mt.count / t_try, "s": t_try, **st_try,
                                        "worst_backward_error_sample": worst(Xtry)},
           "router": {"solves_per_s": mt.count / t_r, "s": t_r, **st_r, "worst_backward_error_sample": worst(Xr)},
           "per_matrix_plain_gpu_fp64": {"solves_per_s": per_matrix, "sample": len(psample)},
           "phases_ms": {"fp64_all": {k: v["ms"] for k, v in ph64.items()},
                         "fp32_ir_all": {k: v["ms"] for k, v in ph32.items()},
                         "gmres_ir_on_ir_failures": {k: v["ms"] for k, v in phgm.items()}},
           "tier_convergence_by_log10_kappa": by_kappa,
           "features_s": t_features,
           "network": {"train_systems": int(ntrain), "generate_s": t_gen, "labels_s": t_lab, "features_s": t_feat,
                       "fit_s": t_fit,
                       "final_train_mse_scaled": loss,
                       "test_median_abs_err_log10_kappa": float((pred - ytest).abs().median().item()),
                       "t_ir_log10_kappa": r.t_ir, "t_gmres_log10_kappa": r.t_gmres}}
    line = {"metric": METRIC, "value": res["router"]["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": 1,
            "warmup": 0, "ms_per_step": 1e3 * t_r, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic: A = U diag(s) V^T, Haar U, V, log10 kappa ~ U[1,12], seeded",
            "config": {"workload": "router: 20,000 PartialPivLU systems n 32..512, 1 RHS", "count": 20000},
            "router": res}
    print(json.dumps(line), flush=True)
    return 0


def run_mbatch(args):
    """The router workload's medium batch (n ~ U{32..512}, log10 kappa ~
    U[1, 12]) through each tier once: FP64 LU + solve, FP32 LU + FP64
    refinement (small counts keep an ncu capture short)."""
    import torch

    from eigen_gb300 import router as R
    mt, At, Bt, _ = R.generate(args.count, seed=7, nmin=32, nmax=512)
    _, t64 = R.timed(lambda: R.solve_fp64(mt, At, Bt))
    (_, st), t32 = R.timed(lambda: R.solve_fp32_ir(mt, At, Bt))
    conv = int((st >= 0).sum().item())
    print(json.dumps({"config": "mbatch", "count": args.count, "fp64_s": t64, "fp32_ir_s": t32,
                      "fp32_converged": conv}), flush=True)
    return 0


def main():
    args = args_parse()
    if args.factor_once:
        return factor_once(args)
    if args.impl == "ours" and args.config != "lu8192":
        return {"llt512": run_llt512, "llt16384": run_llt16384, "batched": run_batched, "router": run_router,
                "mbatch": run_mbatch}[args.config](args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
