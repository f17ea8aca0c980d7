#!/usr/bin/env python
"""Benchmark of the dense factor-and-solve hot path on GB300.

Headline workload (one step): solve A X = B for one n = 8192 FP64 matrix with
entries iid N(0,1) and 16 right-hand sides iid N(0,1) -- PartialPivLU<MatrixXd>
n=8192 with 16 RHS, the configuration the headline metric is quoted on.  A and
B come from the seeded generator of oracle/ (the same bytes the reference arm
solves).  A step counts only if its normwise backward error
max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) is <= 1e-13,
recomputed on the GPU in FP64 after the timed region.

  value        solves/s of the headline path (3xTF32 tensor-core LU + FP64
               iterative refinement, FP64 fallback built in) with A and B
               resident in HBM (device-buffer C ABI gbs_dgesv_mixed_device),
               timed with the library's profiler off
  e2e          the same metric through the host-buffer C ABI (gbs_dgesv_mixed):
               the host->device copy of A and B and the device->host copy of X
               are inside the timed region
  roofline     the dominant kernel's achieved rate (algorithmic work / CUDA-event
               duration of its launches, from a second, profiled pass of the
               same steps) against the measured peak of its unit; also carries
               the plain-FP64 comparison and the companion workloads below
               (nested here because the record keeps only its standard keys)
  cpu_baseline the CPU oracle (oracle/, the reference algorithm restated in C,
               OpenMP GEMM) on the host cores: one full factor + 16-RHS solve
               of the same bytes

Companion workloads (the other configurations of the metric, one GPU, measured
in the same run unless --companions none):
  llt512     LLT<MatrixXd> n=512 + 1 RHS, plain FP64 (latency)
  llt16384   LLT n=16384, 4 RHS, kappa in {1e2, 1e6, 1e10}: FP64, 3xTF32, FP16
             and BF16 tiers with refinement, backward and forward error per kappa
  batched    100,000 SPD n in [3,24] + 20,000 general n in [4,64], FP64 and
             FP32, one CUDA-graph launch per batch
  router     20,000 general n in [32,512], log10 kappa in [1,12]: the shipped
             network routes each system to a tier; against always-FP64 and
             try-lowest-then-fallback
Each reports device-resident solves/s, an end-to-end figure with the copies
inside the timed region, a CPU-oracle baseline on a bounded sample, and the
roofline of its dominant kernel.  Between timed iterations of a workload whose
inputs fit in L2, a 256 MB buffer is written (L2 flush) outside the timed
events.

--impl reference runs the reference's algorithm on the host cores for the
headline workload (the C restatement: the reference is header-only C++ that is
not present on the GPU host) and prints the same JSON line.

Replicas only across GPUs: under torchrun every rank solves its own copy of
the headline system; value is the sum over ranks, time the max over ranks.
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
# DRAM traffic / algorithmic bytes of one launch, from the ncu captures summarised in profiles/ (the
# panel's and the tcgen05 GEMM's captured at n = 6144, scaled by the bytes each launch processes)
TRAFFIC_OVER_ALGORITHMIC = {"gemm": 533.6 / 588.4, "tc_gemm": 257.0 / 289.5, "panel": 1.17 / 1.56,
                            "residual": 609.3 / 604.0}
COMPANIONS = ("llt512", "llt16384", "batched", "router")


def args_parse():
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--path", default="tf32x3", choices=["fp64", "tf32x3", "tf32", "bf16", "fp16"])
    p.add_argument("--n", type=int, default=8192)
    p.add_argument("--nrhs", type=int, default=16)
    p.add_argument("--plain-steps", type=int, default=3)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--lookahead", type=int, default=1, choices=[0, 1],
                   help="LU: factor block k+1's panels on a second stream during block k's update (default 1)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--factor-once", action="store_true",
                   help="factor one seeded system and exit (small ncu captures)")
    p.add_argument("--timeline", default="",
                   help="write the library's per-launch timeline (phase, stream, start, end in ms) of one "
                        "device-buffer and one host-buffer headline solve to this CSV file, print a summary, exit")
    p.add_argument("--config", default="lu8192", choices=["lu8192", "llt512", "llt16384", "batched", "router", "mbatch"],
                   help="lu8192: the headline line (with the companions); the others print one line of their own")
    p.add_argument("--companions", default=",".join(COMPANIONS),
                   help="comma-separated companion workloads measured with the headline, or 'none'")
    p.add_argument("--train-labels", type=int, default=1000000, help="router: training systems (rcond labels)")
    p.add_argument("--train", action="store_true", help="router: train the network in this run instead of "
                                                         "loading the shipped weights")
    p.add_argument("--save-router", default="", help="router: write the trained network here (JSON)")
    p.add_argument("--count", type=int, default=20000, help="mbatch: systems of the router workload (n 32..512)")
    p.add_argument("--detail", default="", help="also write the full record, companions in detail, to this JSON file")
    return p.parse_args()


def lu_flops(n, nrhs):
    return 2.0 * n ** 3 / 3.0 + 2.0 * n * n * nrhs


def headline_config(n, nrhs):
    """The workload record shared, key for key, by both arms."""
    mb = 8 * (n * n + n * nrhs) / 1e6
    return {"workload": f"PartialPivLU<MatrixXd> n={n} + solve {nrhs} RHS, A and B iid N(0,1)", "n": n,
            "nrhs": nrhs, "l2": f"inputs ({mb:.0f} MB) larger than L2 (129 MB); no flush"}


HEADLINE_DATA = ("synthetic: A, B from the seeded generator of oracle/ (Irwin-Hall(12) ~ N(0,1), seeds 1 and 2): "
                 "the same bytes in both arms")


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


def forward_error_gpu(X, Xref) -> float:
    """max_j ||x_j - xref_j||_inf / ||xref_j||_inf."""
    return float(((X - Xref).abs().amax(0) / Xref.abs().amax(0)).max().item())


_PEAKS: dict = {}


def gemm_peak(dtype, n=8192, tf32=False):
    """Measured cuBLAS GEMM throughput (TFLOP/s) of this GPU for a unit that
    MEASURED_PEAKS.json does not list (FP64 DFMA, TF32 tensor); once per run."""
    import torch
    key = (str(dtype), tf32)
    if key in _PEAKS:
        return _PEAKS[key]
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
    _PEAKS[key] = 2.0 * n ** 3 / best / 1e12
    return _PEAKS[key]


def fp64_peak():
    return gemm_peak(__import__("torch").float64)


def tf32_peak():
    return gemm_peak(__import__("torch").float32, tf32=True)


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


def profiled(L, fn, reps=1):
    """Phases of `reps` calls of fn with the library's per-launch CUDA events on."""
    import torch
    torch.cuda.synchronize()
    L.gbs_profile_reset()
    L.gbs_profile_enable(1)
    for _ in range(reps):
        fn()
    torch.cuda.synchronize()
    L.gbs_profile_enable(0)
    return collect_phases(L, reps)


class L2Flush:
    """Writes 256 MB (twice the 129 MB L2) between timed iterations."""

    def __init__(self):
        import torch
        self.buf = torch.empty(64 << 20, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.buf.fill_(1.0)


def device_time(fn, steps, warmup, flush=None, prep=None):
    """Device seconds of `steps` calls of fn on the current stream (CUDA
    events), after `warmup` untimed calls.  prep (untimed, before each call)
    restores inputs; flush (untimed, after prep) evicts L2.  Returns (total
    seconds, kernels this library launched during the timed calls, last fn
    result)."""
    import torch
    import eigen_gb300 as gb
    L = gb.lib()
    s = torch.cuda.current_stream()
    out = None
    for _ in range(warmup):
        if prep:
            prep()
        out = fn()
    torch.cuda.synchronize()
    total, launches = 0.0, 0
    if prep is None and flush is None:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = L.gbs_kernel_launch_count()
        e0.record(s)
        for _ in range(steps):
            out = fn()
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, int(L.gbs_kernel_launch_count() - l0), out
    for _ in range(steps):
        if prep:
            prep()
        if flush:
            flush()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = L.gbs_kernel_launch_count()
        e0.record(s)
        out = fn()
        e1.record(s)
        torch.cuda.synchronize()
        launches += int(L.gbs_kernel_launch_count() - l0)
        total += e0.elapsed_time(e1) / 1e3
    return total, launches, out


def phase_roofline(name, ph, step_s, note_latency=True):
    """Roofline entry of one profiled phase against the peak of its unit."""
    t = ph["ms"] / 1e3
    if name == "tc_gemm":
        e = {"bound": "tensor", "kernel": "tc_gemm_kernel (tcgen05 kind::tf32)",
             "achieved": ph["flops"] / t / 1e12 if t else 0.0, "peak": tf32_peak(), "unit": "TFLOP/s",
             "peak_source": "of measured: cuBLAS TF32 GEMM 8192^3 timed in this run",
             "note": "algorithmic flops 2 M N K; a 3xTF32 update issues three such products"}
    elif name == "residual":
        e = {"bound": "hbm", "kernel": "oz_product_kernel (FP64-accurate r = b - A x on bf16 tcgen05, Ozaki "
                                       "slices) + the slicing of A",
             "achieved": ph["bytes"] / t / 1e9 if t else 0.0, "peak": measured_hbm_gbs(), "unit": "GB/s",
             "peak_source": "of measured: MEASURED_PEAKS.json hbm_gbs"}
    elif name in ("gemm", "syrk", "batched"):
        e = {"bound": "fp64", "kernel": {"gemm": "gemm_sub_kernel<double> (trailing update)",
                                         "syrk": "gemm_sub_kernel<double> lower (SYRK)",
                                         "batched": "batched LLT / LU kernels"}[name],
             "achieved": ph["flops"] / t / 1e12 if t else 0.0, "peak": fp64_peak(), "unit": "TFLOP/s",
             "peak_source": "of measured: cuBLAS DGEMM 8192^3 timed in this run (FP64 has no entry in "
                            "MEASURED_PEAKS.json)"}
    else:
        e = {"bound": "hbm", "kernel": name, "achieved": ph["bytes"] / t / 1e9 if t else 0.0,
             "peak": measured_hbm_gbs(), "unit": "GB/s", "peak_source": "of measured: MEASURED_PEAKS.json hbm_gbs"}
        if note_latency:
            e["note"] = ("latency-bound (barrier or dependency chain per column / block): the fraction shows the "
                         "distance from the memory roof")
    e["frac"] = e["achieved"] / e["peak"] if e["peak"] else None
    ratio = TRAFFIC_OVER_ALGORITHMIC.get(name)
    e["traffic"] = (ratio * ph["bytes"] / max(ph["launches"], 1)) if ratio else None
    e.update({"phase": name, "share_of_step": ph["ms"] / (1e3 * step_s) if step_s else None,
              "launches_per_step": ph["launches"],
              "algorithmic_bytes_per_launch": ph["bytes"] / max(ph["launches"], 1),
              "algorithmic_flops_per_launch": ph["flops"] / max(ph["launches"], 1)})
    return e


def compact(e):
    keep = ("bound", "kernel", "phase", "achieved", "peak", "unit", "frac", "share_of_step", "launches_per_step")
    return {k: (round(v, 4) if isinstance(v, float) else v) for k, v in e.items() if k in keep}


# ----------------------------------------------------------------- CPU oracle
def cpu_oracle_solve(a_np, b_np):
    import oracle as O
    t0 = time.perf_counter()
    f, tr, _, _ = O.lu(a_np)
    x = O.lu_solve(f, tr, b_np)
    return x, time.perf_counter() - t0


def headline_inputs(n, nrhs):
    import oracle as O
    return O.gauss(1, n, n), O.gauss(2, n, nrhs)


# ----------------------------------------------------------------- reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle as O
    n, nrhs = args.n, args.nrhs
    a, b = headline_inputs(n, nrhs)
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
            "data": HEADLINE_DATA, "config": headline_config(n, nrhs),
            "tflops": lu_flops(n, nrhs) * v / 1e12,
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
                             "sample": f"full PartialPivLU n={n} factor + {nrhs}-RHS solve per step (the reference "
                                       "algorithm restated in C: same blocking, OpenMP GEMM)"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- headline arm
def run_ours(args):
    import numpy as np
    import torch

    import eigen_gb300 as gb
    import oracle as O
    from eigen_gb300 import _lib
    from eigen_gb300.mixed import RefineInfo, options
    world, rank, local = dist_setup(args)
    L = gb.lib()
    n, nrhs = args.n, args.nrhs
    stream = torch.cuda.current_stream()
    a_host, b_host = headline_inputs(n, nrhs)
    # column-major device copies (a row-major tensor of A^T is column-major A)
    A = torch.from_numpy(np.ascontiguousarray(a_host.T)).cuda().t()
    B = torch.from_numpy(np.ascontiguousarray(b_host.T)).cuda().t()
    X = torch.empty(nrhs, n, dtype=torch.float64, device="cuda").t()
    opt = options(args.path, tol=BE_BAR, lookahead=bool(args.lookahead))
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

    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    dt, launches, _ = device_time(step, args.steps, args.warmup)
    clk = clocks.stop()
    dt_max = max_over_ranks(world, dt)
    be = backward_error_gpu(A, X, B)
    X_main = X.clone()
    value = world * args.steps / dt_max if be <= BE_BAR else 0.0
    refine = info.as_dict()
    # phases: a second pass of the same steps with per-launch CUDA events on
    prof = profiled(L, step, reps=args.steps)
    prof_step_s = sum(v["ms"] for v in prof.values()) / 1e3

    plain = None
    fwd = None
    if args.path != "fp64" and args.plain_steps > 0:
        pdt, _, _ = device_time(step_plain, args.plain_steps, 1)
        pbe = backward_error_gpu(A, X, B)
        fwd = forward_error_gpu(X_main, X)
        pdt = max_over_ranks(world, pdt)
        plain = {"value": world * args.plain_steps / pdt, "unit": "solves/s",
                 "ms_per_step": 1e3 * pdt / args.plain_steps, "backward_error": pbe,
                 "tflops": lu_flops(n, nrhs) * world * args.plain_steps / pdt / 1e12,
                 "api": "gbs_lu_compute_device + gbs_lu_solve_device (pivots identical to the reference)"}

    order = sorted(prof.items(), key=lambda kv: -kv[1]["ms"])
    roofline = phase_roofline(*order[0], prof_step_s) if order else {}
    roofline["other_phases"] = [compact(phase_roofline(k, v, prof_step_s)) for k, v in order[1:]]
    roofline["profiled_pass"] = ("phases from a second pass of the same steps with per-launch CUDA events; "
                                 "value is timed without them")

    e2e = None
    if not args.no_e2e:
        Ah = torch.from_numpy(np.ascontiguousarray(a_host.T)).pin_memory()   # row-major A^T == column-major A
        Bh = torch.from_numpy(np.ascontiguousarray(b_host.T)).pin_memory()
        Xh = torch.empty((nrhs, n), dtype=torch.float64).pin_memory()
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

        # the host link's rate for this buffer: one plain copy of A (not part of the measurement)
        Ad = torch.empty_like(Ah, device="cuda")
        h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        Ad.copy_(Ah, non_blocking=True)
        h0.record(stream)
        Ad.copy_(Ah, non_blocking=True)
        h1.record(stream)
        torch.cuda.synchronize()
        h2d_gbs = Ah.numel() * 8 / (h0.elapsed_time(h1) * 1e-3) / 1e9
        del Ad
        for _ in range(max(1, args.warmup)):
            e2e_step()
        torch.cuda.synchronize()
        barrier(world)
        per_step = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ts = time.perf_counter()
            e2e_step()
            per_step.append(time.perf_counter() - ts)
        torch.cuda.synchronize()
        t_e2e = max_over_ranks(world, time.perf_counter() - t0)
        be2 = backward_error_gpu(A, Xh.to("cuda").t(), B)
        e2e = {"value": (world * args.steps / t_e2e) if be2 <= BE_BAR else 0.0, "unit": "solves/s",
               "h2d_bytes_per_step": 8 * (n * n + n * nrhs), "d2h_bytes_per_step": 8 * n * nrhs,
               "ms_per_step_median": 1e3 * statistics.median(per_step), "h2d_gbs_of_A": h2d_gbs,
               "backward_error": be2,
               "api": ("gbs_dgesv_mixed" if args.path != "fp64" else "gbs_lu_compute + gbs_lu_solve") +
                      " on pinned host buffers"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        x, dt_cpu = cpu_oracle_solve(a_host, b_host)
        cpu = {"value": 1.0 / dt_cpu, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
               "sample": f"one full PartialPivLU n={n} FP64 factor + {nrhs}-RHS solve of the same bytes (oracle/ C "
                         f"restatement of the reference algorithm, OpenMP GEMM), {dt_cpu:.2f} s, backward error "
                         f"{O.backward_error(a_host, x[:, :1], b_host[:, :1]):.1e}",
               "seconds": dt_cpu}

    companions = {}
    if world == 1 and args.companions != "none":
        del A, B, X, X_main
        torch.cuda.empty_cache()
        for name in [c for c in args.companions.split(",") if c]:
            t0 = time.perf_counter()
            try:
                companions[name] = COMPANION_FNS[name](args)
            except Exception as ex:           # a companion's failure must not void the headline line
                companions[name] = {"error": f"{type(ex).__name__}: {ex}"[:300]}
            companions[name]["wall_s"] = round(time.perf_counter() - t0, 1)
            torch.cuda.empty_cache()

    if plain is not None:
        roofline["vs_plain_fp64"] = {"plain_fp64_solves_per_s": plain["value"],
                                     "speedup": value / plain["value"] if plain["value"] else None,
                                     "plain_backward_error": plain["backward_error"],
                                     "forward_error_vs_fp64": fwd}
    if companions:
        roofline["companion_workloads"] = {k: summarize_companion(v) for k, v in companions.items()}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * dt_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": HEADLINE_DATA,
                "config": headline_config(n, nrhs),
                "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "e2e": e2e,
                "path": args.path, "parallelism": f"replicas x{world}",
                "tflops": lu_flops(n, nrhs) * value / 1e12, "backward_error": be, "forward_error_vs_fp64": fwd,
                "refinement": refine, "plain_fp64": plain,
                "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
                "phases_ms_per_step": {k: round(v["ms"], 3) for k, v in prof.items()}}
        if args.detail:
            with open(args.detail, "w") as f:
                json.dump(dict(line, companions=companions), f, indent=1)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def summarize_companion(c):
    """The figures of a companion workload that the record keeps (nested in roofline)."""
    if "error" in c:
        return {"error": c["error"]}
    keep = ("workload", "value", "unit", "steps", "warmup", "ms_per_step", "backward_error", "gpu_launches",
            "speedup", "summary")
    out = {k: c[k] for k in keep if k in c}
    if c.get("e2e"):
        out["e2e"] = c["e2e"].get("value")
    if c.get("cpu_baseline"):
        cb = c["cpu_baseline"]
        out["cpu_baseline"] = {"value": cb.get("value"), "cores": cb.get("cores"), "kind": cb.get("kind")}
    if c.get("roofline"):
        out["roofline"] = compact(c["roofline"])
    return out


# ----------------------------------------------------------------- companions
def c1_llt512(args):
    """LLT<MatrixXd> n = 512: A = G G^T / 512 + I (G iid N(0,1)), one RHS,
    plain FP64 through the LLT object on device buffers (and end to end from
    host buffers), parity against the oracle on the same input, the oracle
    port timed beside it on the host cores."""
    import numpy as np
    import torch

    import oracle as O
    import eigen_gb300 as gb
    n = 512
    steps, warmup = max(args.steps, 20), max(args.warmup, 3)
    G = O.gauss(42, n, n)
    a = np.asfortranarray(G @ G.T / n + np.eye(n))
    b = O.gauss(43, n, 1)
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    Bd = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    llt = gb.LLT(dtype=np.float64)
    L = gb.lib()
    L.gbs_llt_set_stream(llt._h, C.c_void_p(torch.cuda.current_stream().cuda_stream))

    def step():
        llt.compute(A)
        return llt.solve(Bd)
    dt, launches, X = device_time(step, steps, warmup, flush=L2Flush())
    dt /= steps
    prof = profiled(L, step, reps=steps)
    x = X.cpu().numpy()
    f_o, _ = O.llt(a)
    x_o = O.llt_solve(f_o, b)
    fwd = float(np.linalg.norm(x - x_o) / np.linalg.norm(x_o))
    be = O.backward_error(a, x, b)
    llt_h = gb.LLT(dtype=np.float64)
    for _ in range(warmup):
        llt_h.compute(a)
        llt_h.solve(b)
    t0 = time.perf_counter()
    for _ in range(steps):
        llt_h.compute(a)
        llt_h.solve(b)
    e2e = steps / (time.perf_counter() - t0)
    t0 = time.perf_counter()
    reps = 40
    for _ in range(reps):
        f_c, _ = O.llt(a)
        O.llt_solve(f_c, b)
    cpu = reps / (time.perf_counter() - t0)
    flops = n ** 3 / 3 + 2 * n * n
    top = max(prof.items(), key=lambda kv: kv[1]["ms"])
    roof = {"bound": "latency", "kernel": top[0], "phase": top[0],
            "achieved": flops / dt / 1e12, "peak": fp64_peak(), "unit": "TFLOP/s",
            "frac": flops / dt / 1e12 / fp64_peak(), "share_of_step": top[1]["ms"] / 1e3 / dt,
            "note": "n = 512: 4.5e7 flop per solve in a chain of dependent FP64 steps; the fraction is of the "
                    "measured DGEMM rate"}
    return {"workload": "LLT<MatrixXd> n=512 + solve 1 RHS, plain FP64, A = G G^T/512 + I", "value": 1.0 / dt,
            "unit": "solves/s", "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * dt,
            "l2": "inputs 2 MB: L2 flushed (256 MB written) between timed steps",
            "tflops": flops / dt / 1e12, "backward_error": be, "forward_diff_vs_oracle": fwd,
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": 8 * (n * n + n),
                    "d2h_bytes_per_step": 8 * n, "api": "gbs_llt_compute / gbs_llt_solve on host buffers"},
            "cpu_baseline": {"value": cpu, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
                             "sample": f"{reps} factor + solve of the same system (LLT is unblocked per column "
                                       "and single-threaded in the reference)"},
            "gpu_launches": launches // steps, "roofline": roof,
            "phases_ms_per_step": {k: round(v["ms"], 4) for k, v in prof.items()}}


def c3_llt16384(args):
    """LLT n = 16384, A = Q diag(sigma) Q^T (Haar Q, sigma log-spaced 1..kappa),
    4 right-hand sides, kappa in {1e2, 1e6, 1e10}: each tier's solves/s at
    backward error <= 1e-13, its forward error against the FP64 solution and
    its speed-up over plain FP64."""
    import numpy as np
    import torch

    import oracle as O
    import eigen_gb300 as gb
    from eigen_gb300.mixed import RefineInfo, options
    from eigen_gb300 import _lib
    n = 16384 if args.config == "lu8192" or args.n == 8192 else args.n
    nrhs = 4
    L = gb.lib()
    g = torch.Generator(device="cuda").manual_seed(7)
    Gm = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    Q, Rq = torch.linalg.qr(Gm)
    Q = Q * torch.sign(torch.diagonal(Rq))
    del Gm, Rq
    B = torch.randn(nrhs, n, dtype=torch.float64, device="cuda", generator=g).t()
    flops = n ** 3 / 3.0 + 2.0 * n * n * nrhs
    per_kappa = {}
    head = None
    for kappa in (1e2, 1e6, 1e10):
        s = torch.logspace(0, float(np.log10(kappa)), n, dtype=torch.float64, device="cuda")
        A = (Q * s) @ Q.t()
        A = ((A + A.t()) / 2).contiguous().t()
        rows = {}
        x64 = None
        for tier in ("fp64", "tf32x3", "fp16", "bf16"):
            fast = tier == "tf32x3"
            st, wu = (3, 1) if fast else (1, 1)
            dt, launches, (X, info) = device_time(lambda: gb.solve_spd_mixed(A, B, tier=tier), st, wu)
            dt /= st
            if tier == "fp64":
                x64 = X.clone()
            prof = profiled(L, lambda: gb.solve_spd_mixed(A, B, tier=tier))
            be = backward_error_gpu(A, X, B)
            rows[tier] = {"solves_per_s": 1.0 / dt if be <= BE_BAR else 0.0, "ms": round(1e3 * dt, 2),
                          "tflops": round(flops / dt / 1e12, 3), "backward_error": be,
                          "forward_error_vs_fp64": forward_error_gpu(X, x64), "steps": st, "warmup": wu,
                          "tier_used": info["tier_used"], "iterations": info["iterations"],
                          "inner_iterations": info["inner_iterations"], "fell_back": bool(info["fell_back"]),
                          "gpu_launches": launches // st,
                          "phases_ms": {k: round(v["ms"], 3) for k, v in prof.items()}}
        fastest = max(rows, key=lambda t: rows[t]["solves_per_s"])
        per_kappa[f"{kappa:.0e}"] = {"tiers": rows, "fastest": fastest,
                                     "speedup_vs_fp64": rows[fastest]["solves_per_s"] / rows["fp64"]["solves_per_s"]}
        if kappa == 1e2:
            head = (fastest, rows[fastest], A.clone() if not args.no_e2e else None)
        del A
        torch.cuda.empty_cache()
    fastest, best, A1 = head
    top = max(best["phases_ms"].items(), key=lambda kv: kv[1]) if best["phases_ms"] else ("", 0.0)
    # the dominant phase of the fastest tier at kappa = 1e2, from its profiled pass
    roof = {"bound": "tensor" if top[0] in ("tc_gemm", "syrk") else "latency", "kernel": top[0], "phase": top[0],
            "achieved": flops / (best["ms"] / 1e3) / 1e12, "peak": tf32_peak(), "unit": "TFLOP/s",
            "frac": flops / (best["ms"] / 1e3) / 1e12 / tf32_peak(),
            "share_of_step": top[1] / best["ms"] if best["ms"] else None,
            "note": "whole solve at kappa=1e2 (algorithmic n^3/3 + 2 n^2 nrhs) over the measured TF32 rate"}
    e2e = None
    if A1 is not None:
        Ah = A1.t().contiguous().cpu().pin_memory()     # row-major A^T == column-major A (symmetric anyway)
        Bh = B.t().contiguous().cpu().pin_memory()
        Xh = torch.empty((nrhs, n), dtype=torch.float64).pin_memory()
        opt = options(fastest, tol=BE_BAR)
        einfo = RefineInfo()

        def e2e_step():
            _lib.check(L.gbs_dposv_mixed(n, nrhs, C.c_void_p(Ah.data_ptr()), n, C.c_void_p(Bh.data_ptr()), n,
                                         C.c_void_p(Xh.data_ptr()), n, C.byref(opt), C.byref(einfo)),
                       "gbs_dposv_mixed")
        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        # the SPD solve copies the lower trapezoid of each 512-column block (it reads A's lower triangle only)
        lower = sum((n - c0) * min(512, n - c0) for c0 in range(0, n, 512))
        e2e = {"value": 2 / (time.perf_counter() - t0), "unit": "solves/s", "h2d_bytes_per_step": 8 * (lower + n * nrhs),
               "d2h_bytes_per_step": 8 * n * nrhs, "api": f"gbs_dposv_mixed ({fastest}) on pinned host buffers, kappa=1e2"}
        del A1, Ah
    # CPU: the oracle's LLT (single-threaded, like the reference's LLT) on a
    # bounded sample: an n/4 system of the same family, scaled by the n^3 work
    m = n // 4
    Gs = O.gauss(17, m, m)
    qs, _ = np.linalg.qr(Gs)
    a_s = np.asfortranarray((qs * np.logspace(0, 2, m)) @ qs.T)
    b_s = O.gauss(18, m, nrhs)
    t0 = time.perf_counter()
    f_s, _ = O.llt(a_s)
    O.llt_solve(f_s, b_s)
    t_s = time.perf_counter() - t0
    cpu_value = 1.0 / (t_s * (n / m) ** 3)
    summary = {k: {"fastest": v["fastest"], "speedup_vs_fp64": round(v["speedup_vs_fp64"], 2),
                   **{t: {"solves_per_s": round(r["solves_per_s"], 3), "backward_error": r["backward_error"],
                          "forward_error_vs_fp64": r["forward_error_vs_fp64"], "fell_back": r["fell_back"]}
                      for t, r in v["tiers"].items()}} for k, v in per_kappa.items()}
    return {"workload": f"LLT<MatrixXd> n={n}, {nrhs} RHS, A = Q diag(sigma) Q^T, kappa in 1e2/1e6/1e10 "
                        "(value: kappa=1e2, fastest tier)",
            "value": best["solves_per_s"], "unit": "solves/s", "steps": best["steps"], "warmup": best["warmup"],
            "ms_per_step": best["ms"], "backward_error": best["backward_error"], "gpu_launches": best["gpu_launches"],
            "l2": "inputs (2 GB) larger than L2; no flush",
            "speedup": {k: round(v["speedup_vs_fp64"], 2) for k, v in per_kappa.items()},
            "summary": summary, "per_kappa": per_kappa, "e2e": e2e, "roofline": roof,
            "cpu_baseline": {"value": cpu_value, "unit": "solves/s", "cores": 1, "kind": "port",
                             "sample": f"oracle LLT + {nrhs}-RHS solve of one n={m} system of the same family "
                                       f"({t_s:.2f} s), scaled by (n/{m})^3; the reference's LLT is single-threaded"}}


def c4_batched(args):
    """100,000 SPD systems n ~ U{3..24} (G G^T + 0.1 I) and 20,000 general n ~
    U{4..64} (iid N(0,1)), one RHS each, FP64 and FP32: one graph launch per
    batch, autotuned; end to end from pinned host buffers; the CPU oracle
    (one object per matrix, all host cores) beside it."""
    import numpy as np
    import torch

    import oracle as O
    from eigen_gb300.batched import BatchedSolver
    steps, warmup = max(args.steps, 5), max(args.warmup, 3)
    rng = np.random.default_rng(0)
    sizes = np.concatenate([rng.integers(3, 25, 100000), rng.integers(4, 65, 20000)]).astype(np.int32)
    kinds = np.concatenate([np.zeros(100000), np.ones(20000)]).astype(np.int32)
    flops = float(np.sum(np.where(kinds == 0, sizes ** 3 / 3 + 2 * sizes ** 2, 2 * sizes ** 3 / 3 + 2 * sizes ** 2)))
    flush = L2Flush()
    out = {}
    ah64 = None
    for dtype, tdt, name in ((np.float64, torch.float64, "f64"), (np.float32, torch.float32, "f32")):
        bs = BatchedSolver(sizes, kinds, dtype=dtype)
        if ah64 is None:
            ah64 = np.empty(bs.a_elems, dtype=np.float64)
            for i, nn in enumerate(sizes):
                m = rng.standard_normal((nn, nn))
                if kinds[i] == 0:
                    m = m @ m.T + 0.1 * np.eye(nn)
                ah64[bs.a_off[i]:bs.a_off[i] + nn * nn] = m.reshape(-1, order="F")
            bh64 = rng.standard_normal(bs.b_elems)
        A0 = torch.from_numpy(ah64).to(tdt).cuda()
        B0 = torch.from_numpy(bh64).to(tdt).cuda()
        A, B = A0.clone(), B0.clone()
        info = torch.empty(len(sizes), dtype=torch.int32, device="cuda")
        piv = torch.empty(bs.b_elems, dtype=torch.int32, device="cuda")

        def prep():
            A.copy_(A0)
            B.copy_(B0)
        dflt, _, _ = device_time(lambda: bs.solve(A, B, info, piv), 3, warmup, flush=flush, prep=prep)
        cfg = bs.autotune(A.clone(), B.clone(), info, piv)
        dt, launches, _ = device_time(lambda: bs.solve(A, B, info, piv), steps, warmup, flush=flush, prep=prep)
        dt /= steps
        prep()
        prof = profiled(gb_lib(), lambda: bs.solve(A, B, info, piv))
        failures = int((info >= 0).sum().item())
        # end to end: pinned host buffers in, solutions and info out, every step
        Ah = torch.from_numpy(ah64.astype(dtype)).pin_memory()
        Bh = torch.from_numpy(bh64.astype(dtype)).pin_memory()
        Xh = torch.empty_like(Bh).pin_memory()
        Ih = torch.empty(len(sizes), dtype=torch.int32).pin_memory()

        def e2e_step():
            # the library's host-buffer solve: parts of the batch cross in and out while others are solved
            bs.solve_host(Ah, Bh, Ih, x=Xh)
        for _ in range(warmup):
            e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e = steps * len(sizes) / (time.perf_counter() - t0)
        # CPU oracle: the whole batch, one object per matrix, all host cores
        a_np = ah64.astype(dtype)
        b_np = bh64.astype(dtype)
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
        byts = float(np.sum(2 * sizes.astype(np.float64) ** 2 + 3 * sizes)) * np.dtype(dtype).itemsize
        out[name] = {"solves_per_s": len(sizes) / dt, "ms": 1e3 * dt, "tflops": flops / dt / 1e12,
                     "hbm_gbs": byts / dt / 1e9, "algorithmic_bytes": byts, "failures": failures,
                     "autotuned": cfg, "default_variants_ms": 1e3 * dflt / 3, "gpu_launches": launches // steps,
                     "e2e_solves_per_s": e2e, "h2d_bytes_per_step": int(Ah.numel() * Ah.element_size() +
                                                                           Bh.numel() * Bh.element_size()),
                     "d2h_bytes_per_step": int(Xh.numel() * Xh.element_size() + 4 * len(sizes)),
                     "cpu_oracle_solves_per_s": cpu, "cpu_cores": O.num_threads(),
                     "phases_ms": {k: round(v["ms"], 3) for k, v in prof.items()}}
        del A0, B0, A, B, Ah, Bh
        torch.cuda.empty_cache()
    f64 = out["f64"]
    fr_fp64 = f64["tflops"] / fp64_peak()
    fr_hbm = f64["hbm_gbs"] / measured_hbm_gbs()
    roof = {"bound": "fp64" if fr_fp64 >= fr_hbm else "hbm", "kernel": "batched LLT / LU kernels (one graph)",
            "phase": "batched",
            "achieved": f64["tflops"] if fr_fp64 >= fr_hbm else f64["hbm_gbs"],
            "peak": fp64_peak() if fr_fp64 >= fr_hbm else measured_hbm_gbs(),
            "unit": "TFLOP/s" if fr_fp64 >= fr_hbm else "GB/s", "frac": max(fr_fp64, fr_hbm),
            "fp64_frac": fr_fp64, "hbm_frac": fr_hbm,
            "note": "algorithmic flops per item n^3/3 + 2n^2 (LLT), 2n^3/3 + 2n^2 (LU); bytes per item "
                    "8 (2 n^2 + 3 n); peaks: measured DGEMM in this run, MEASURED_PEAKS.json hbm_gbs"}
    return {"workload": "batched: 100,000 LLT (n 3..24) + 20,000 PartialPivLU (n 4..64), 1 RHS each, FP64 "
                        "(FP32 beside), one CUDA-graph launch per batch",
            "value": f64["solves_per_s"], "unit": "solves/s", "steps": steps, "warmup": warmup,
            "ms_per_step": f64["ms"], "gpu_launches": f64["gpu_launches"],
            "l2": "inputs restored then L2 flushed (256 MB written) before each timed step",
            "summary": {"f32_solves_per_s": out["f32"]["solves_per_s"], "failures_f64": f64["failures"]},
            "e2e": {"value": f64["e2e_solves_per_s"], "unit": "solves/s",
                    "h2d_bytes_per_step": f64["h2d_bytes_per_step"], "d2h_bytes_per_step": f64["d2h_bytes_per_step"],
                    "api": "gbs_batched_solve_host on pinned host buffers (the batch in four parts: each part's "
                           "copies overlap the other parts' solves), every step"},
            "cpu_baseline": {"value": f64["cpu_oracle_solves_per_s"], "unit": "solves/s", "cores": f64["cpu_cores"],
                             "kind": "port", "sample": "the whole FP64 batch, one oracle factor + solve per item, "
                                                       "OpenMP over items"},
            "roofline": roof, "batched": out}


def gb_lib():
    import eigen_gb300 as gb
    return gb.lib()


def c5_router(args):
    """20,000 general systems n ~ U{32..512}, A = U diag(s) V^T (Haar U, V),
    log10 kappa ~ U[1, 12]: the network (shipped weights, or trained here with
    --train) routes each system to a tier; against always-FP64 (the batched
    FP64 kernel) and try-lowest-then-fallback, all at backward error <= 1e-13."""
    import numpy as np
    import torch

    import oracle as O
    from eigen_gb300 import router as R
    steps, warmup = max(3, min(args.steps, 3)), max(args.warmup, 1)
    training = None
    if args.train:
        r, training = train_router(args)
    else:
        r = R.Router.pretrained()
    mt, At, Bt, logk = R.generate(20000, seed=7, nmin=32, nmax=512)
    L = gb_lib()
    t64, l64, X64 = device_time(lambda: R.solve_fp64(mt, At, Bt), steps, warmup)
    t64 /= steps
    ttry, _, (Xtry, st_try) = device_time(lambda: R.solve_cascade(mt, At, Bt), steps, warmup)
    ttry /= steps
    tr_, lr_, (Xr, st_r) = device_time(lambda: R.route_and_solve(r, mt, At, Bt), steps, warmup)
    tr_ /= steps
    prof = profiled(L, lambda: R.route_and_solve(r, mt, At, Bt))
    t_feat, _, _ = device_time(lambda: R.features(mt, At), 3, 1)
    sample = np.random.default_rng(0).choice(mt.count, 500, replace=False)

    def worst(X):
        return float(max(float(((mt.vector(Bt, i) - mt.matrix(At, i) @ mt.vector(X, i)).abs().max() /
                                (mt.matrix(At, i).abs().sum(1).max() * mt.vector(X, i).abs().max() +
                                 mt.vector(Bt, i).abs().max())).item()) for i in sample))
    pred = r.predict(R.features(mt, At))
    ytest = R.labels(mt, At)
    # end to end: pinned host A and b in, x out, every step
    Ah = At.cpu().pin_memory()
    Bh = Bt.cpu().pin_memory()
    Xh = torch.empty_like(Bh).pin_memory()
    Ad, Bd = torch.empty_like(At), torch.empty_like(Bt)

    def e2e_step():
        Ad.copy_(Ah, non_blocking=True)
        Bd.copy_(Bh, non_blocking=True)
        X, _ = R.route_and_solve(r, mt, Ad, Bd)
        Xh.copy_(X, non_blocking=True)
    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e = steps * mt.count / (time.perf_counter() - t0)
    # CPU oracle: always-FP64 LU + solve, one object per system, all host cores,
    # on a bounded sample of 2,000 systems of the batch
    cs = np.random.default_rng(3).choice(mt.count, 2000, replace=False)
    ns = mt.sizes[cs].astype(np.int32)
    off = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    voff = np.concatenate([[0], np.cumsum(ns.astype(np.int64))[:-1]]).astype(np.int64)
    a_np = np.concatenate([mt.matrix(At, int(i)).t().contiguous().cpu().numpy().reshape(-1) for i in cs])
    b_np = np.concatenate([mt.vector(Bt, int(i)).cpu().numpy() for i in cs])
    t0 = time.perf_counter()
    O.port().oracle_batched_lu_solve_d(len(cs), ns, off, a_np.ctypes.data_as(C.c_void_p), voff,
                                       b_np.ctypes.data_as(C.c_void_p), np.zeros(int(ns.sum()), dtype=np.int32),
                                       np.zeros(len(cs), dtype=np.int32))
    cpu = len(cs) / (time.perf_counter() - t0)
    flops = float(np.sum(2 * mt.sizes.astype(np.float64) ** 3 / 3 + 2 * mt.sizes.astype(np.float64) ** 2))
    top = max(prof.items(), key=lambda kv: kv[1]["ms"])
    # the dominant kernels of the routed step are the batched LU kernels; their
    # FP64 rate is measured on the always-FP64 run over all 20,000 systems
    roof = {"bound": "fp64", "kernel": "mbatch_getrf64_kernel + solve (batched FP64 LU, always-FP64 run)",
            "phase": top[0], "achieved": flops / t64 / 1e12, "peak": fp64_peak(), "unit": "TFLOP/s",
            "frac": flops / t64 / 1e12 / fp64_peak(),
            "share_of_step": top[1]["ms"] / sum(v["ms"] for v in prof.values()),
            "note": "algorithmic 2n^3/3 + 2n^2 per system; the routed step spends share_of_step in these kernels "
                    "(FP64 and FP32 tiers)"}
    res = {"always_fp64": {"solves_per_s": mt.count / t64, "s": t64, "worst_backward_error_sample": worst(X64)},
           "try_lowest_then_fallback": {"solves_per_s": mt.count / ttry, "s": ttry, **st_try,
                                        "worst_backward_error_sample": worst(Xtry)},
           "router": {"solves_per_s": mt.count / tr_, "s": tr_, **st_r, "worst_backward_error_sample": worst(Xr)},
           "features_s": t_feat / 3,
           "network": {"weights": "trained in this run" if training else "shipped (eigen_gb300/router_weights.json)",
                       "test_median_abs_err_log10_kappa": float((pred - ytest).abs().median().item()),
                       "t_ir_log10_kappa": r.t_ir, "t_gmres_log10_kappa": r.t_gmres, **(training or {})},
           "phases_ms": {k: round(v["ms"], 3) for k, v in prof.items()}}
    be = max(res["router"]["worst_backward_error_sample"], 0.0)
    return {"workload": "router: 20,000 PartialPivLU systems n 32..512, log10 kappa U[1,12], 1 RHS; routed tiers",
            "value": res["router"]["solves_per_s"], "unit": "solves/s", "steps": steps, "warmup": warmup,
            "ms_per_step": 1e3 * tr_, "backward_error": be, "gpu_launches": lr_ // steps,
            "l2": "inputs (about 15 GB) larger than L2; no flush",
            "speedup": {"vs_always_fp64_batched": res["router"]["solves_per_s"] / res["always_fp64"]["solves_per_s"],
                        "vs_try_lowest_then_fallback":
                            res["router"]["solves_per_s"] / res["try_lowest_then_fallback"]["solves_per_s"]},
            "summary": {"always_fp64_solves_per_s": res["always_fp64"]["solves_per_s"],
                        "cascade_solves_per_s": res["try_lowest_then_fallback"]["solves_per_s"],
                        "routed": st_r, "cascade": st_try},
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(8 * (At.numel() + Bt.numel())),
                    "d2h_bytes_per_step": int(8 * Bt.numel()),
                    "api": "host->device copies + route_and_solve + device->host copy, every step"},
            "cpu_baseline": {"value": cpu, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
                             "sample": "always-FP64 oracle LU + solve of 2,000 systems drawn from the batch"},
            "roofline": roof, "tflops_routed": flops / tr_ / 1e12, "router": res}


def train_router(args):
    """Trains the network on method-generated rcond labels (the bench's
    --train path; the shipped weights came from this with 1M labels)."""
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
    return r, {"train_systems": int(ntrain), "generate_s": t_gen, "labels_s": t_lab, "features_s": t_feat,
               "fit_s": t_fit, "final_train_mse_scaled": loss}


COMPANION_FNS = {"llt512": c1_llt512, "llt16384": c3_llt16384, "batched": c4_batched, "router": c5_router}


def run_single(args):
    """One companion workload as a line of its own (--config llt512 | llt16384 | batched | router)."""
    dist_setup(args)
    c = COMPANION_FNS[args.config](args)
    line = {"metric": METRIC, "value": c["value"], "unit": c["unit"], "n_gpus": 1, "steps": c["steps"],
            "warmup": c["warmup"], "ms_per_step": c["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic, seeded",
            "config": {"workload": c["workload"], "l2": c.get("l2")}, "gpu_launches": c.get("gpu_launches"),
            "roofline": c.get("roofline"), "cpu_baseline": c.get("cpu_baseline"), "e2e": c.get("e2e"),
            "detail": c}
    print(json.dumps(line), flush=True)
    return 0


def factor_once(args):
    import numpy as np
    import torch

    import eigen_gb300 as gb
    n = args.n
    a = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(3)).t()
    b = torch.randn(args.nrhs, n, dtype=torch.float64, device="cuda",
                    generator=torch.Generator("cuda").manual_seed(4)).t()
    torch.cuda.synchronize()
    if args.path == "fp64":
        lu = gb.PartialPivLU(a)
        torch.cuda.synchronize()
        ok = lu.first_zero_pivot() < 0
        out = {"first_zero_pivot": lu.first_zero_pivot()}
    else:
        x, info = gb.solve_mixed(a, b, tier=args.path, lookahead=bool(args.lookahead))
        torch.cuda.synchronize()
        ok = info["backward_error"] <= BE_BAR
        out = info
    print(json.dumps({"factor_once": n, "path": args.path, **out}))
    return 0 if ok else 1


def run_mbatch(args):
    """The router workload's medium batch (n ~ U{32..512}, log10 kappa ~
    U[1, 12]) through each tier once: FP64 LU + solve, FP32 LU + FP64
    refinement (small counts keep an ncu capture short)."""
    from eigen_gb300 import router as R
    mt, At, Bt, _ = R.generate(args.count, seed=7, nmin=32, nmax=512)
    _, t64 = R.timed(lambda: R.solve_fp64(mt, At, Bt))
    (_, st), t32 = R.timed(lambda: R.solve_fp32_ir(mt, At, Bt))
    conv = int((st >= 0).sum().item())
    print(json.dumps({"config": "mbatch", "count": args.count, "fp64_s": t64, "fp32_ir_s": t32,
                      "fp32_converged": conv}), flush=True)
    return 0


PHASE_NAMES = ("panel", "laswp", "trsm_lu", "gemm", "potrf_diag", "trsm_llt", "syrk", "tri_solve", "norm", "mixed",
               "tc_gemm", "residual", "batched", "router", "copy")


def timeline(args):
    """One device-buffer and one host-buffer solve of the headline workload
    (after warm-up), each with the library's per-launch CUDA events on: every
    launch's phase, stream (0, 1, ... in order of first use) and start / end
    time goes to the CSV file, and a summary per stream (launches, busy time,
    span) and of the panel chain's block period is printed.  The events sit
    between the kernels, so programmatic dependent launch is off in this run
    and its times are not the bench's."""
    import ctypes as C
    import numpy as np
    import torch

    import eigen_gb300 as gb
    from eigen_gb300 import _lib
    from eigen_gb300.mixed import RefineInfo, options
    L = gb.lib()
    n, nrhs = args.n, args.nrhs
    a_host, b_host = headline_inputs(n, nrhs)
    A = torch.from_numpy(np.ascontiguousarray(a_host.T)).cuda().t()
    B = torch.from_numpy(np.ascontiguousarray(b_host.T)).cuda().t()
    X = torch.empty(nrhs, n, dtype=torch.float64, device="cuda").t()
    Ah = torch.from_numpy(np.ascontiguousarray(a_host.T)).pin_memory()
    Bh = torch.from_numpy(np.ascontiguousarray(b_host.T)).pin_memory()
    Xh = torch.empty((nrhs, n), dtype=torch.float64).pin_memory()
    opt = options(args.path, tol=BE_BAR, lookahead=bool(args.lookahead))
    info = RefineInfo()
    s = torch.cuda.current_stream()

    def dev():
        _lib.check(L.gbs_dgesv_mixed_device(n, nrhs, C.c_void_p(A.data_ptr()), n, C.c_void_p(B.data_ptr()), n,
                                            C.c_void_p(X.data_ptr()), n, C.byref(opt), C.byref(info),
                                            C.c_void_p(s.cuda_stream)), "gbs_dgesv_mixed_device")

    def host():
        _lib.check(L.gbs_dgesv_mixed(n, nrhs, C.c_void_p(Ah.data_ptr()), n, C.c_void_p(Bh.data_ptr()), n,
                                     C.c_void_p(Xh.data_ptr()), n, C.byref(opt), C.byref(info)), "gbs_dgesv_mixed")

    cap = 1 << 16
    with open(args.timeline, "w") as f:
        f.write("api,phase,stream,start_ms,end_ms\n")
        for name, fn in (("device", dev), ("host", host)):
            for _ in range(max(1, args.warmup)):
                fn()
            torch.cuda.synchronize()
            L.gbs_profile_reset()
            L.gbs_profile_enable(1)
            fn()
            torch.cuda.synchronize()
            ph, st = (C.c_int * cap)(), (C.c_int * cap)()
            t0, t1 = (C.c_double * cap)(), (C.c_double * cap)()
            m = L.gbs_profile_timeline(ph, st, t0, t1, cap)
            L.gbs_profile_enable(0)
            if m < 0:
                raise RuntimeError(f"gbs_profile_timeline failed ({m})")
            m = min(m, cap)
            rec = [(ph[i], st[i], t0[i], t1[i]) for i in range(m)]
            for p_, s_, a_, b_ in rec:
                f.write(f"{name},{PHASE_NAMES[p_] if 0 <= p_ < len(PHASE_NAMES) else p_},{s_},{a_:.4f},{b_:.4f}\n")
            first = min(r[2] for r in rec)
            summary = {"api": name, "launches": m, "span_ms": round(max(r[3] for r in rec) - first, 3), "streams": {}}
            for sid in sorted({r[1] for r in rec}):
                rs = [r for r in rec if r[1] == sid]
                summary["streams"][sid] = {"launches": len(rs), "busy_ms": round(sum(r[3] - r[2] for r in rs), 3),
                                           "first_ms": round(min(r[2] for r in rs) - first, 3),
                                           "last_ms": round(max(r[3] for r in rs) - first, 3)}
            panels = sorted(r[2] for r in rec if r[0] == 0)
            starts = panels[::4]                        # four 32-column panels per 128-column block
            if len(starts) > 8:
                summary["block_period_us"] = round(1e3 * (starts[-4] - starts[4]) / (len(starts) - 8), 1)
            print(json.dumps(summary), flush=True)
    return 0


def main():
    args = args_parse()
    if args.timeline:
        return timeline(args)
    if args.factor_once:
        return factor_once(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "mbatch":
        return run_mbatch(args)
    if args.config != "lu8192":
        return run_single(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
