#!/usr/bin/env python
"""Benchmark of the HSS ULV solve on one GB300 (or N independent replicas).

Workload (the precision configuration the solve-rate metric is quoted on):
a synthetic HSS matrix, n = 65536 as a perfect binary tree of depth 9 with
leafsize 128 and rank k = 32 (leaf D = randn/sqrt(128) + 4I, orthonormal U, V,
R, W, B = 0.5 randn/sqrt(32), seed 3), and r = 32 right-hand sides ~ N(0,1).

One step = one ``hssA \\ B``: ULV factorization + solve, in the mixed form
(FP32 factorization and solve, FP64 HSS-product residual and update, refined
to a relative residual of 1e-10).  The plain FP64 form of the same step is
timed on the same GPU for comparison.  ``value`` counts steps (solves with 32
right-hand sides each) per second over all ranks, with the generators and B
resident in HBM; ``e2e`` is the same step through the C ABI's host-buffer
entry point (``hss_ulvfactsolve_host``) from pinned memory, copies included.
L2 is flushed (a 512 MB write) before every timed step.

``--impl reference`` times the CPU restatement of the reference algorithm
(``oracle/``, NumPy + LAPACK, all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "HSS ULV solves/s + p50/p99 at 1e-10 resid (mixed+batched vs plain FP64 GPU)"
UNIT = "solves/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=65536)
    p.add_argument("--leafsize", type=int, default=128)
    p.add_argument("--rank", type=int, default=32)
    p.add_argument("--rhs", type=int, default=32)
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--seed", type=int, default=3)
    p.add_argument("--roofline-kernel", default="factor_leaf")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def config(args, n_gpus):
    return {
        "workload": (f"precision: synthetic HSS n={args.n}, perfect tree leafsize {args.leafsize}, "
                     f"k={args.rank}, r={args.rhs} RHS; step = ULV factor + solve (hssA\\B), "
                     f"FP32 ULV + FP64-residual refinement to {args.tol:g}"),
        "n": args.n, "leafsize": args.leafsize, "k": args.rank, "rhs": args.rhs, "tol": args.tol,
        "seed": args.seed, "l2": "flushed before every timed step (512 MB write)",
        "parallelism": "replicas" if n_gpus > 1 else "single",
    }


# ---------------------------------------------------------------------------
# CPU side: the oracle restatement (reference arm and cpu_baseline)
# ---------------------------------------------------------------------------


def cpu_solve_sample(args, calls):
    import numpy as np
    from oracle import hss_oracle as orc
    h = orc.synthetic_hss(args.n, args.leafsize, args.rank, np.random.default_rng(args.seed))
    b = np.random.default_rng(1).standard_normal((args.n, args.rhs))
    times = []
    for _ in range(calls):
        t0 = time.perf_counter()
        orc.ulvfactsolve(h, b)
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    for _ in range(args.warmup):
        cpu_solve_sample(args, 1)
    times = cpu_solve_sample(args, args.steps)
    ms = 1000.0 * statistics.mean(times)
    value = 1000.0 / ms
    cores = os.cpu_count()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(args, world),
        "p50_ms": 1000.0 * statistics.median(times),
        "p99_ms": 1000.0 * sorted(times)[min(len(times) - 1, int(math.ceil(0.99 * len(times))) - 1)],
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full hssA\\B calls (n={args.n}, r={args.rhs}) with the "
                                   "NumPy/LAPACK restatement of ulvfactsolve (Julia is not installed)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------


class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
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
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------


def factor_leaf_bytes(A, factor_itemsize):
    """Algorithmic bytes of one leaf-level ULV launch: read every leaf's D, U, V
    (FP64 generators) once and write its reduced blocks + tau vectors once."""
    tot_read = tot_write = 0

    def walk(x, root):
        nonlocal tot_read, tot_write
        if x.leafnode:
            m, n = x.D.shape
            ku, kv = (0, 0) if root else (x.U.shape[1], x.V.shape[1])
            tot_read += 8 * (m * n + m * ku + n * kv)
            k = min(ku, m)
            tot_write += factor_itemsize * (m * n + m * ku + n * kv + k + (m - k))
            return
        walk(x.A11, False)
        walk(x.A22, False)

    walk(A, True)
    return tot_read + tot_write


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    import __graft_entry__ as g

    torch.cuda.set_device(local_rank)
    pkg = g.load_package()
    from hssmatrices_gb300 import linalg as L
    dist = world > 1
    if dist:
        import torch.distributed as td

    def barrier():
        if dist:
            td.barrier()
        torch.cuda.synchronize()

    n, r = args.n, args.rhs
    A = pkg.synthetic_hss(n, args.leafsize, args.rank, np.random.default_rng(args.seed))
    dev = A.device()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(1)
    Bh = rng.standard_normal((n, r))
    # an n x r column-major matrix is an r x n row-major tensor
    dB = torch.from_numpy(np.ascontiguousarray(Bh.T)).cuda()
    dX = torch.zeros_like(dB)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    F32 = dev.ulvfactor("fp32", stream=stream)
    F64 = dev.ulvfactor("fp64", stream=stream)

    def step32():
        F32.refactor(stream=stream)
        return F32.solve_device(dB, n, r, dX, n, tol=args.tol, maxit=20, stream=stream)

    def step64(dX64):
        F64.refactor(stream=stream)
        return F64.solve_device(dB, n, r, dX64, n, tol=0.0, stream=stream)

    for _ in range(args.warmup):
        step32()
    barrier()
    # timed region: K mixed-precision steps
    clocks = Clocks(local_rank)
    clocks.start()
    L.trace_begin(args.roofline_kernel)
    launches0 = L.launch_counter()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    iters = []
    barrier()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        st = step32()
        ev[i][1].record(stream)
        iters.append(st.iterations)
    barrier()
    launches = L.launch_counter() - launches0
    clk = clocks.stop()
    k_ms, k_cnt = L.trace_end()
    times = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(times)
    # per kernel kind: device time per mixed step (CUDA events around each
    # launch of one kind at a time, a few extra steps per kind)
    breakdown = {}
    for kind in ("factor_leaf", "factor_merge", "solve_up", "solve_down", "mv_leaf", "mv_up", "mv_down",
                 "mv_final"):
        L.trace_begin(kind)
        for _ in range(3):
            step32()
        kms, _kn = L.trace_end()
        breakdown[kind] = kms / 3
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        td.all_reduce(t, op=td.ReduceOp.MAX)
        total_ms = float(t.item())
    ms = total_ms / args.steps
    value = world * 1000.0 / ms
    Xh = dX.cpu().numpy().T
    res32 = float(np.max(np.linalg.norm(Bh - pkg.matmul(A, Xh), axis=0) / np.linalg.norm(Bh, axis=0)))
    # plain FP64 form on the same GPU
    dX64 = torch.zeros_like(dB)
    for _ in range(max(1, args.warmup)):
        step64(dX64)
    ev64 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in range(args.steps)]
    barrier()
    for i in range(args.steps):
        flush.zero_()
        ev64[i][0].record(stream)
        step64(dX64)
        ev64[i][1].record(stream)
    barrier()
    t64 = [a.elapsed_time(b) for a, b in ev64]
    ms64 = sum(t64) / args.steps
    X64 = dX64.cpu().numpy().T
    res64 = float(np.max(np.linalg.norm(Bh - pkg.matmul(A, X64), axis=0) / np.linalg.norm(Bh, axis=0)))
    # end to end through the host-buffer C entry point, pinned memory
    import ctypes as C
    Bp = torch.from_numpy(np.asfortranarray(Bh).T.copy()).pin_memory()   # r x n rows = columns of B
    Xp = torch.zeros_like(Bp).pin_memory()
    stats = pkg._lib.SolveStats()
    lib = dev.lib

    def e2e_call():
        rc = lib.hss_ulvfactsolve_host(dev.handle, pkg._lib.HSS_PREC_FP32,
                                       C.cast(C.c_void_p(Bp.data_ptr()), pkg._lib.PD), n, r,
                                       C.cast(C.c_void_p(Xp.data_ptr()), pkg._lib.PD), n, args.tol, 20, C.byref(stats))
        pkg._lib.check(rc)

    for _ in range(args.warmup):
        e2e_call()
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_call()
        e2e_t.append(time.perf_counter() - t0)
    barrier()
    e2e_total = sum(e2e_t)
    if dist:
        t = torch.tensor([e2e_total], device="cuda")
        td.all_reduce(t, op=td.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = world * args.steps / e2e_total
    if rank != 0:
        return 0
    # roofline of the dominant kernel (per launch)
    per_launch_ms = k_ms / max(k_cnt, 1)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    alg_bytes = factor_leaf_bytes(A, 4) if args.roofline_kernel == "factor_leaf" else None
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9 if alg_bytes and per_launch_ms > 0 else None
    roof = {"kernel": args.roofline_kernel, "bound": "hbm", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "traffic": None,
            "peak_source": peak_src, "launch_ms": per_launch_ms, "launches": k_cnt,
            "algorithmic_bytes": alg_bytes}
    cpu = None
    if not args.no_cpu_baseline:
        ct = cpu_solve_sample(args, 2)
        cms = 1000.0 * min(ct)
        cpu = {"value": 1000.0 / cms, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"2 full hssA\\B calls (n={n}, r={r}), NumPy/LAPACK restatement, best of 2"}
    st_sorted = sorted(times)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32+fp64", "data": "synthetic", "config": config(args, world),
        "p50_ms": statistics.median(times),
        "p99_ms": st_sorted[min(len(st_sorted) - 1, int(math.ceil(0.99 * len(st_sorted))) - 1)],
        "rhs_per_s": value * r, "refine_iters": iters, "residual": res32,
        "fp64": {"solves_per_s": world * 1000.0 / ms64, "ms_per_step": ms64, "residual": res64,
                 "p50_ms": statistics.median(t64)},
        "speedup_vs_fp64": ms64 / ms,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n * r,
                "d2h_bytes_per_step": 8 * n * r, "ms_per_step": 1000.0 * e2e_total / args.steps},
        "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
        "breakdown_ms_per_step": breakdown,
        "factor_bytes": {"fp32": F32.nbytes(), "fp64": F64.nbytes()},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local_rank)
        td.init_process_group("nccl")
    rc = run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
