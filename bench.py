"""Benchmark: AMG-PCG time to a 1e-10 relative residual on one GB300.

Workload (default ``c4``): 256^3 variable-coefficient Poisson with log-normal
cell conductances exp(N(0, 2^2)), harmonic-mean face coefficients, a seeded
random cell permutation (unstructured LDU addressing), rhs N(0,1) with zero
mean, diagonal shift 1e-8.  The timed method is the mixed-precision AMG-PCG
(FP32 V-cycle with forward/backward Gauss-Seidel 2/2 inside an FP64 flexible
PCG, dense FP64 coarsest solve, coarsest <= 1000 cells); the plain FP64
AMG-PCG on the same matrix is timed beside it.

A "step" is one complete solve from x = 0 to ||b - A x|| <= 1e-10 ||b||
(setup -- agglomeration, coarse matrices, coarsest inverse -- is done once,
outside the timed region, as for the reference's handle API).  `value` is
the device time of one solve (CUDA events on the solver's stream), inputs
resident in HBM; `e2e` is the same solve through the host-array C ABI entry
point (unap_cuda_amg_solve_host) with the b/x host<->device copies inside.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c4]
    python bench.py --impl reference      # the CPU reference arm

Multi-GPU runs are independent replicas (one system per rank, no collective
on the data path); the reported time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    "c4": dict(desc="256^3 log-normal(sigma=2) Poisson, permuted LDU, mixed AMG-PCG tol 1e-10",
               method="amg", precision=1),
    "c2": dict(desc="128^3 7-point Laplacian, permuted LDU, FP64 AMG-PCG tol 1e-10",
               method="amg", precision=0),
}
L2_BYTES = 129 * 2 ** 20
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        backend = os.environ.get("UNAP_BENCH_BACKEND", "nccl")
        dist.init_process_group(backend=backend)
    return world, rank, local, dist


def max_over_ranks(value: float, dist, device=None) -> float:
    """Max of a per-rank float over all ranks (identity without a group)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, device=None):
    if dist is not None:
        if device is not None and str(device).startswith("cuda"):
            dist.barrier(device_ids=[int(str(device).split(":")[1])])
        else:
            dist.barrier()


def gs32_sweep_bytes(n: int, nf: int) -> int:
    """Algorithmic bytes of one FP32 Gauss-Seidel sweep over a symmetric LDU
    matrix: per cell b, x read, x write, diag (4 B each); per face one value
    and two int32 addresses (compulsory LDU data, each touched once)."""
    return 16 * n + 12 * nf


def spmv64_bytes(n: int, nf: int) -> int:
    """Algorithmic bytes of an FP64 symmetric LDU SpMV: diag, x, y (8 B each)
    per cell, one value and two int32 addresses per face."""
    return 24 * n + 16 * nf


def cpu_baseline(s, gpu_iters: int, budget_s: float = 25.0):
    """The oracle's FP64 AMG-PCG (C restatement, one host thread) on the same
    matrix: setup untimed, then a bounded sample of PCG iterations timed and
    scaled to the iteration count the GPU's FP64 solve needed."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle, OracleAmg
    orc = Oracle("orc")
    t0 = time.perf_counter()
    probe = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=1e-10, max_iter=1)
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    probe.solve(s.b)
    t1 = time.perf_counter() - t0
    probe.close()
    k = max(2, min(20, int(budget_s / max(t1, 1e-3))))
    O = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=1e-10, max_iter=k)
    t0 = time.perf_counter()
    _, st = O.solve(s.b)
    tk = time.perf_counter() - t0
    O.close()
    per_iter = (tk - t1) / max(k - 1, 1)
    est = t1 + per_iter * max(gpu_iters - 1, 0)
    return {"value": est, "unit": "s", "cores": 1, "kind": "port",
            "sample": (f"oracle FP64 AMG-PCG on the same {s.n}-cell matrix: {k} PCG iterations "
                       f"timed ({tk:.2f} s, {per_iter:.3f} s/iteration after the first), scaled "
                       f"to the GPU FP64 solve's {gpu_iters} iterations; setup {setup:.1f} s "
                       f"untimed"),
            "iterations_timed": st["n_iter"]}


def reference_arm(args, rank, dist):
    """CPU reference arm: the oracle (the reference restated; the reference's
    own build needs its source tree, absent on the GPU host) on the host."""
    if rank != 0:
        return
    from unap_gb300 import workloads as W
    wl = WORKLOADS[args.workload]
    s = W.config(args.workload, args.scale, seed=0)
    # the GPU path's FP64 iteration count is not known here: run the sample to
    # a bounded iteration count and scale by the oracle's own convergence rate
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle, OracleAmg
    orc = Oracle("orc")
    samples = []
    iters_needed = None
    for step in range(args.warmup + args.steps):
        O = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=1e-10,
                      max_iter=args.ref_iters)
        t0 = time.perf_counter()
        _, st = O.solve(s.b)
        dt = time.perf_counter() - t0
        O.close()
        # geometric convergence rate of the sample -> iterations to 1e-10
        rate = (st["final_res"] / st["init_res"]) ** (1.0 / max(st["n_iter"], 1))
        iters_needed = int(np.ceil(np.log(1e-10) / np.log(rate))) if 0 < rate < 1 else st["n_iter"]
        if step >= args.warmup:
            samples.append(dt / st["n_iter"] * iters_needed)
    value = statistics.mean(samples)
    line = {"impl": "reference", "metric": "amg_pcg_time_to_1e-10", "value": value, "unit": "s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{args.workload}: {wl['desc']} (CPU: FP64 V-cycle)",
                       "cells": s.n, "faces": s.nf},
            "cpu_baseline": {"value": value, "unit": "s", "cores": 1, "kind": "port",
                             "sample": (f"each step: oracle FP64 AMG-PCG, {args.ref_iters} PCG "
                                        f"iterations timed, scaled to the {iters_needed} "
                                        f"iterations its measured convergence rate needs for "
                                        f"1e-10; hierarchy setup untimed")},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c4", choices=sorted(WORKLOADS))
    ap.add_argument("--scale", type=float, default=1.0, help="grid edge scale (testing)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-iters", type=int, default=3)
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    world, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        reference_arm(args, rank, dist)
        if dist is not None:
            dist.destroy_process_group()
        return

    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    wl = WORKLOADS[args.workload]
    s = W.config(args.workload, args.scale, seed=rank)
    A = capi.DeviceMatrix(s)
    G = capi.DeviceAmg(A, precision=wl["precision"], rel_tol=1e-10, n_coarsest=1000)
    G64 = capi.DeviceAmg(A, precision=0, rel_tol=1e-10, n_coarsest=1000) \
        if wl["precision"] == 1 else G
    info = G.info()
    b = torch.tensor(s.b, device=device)
    x = torch.zeros(s.n, dtype=torch.float64, device=device)

    def solve(g):
        x.zero_()
        st = g.solve(x, b)
        if not st["converged"]:
            raise RuntimeError(f"solve did not converge: {st}")
        return st

    for _ in range(args.warmup):
        solve(G)
    torch.cuda.synchronize()
    barrier(dist, device)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = capi.load().unap_cuda_launch_count()
    t_wall0 = time.perf_counter()
    stats = [solve(G) for _ in range(args.steps)]
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    launches = capi.load().unap_cuda_launch_count() - launches0
    clk = clocks.stop()
    barrier(dist, device)
    dev_s = [st["seconds"] for st in stats]
    per_solve = max_over_ranks(statistics.mean(dev_s), dist, device)
    iters = stats[-1]["nIterations"]
    true_rel = stats[-1]["trueResidual"] / stats[-1]["initialResidual"]

    # FP64 AMG-PCG on the same matrix (the metric's "mixed vs FP64")
    fp64 = None
    if G64 is not G:
        for _ in range(args.warmup):
            solve(G64)
        st64 = [solve(G64) for _ in range(args.steps)]
        t64 = max_over_ranks(statistics.mean(st["seconds"] for st in st64), dist, device)
        fp64 = {"value": t64, "unit": "s", "iterations": st64[-1]["nIterations"],
                "speedup_mixed_vs_fp64": t64 / per_solve}
    gpu_iters64 = fp64["iterations"] if fp64 else iters

    # e2e: the host-array C ABI call, b/x copies inside the timed region
    xh = torch.zeros(s.n, dtype=torch.float64).pin_memory()
    bh = torch.tensor(s.b, dtype=torch.float64).pin_memory()
    for _ in range(args.warmup):
        xh.zero_()
        G.solve_host(xh.data_ptr(), bh.data_ptr())
    barrier(dist, device)
    e2e_t = []
    for _ in range(args.steps):
        xh.zero_()
        t0 = time.perf_counter()
        G.solve_host(xh.data_ptr(), bh.data_ptr())
        e2e_t.append(time.perf_counter() - t0)
    e2e_v = max_over_ranks(statistics.mean(e2e_t), dist, device)

    # roofline of the dominant kernel: the finest level's FP32 Gauss-Seidel
    # sweep (all wavefront launches of one sweep), timed with CUDA events on
    # the matrix's stream right after the timed region
    prof = A.profile(reps=10)
    peak, peak_kind = hbm_peak()
    if wl["precision"] == 1:
        k_ms = prof["gs_fwd32"]
        k_bytes = gs32_sweep_bytes(s.n, s.nf)
        k_name = "gs_kernel<float> (finest-level FP32 Gauss-Seidel sweep)"
    else:
        k_ms = prof["gs_fwd"]
        k_bytes = 32 * s.n + 16 * s.nf
        k_name = "gs_kernel<double> (finest-level FP64 Gauss-Seidel sweep)"
    achieved = k_bytes / (k_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None, "kernel": k_name,
                "algorithmic_bytes_per_launch": k_bytes, "launch_ms": k_ms,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "spmv64": {"achieved": spmv64_bytes(s.n, s.nf) / (prof["spmv"] * 1e-3) / 1e9,
                           "ms": prof["spmv"]}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(s, gpu_iters64)
        except Exception as e:  # reported, never fatal
            cpu = {"value": None, "unit": "s", "cores": 1, "kind": "port",
                   "sample": f"failed: {e}"}

    matrix_bytes = A.info()["device_bytes"]
    line = {
        "metric": "amg_pcg_time_to_1e-10",
        "value": per_solve,
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": per_solve * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 outer PCG + f32 V-cycle" if wl["precision"] == 1 else "f64",
        "data": "synthetic (seeded generator; the reference ships no data sets)",
        "config": {"workload": f"{args.workload}: {wl['desc']}", "cells": s.n, "faces": s.nf,
                   "levels": info["n_levels"], "level_cells": info["cells"],
                   "coarsest": info["cells"][-1], "iterations": iters,
                   "true_relative_residual": true_rel,
                   "l2": f"inputs larger than L2: matrix {matrix_bytes / 1e9:.2f} GB on device "
                         f"> {L2_BYTES / 1e6:.0f} MB",
                   "setup_s": info["setup_s"], "wall_s_per_step": t_wall / args.steps,
                   "parallelism": f"replicas x{world}"},
        "fp64": fp64,
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": 2 * 8 * s.n,
                "d2h_bytes_per_step": 8 * s.n},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    G.close()
    if G64 is not G:
        G64.close()
    A.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
