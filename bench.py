"""Benchmark: AMG-PCG time to a 1e-10 relative residual on one GB300.

Workload (default ``c4``): 256^3 variable-coefficient Poisson with log-normal
cell conductances exp(N(0, 2^2)), harmonic-mean face coefficients, a seeded
random cell permutation (unstructured LDU addressing), rhs N(0,1) with zero
mean, diagonal shift 1e-8.  The timed method is the mixed-precision AMG-PCG:
an FP32 V-cycle inside an FP64 flexible PCG, dense FP64 coarsest solve,
coarsest <= 1000 cells, the finest level smoothed by one forward and one
backward Gauss-Seidel sweep and every coarser level by the reference's
Chebyshev iteration of degree 3 (eigenvalue interval [lambda/30, 1.1
lambda], lambda estimated once per level at setup).  The same method in FP64 is timed beside
it, and the all-Gauss-Seidel V-cycle in both precisions for comparison.

A "step" is one complete solve from x = 0 to ||b - A x|| <= 1e-10 ||b||
(setup -- agglomeration, coarse matrices, eigenvalue estimates, coarsest
inverse -- is done once, outside the timed region, as for the reference's
handle API).  `value` is the device time of one solve (CUDA events on the
solver's stream), inputs resident in HBM; `e2e` is the same solve through
the host-array C ABI entry point (unap_cuda_amg_solve_host) with the b/x
host<->device copies inside.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c4]
    python bench.py --impl reference      # the CPU reference arm

A 1-GPU run also reports configs c1-c3 (GPU device time, e2e through the
reference's one-shot C ABI calls, the oracle's CPU time on a bounded sample)
and serves the seeded 2000-request stream of config c5 (`serving`: solves/s
and p50/p99 latency from each request's scheduled arrival, beside the plain
one-at-a-time FP64 path queued on the same arrival schedule; `--serve 0`
skips it, `--no-configs` skips c1-c3).

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

# the headline V-cycle: one forward and one backward Gauss-Seidel sweep on
# the two finest levels, Chebyshev of degree 3 (interval [lambda/60,
# 1.1 lambda]) on every level below them.  Measured on the 256^3 solve
# against the alternatives: Chebyshev from level 1 0.342 s (68 iterations),
# from level 2 0.330 s (69), from level 3 0.332 s (69), from level 4
# 0.340 s (70); with the interval [lambda/60, 1.1 lambda] from level 2
# 0.320 s (66), [lambda/100, ...] 0.320 s (65), [lambda/45, ...] 0.327 s.
CHEBY = dict(smoother=1, cheby_degree=3, cheby_from=2, eig_ratio=60.0, n_pre=1, n_post=1)
WORKLOADS = {
    "c4": dict(desc="256^3 log-normal(sigma=2) Poisson, permuted LDU, mixed AMG-PCG "
                    "(levels 0-1 Gauss-Seidel 1/1, Chebyshev degree 3 below), tol 1e-10",
               method="amg", precision=1, amg=CHEBY, rel_tol=1e-10),
    "c2": dict(desc="128^3 7-point Laplacian, permuted LDU, FP64 AMG-PCG "
                    "(symmetric Gauss-Seidel 2/2), tol 1e-10",
               method="amg", precision=0, amg=dict(smoother=0), rel_tol=1e-10),
}
# configs reported beside the headline (reference methods where it has them)
CONFIGS = {
    "c1": dict(desc="32^3 Laplacian, natural order, PCG+DIC, tol 1e-8", kind="krylov",
               method=0, precond=2, rel_tol=1e-8),
    "c2": dict(desc="128^3 permuted Laplacian, FP64 AMG-PCG (Gauss-Seidel 2/2), tol 1e-10",
               kind="amg", precision=0, amg=dict(smoother=0), rel_tol=1e-10),
    "c3": dict(desc="200^3 permuted convection-diffusion (Pe 5), PBiCGStab+DILU, tol 1e-9",
               kind="krylov", method=1, precond=3, rel_tol=1e-9),
}
L2_BYTES = 129 * 2 ** 20
# DRAM bytes (read + write) per algorithmic byte of a kernel family, from
# one ncu capture of a smaller case; the roofline's `traffic` scales it to
# the launch group's algorithmic bytes (the traffic grows with the rows)
TRAFFIC_RATIO = {
    "gs_kernel<float>": (
        471.9 / 366.7,
        "ncu dram__bytes_read.sum + dram__bytes_write.sum of the 19 wavefront launches of one "
        "FP32 forward sweep of the 192^3 finest level, caches as the program left them: "
        "471.9 MB against 366.7 MB algorithmic, scaled by the launch group's algorithmic "
        "bytes"),
    "cheb_step_kernel<float>": (
        327.9 / 258.9,
        "ncu dram__bytes_read.sum + dram__bytes_write.sum of one Chebyshev step on level 1 "
        "of the 192^3 hierarchy (3,273,854 rows): 327.9 MB against 258.9 MB algorithmic, "
        "scaled by the launch group's algorithmic bytes"),
}
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


def spmv64_bytes(n: int, nf: int, symm: bool = True) -> int:
    """Algorithmic bytes of an FP64 LDU SpMV: diag, x, y (8 B each) per cell;
    per face one value (two if asymmetric) and two int32 addresses."""
    return 24 * n + (16 if symm else 24) * nf


def amg_kwargs(cfg) -> dict:
    """DeviceAmg / OracleAmg keyword arguments of a workload's V-cycle."""
    return dict(cfg.get("amg", {}))


def oracle_amg_sample(s, cfg, gpu_iters: int, caps=(1, 2)):
    """The oracle's FP64 AMG-PCG (C restatement, one host thread) on `s` with
    the workload's V-cycle: hierarchy and eigenvalue estimates untimed, then
    solves capped at caps[0] and caps[1] iterations; the time per iteration
    is their difference over the iterations between, the fixed cost (initial
    residual, allocations, final true residual) what is left of the shorter
    one, and the estimate is fixed + per_iter * gpu_iters."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle, OracleAmg
    orc = Oracle("orc")
    t0 = time.perf_counter()
    O = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=cfg["rel_tol"],
                  max_iter=caps[0], **amg_kwargs(cfg))
    setup = time.perf_counter() - t0
    t = []
    for k in caps:
        O.set_max_iter(k)
        t0 = time.perf_counter()
        O.solve(s.b)
        t.append(time.perf_counter() - t0)
    O.close()
    per_iter = max((t[1] - t[0]) / (caps[1] - caps[0]), 1e-9)
    fixed = max(t[0] - caps[0] * per_iter, 0.0)
    return {"value": fixed + per_iter * gpu_iters, "unit": "s", "cores": 1, "kind": "port",
            "per_iteration_s": per_iter, "fixed_s": fixed, "setup_s": setup,
            "sample": (f"oracle FP64 AMG-PCG (same V-cycle) on the same {s.n}-cell matrix: solves "
                       f"capped at {caps[0]} and {caps[1]} iterations timed ({t[0]:.2f} s, "
                       f"{t[1]:.2f} s), {per_iter:.3f} s/iteration + {fixed:.2f} s fixed cost, "
                       f"scaled to the GPU FP64 solve's {gpu_iters} iterations; setup "
                       f"{setup:.1f} s untimed")}


def oracle_krylov_sample(s, cfg, gpu_iters: int, full_below: int = 200_000):
    """The oracle's PCG / PBiCGStab (the reference's methods restated, one
    host thread): a full solve on small systems, else solves capped at 1 and
    3 iterations scaled to the GPU's iteration count (fixed cost separate)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    orc = Oracle("orc")
    fn = orc.pcg if cfg["method"] == 0 else orc.pbicgstab
    if s.n <= full_below:
        t0 = time.perf_counter()
        _, st = fn(s, cfg["precond"], s.b, rel_tol=cfg["rel_tol"], max_iter=5000)
        dt = time.perf_counter() - t0
        return {"value": dt, "unit": "s", "cores": 1, "kind": "port", "iterations": st["n_iter"],
                "sample": f"oracle full solve, {st['n_iter']} iterations"}
    t = []
    for k in (1, 3):
        t0 = time.perf_counter()
        fn(s, cfg["precond"], s.b, rel_tol=cfg["rel_tol"], max_iter=k)
        t.append(time.perf_counter() - t0)
    per_iter = max((t[1] - t[0]) / 2, 1e-9)
    fixed = max(t[0] - per_iter, 0.0)
    return {"value": fixed + per_iter * gpu_iters, "unit": "s", "cores": 1, "kind": "port",
            "per_iteration_s": per_iter, "fixed_s": fixed,
            "sample": (f"oracle solves capped at 1 and 3 iterations ({t[0]:.2f} s, {t[1]:.2f} s), "
                       f"scaled to the GPU solve's {gpu_iters} iterations")}


def reference_arm(args, rank, dist):
    """CPU reference arm: the oracle (the reference restated; the reference's
    own build needs its source tree, absent on the GPU host) on the host.
    The reference has no AMG-PCG (its MGPrecond is a stub), so this is the
    restatement's FP64 AMG-PCG with the workload's V-cycle."""
    if rank != 0:
        return
    from unap_gb300 import workloads as W
    wl = WORKLOADS[args.workload]
    s = W.config(args.workload, args.scale, seed=0)
    # A full solve at 256^3 takes the oracle about 15 minutes.  The warm-up
    # builds the hierarchy once (untimed, as the GPU arm's), runs solves
    # capped at 1 and 6 iterations: their time difference gives the cost per
    # iteration and the fixed cost (initial residual, allocations, final true
    # residual) apart, and their residuals the convergence rate, which
    # predicts the iterations to 1e-10.  Each timed step is one capped solve
    # whose iterations are scaled to that count, its fixed cost counted once.
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle, OracleAmg
    orc = Oracle("orc")
    O = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=wl["rel_tol"], max_iter=1,
                  **amg_kwargs(wl))
    t0 = time.perf_counter()
    _, s1 = O.solve(s.b)
    t1 = time.perf_counter() - t0
    O.set_max_iter(6)
    t0 = time.perf_counter()
    _, s6 = O.solve(s.b)
    t6 = time.perf_counter() - t0
    fixed = max(t1 - (t6 - t1) / 5.0, 0.0)
    iters_needed = s6["n_iter"]
    if not s6["converged"] and s1["n_iter"] == 1 and s6["n_iter"] == 6:
        rate = (s6["final_res"] / s1["final_res"]) ** 0.2
        if 0 < rate < 1:
            more = np.log(wl["rel_tol"] * s6["init_res"] / s6["final_res"]) / np.log(rate)
            iters_needed = 6 + max(0, int(np.ceil(more)))
    O.set_max_iter(args.ref_iters)
    samples = []
    for step in range(max(args.warmup - 2, 0) + args.steps):
        t0 = time.perf_counter()
        _, st = O.solve(s.b)
        dt = time.perf_counter() - t0
        if step >= args.warmup - 2:
            per_iter = max(dt - fixed, 0.0) / st["n_iter"]
            samples.append(fixed + per_iter * iters_needed)
    O.close()
    value = statistics.mean(samples)
    line = {"impl": "reference", "metric": "amg_pcg_time_to_1e-10", "value": value, "unit": "s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{args.workload}: {wl['desc']} (CPU: FP64 V-cycle)",
                       "cells": s.n, "faces": s.nf},
            "estimate": True,
            "cpu_baseline": {"value": value, "unit": "s", "cores": 1, "kind": "port",
                             "fixed_s": fixed, "per_iteration_s": (t6 - t1) / 5.0,
                             "iterations_predicted": iters_needed,
                             "sample": (f"each step: oracle FP64 AMG-PCG solve capped at "
                                        f"{args.ref_iters} iteration(s); its time less the "
                                        f"fixed cost ({fixed:.2f} s, from solves capped at 1 "
                                        f"and 6 iterations) is scaled to the {iters_needed} "
                                        f"iterations to {wl['rel_tol']:g} that the convergence "
                                        f"rate between iterations 1 and 6 predicts, and the "
                                        f"fixed cost added once; hierarchy setup untimed; an "
                                        f"estimate, not a measured time to solution")},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# configs c1-c3 beside the headline
# ---------------------------------------------------------------------------
def config_block(name: str, steps: int, warmup: int, cpu: bool):
    """GPU device time, e2e through the reference's C ABI and the oracle's CPU
    time of one of configs c1-c3 (no hierarchy of the headline is alive)."""
    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    cfg = CONFIGS[name]
    t0 = time.perf_counter()
    s = W.config(name, 1.0, seed=0)
    gen = time.perf_counter() - t0
    out = {"desc": cfg["desc"], "cells": s.n, "faces": s.nf, "generate_s": gen}
    A = capi.DeviceMatrix(s)
    b = torch.tensor(s.b, device="cuda")
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    peak, _ = hbm_peak()
    if cfg["kind"] == "krylov":
        def one():
            x.zero_()
            return A.krylov_solve(cfg["method"], cfg["precond"], x, b, rel_tol=cfg["rel_tol"],
                                  max_iter=5000)
    else:
        G = capi.DeviceAmg(A, precision=cfg["precision"], rel_tol=cfg["rel_tol"],
                           n_coarsest=1000, **amg_kwargs(cfg))

        def one():
            x.zero_()
            return G.solve(x, b)
    for _ in range(warmup):
        one()
    st = [one() for _ in range(steps)]
    if not all(q["converged"] for q in st):
        raise RuntimeError(f"{name} did not converge: {st[-1]}")
    out["gpu_s"] = statistics.mean(q["seconds"] for q in st)
    out["iterations"] = st[-1]["nIterations"]
    out["true_relative_residual"] = st[-1]["trueResidual"] / st[-1]["initialResidual"] \
        if st[-1]["trueResidual"] > 0 else None
    if st[-1]["algorithmicBytes"] > 0:
        out["whole_solve_gbs"] = st[-1]["algorithmicBytes"] / out["gpu_s"] / 1e9
    prof = A.profile(reps=10)
    symm = s.symm
    k = {"spmv": ("spmv_kernel<double>", spmv64_bytes(s.n, s.nf, symm))}
    if cfg["kind"] == "krylov":
        key = "dic_apply" if cfg["precond"] == 2 else "dilu_apply"
        k[key] = (("dic" if cfg["precond"] == 2 else "dilu") + "_fwd/bwd_kernel",
                  40 * s.n + (32 if symm else 40) * s.nf)
    out["kernels"] = {key: {"kernel": nm, "ms": prof[key], "algorithmic_bytes": by,
                            "achieved_gbs": by / (prof[key] * 1e-3) / 1e9,
                            "frac": by / (prof[key] * 1e-3) / 1e9 / peak}
                      for key, (nm, by) in k.items()}
    # e2e through the reference-facing C ABI with host arrays
    e2e = []
    if cfg["kind"] == "krylov":
        fn = capi.pcgsolversolve if cfg["method"] == 0 else capi.pbicgstabsolversolve
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            h = capi.ldumatrixcreat(s)
            _, it, _ = fn(np.zeros(s.n), h, s.b, cfg["precond"], rel_tol=cfg["rel_tol"],
                          max_iter=5000)
            if i >= warmup:
                e2e.append(time.perf_counter() - t0)
        out["e2e"] = {"value": statistics.mean(e2e), "unit": "s",
                      "call": "ldumatrixcreat_ + " + fn.__name__ + "_ (host arrays, matrix "
                              "upload and device setup included)",
                      "h2d_bytes_per_step": 16 * s.n + (16 if symm else 24) * s.nf,
                      "d2h_bytes_per_step": 8 * s.n}
    else:
        xh = np.zeros(s.n)
        for i in range(warmup + steps):
            xh[:] = 0
            t0 = time.perf_counter()
            G.solve_host(xh, np.ascontiguousarray(s.b))
            if i >= warmup:
                e2e.append(time.perf_counter() - t0)
        out["e2e"] = {"value": statistics.mean(e2e), "unit": "s", "call": "unap_cuda_amg_solve_host",
                      "h2d_bytes_per_step": 16 * s.n, "d2h_bytes_per_step": 8 * s.n}
        G.close()
    A.close()
    if cpu:
        try:
            out["cpu_baseline"] = (oracle_krylov_sample(s, cfg, out["iterations"])
                                   if cfg["kind"] == "krylov"
                                   else oracle_amg_sample(s, cfg, out["iterations"], caps=(1, 3)))
            out["cpu_over_gpu"] = out["cpu_baseline"]["value"] / out["gpu_s"]
        except Exception as e:  # reported, never fatal
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    return out


# ---------------------------------------------------------------------------
# c5: the served stream
# ---------------------------------------------------------------------------
class _Builder:
    """Builds stream requests in a spawn-context process pool (the parent has
    a CUDA context), at most `window` ahead of the consumer."""

    def __init__(self, specs, window: int, procs: int):
        import multiprocessing as mp
        from unap_gb300 import workloads as W
        self.specs = specs
        self.pool = mp.get_context("spawn").Pool(procs)
        self.window = window
        self.pending = {}
        self.next_submit = 0
        self.fn = W.build_request
        self._fill(0)

    def _fill(self, i):
        while self.next_submit < len(self.specs) and self.next_submit < i + self.window:
            j = self.next_submit
            self.pending[j] = self.pool.apply_async(self.fn, (self.specs[j],))
            self.next_submit += 1

    def get(self, i):
        self._fill(i)
        r = self.pending.pop(i).get()
        self._fill(i + 1)
        return r

    def close(self):
        self.pool.terminate()
        self.pool.join()


def serve_bench(n_requests: int, seed: int = 0, max_slots: int = 12, compare_plain: bool = True,
                window: int = 64, procs: int = 0, prebuild: bool = False):
    """Config c5 served: the seeded request stream (Poisson arrivals at 200/s,
    sizes log-uniform 8k-2M cells, 60% mixed AMG-PCG / 25% PCG+DIC / 15%
    PBiCGStab+DILU, tol 1e-8) submitted on its arrival schedule to the
    continuous-batching server; then the same requests one at a time through
    the plain FP64 path (FP64 AMG-PCG instead of mixed).  Latency is counted
    from each request's scheduled arrival in both: the served requests'
    completions are measured, the plain path's service times are measured one
    by one and queued first-in first-out on the same arrival schedule.
    Request matrices are built by a process pool just ahead of submission;
    `producer` reports whether the server ever waited for them."""
    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    specs = W.serving_stream(count=n_requests, rate=200.0, seed=seed)
    procs = procs or max(2, min(12, (os.cpu_count() or 4) - 4))
    srv = capi.Server(max_slots=max_slots)
    B = _Builder(specs, len(specs) if prebuild else window, procs)
    if prebuild:
        # every request built before the first arrival: the builders'
        # processes are idle while the server runs
        built = [B.get(i) for i in range(len(specs))]
        B.close()
        B = None
    sub_t, ids, ns, inflight_at_late = [], [], [], []
    results = [None] * len(specs)
    done_count = [0]
    lock = threading.Condition()

    def waiter():
        for i in range(len(specs)):
            with lock:
                lock.wait_for(lambda: len(ids) > i)
                rid, n = ids[i], ns[i]
            _, info = srv.wait(rid, n)
            with lock:
                results[i] = info
                done_count[0] += 1
                lock.notify_all()

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    t0 = time.perf_counter()
    for i, sp in enumerate(specs):
        if B is None:
            r = built[i]
            built[i] = None
        else:
            r = B.get(i)
        with lock:  # bounded server queue: at most `window` requests in flight
            lock.wait_for(lambda: len(ids) - done_count[0] < window)
        dt = sp.arrival - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        now = time.perf_counter() - t0
        if now > sp.arrival + 0.001:
            inflight_at_late.append(len(ids) - done_count[0])
        rid = srv.submit(r.system, r.method, rel_tol=1e-8, max_iter=2000)
        with lock:
            sub_t.append(now)
            ids.append(rid)
            ns.append(r.system.n)
            lock.notify_all()
        del r
    th.join()
    srv.close()
    if B is not None:
        B.close()
    lat, setup, solve_t, queue, batched = [], [], [], [], 0
    for sp, st_, info in zip(specs, sub_t, results):
        if not info["converged"]:
            raise RuntimeError(f"served request did not converge: {info}")
        lat.append(st_ + info["latencySeconds"] - sp.arrival)
        setup.append(info["setupSeconds"])
        solve_t.append(info["solveSeconds"])
        queue.append(info["queueSeconds"])
        batched += info["batched"]
    last = max(st_ + info["latencySeconds"] for st_, info in zip(sub_t, results))
    pct = lambda v, q: float(np.percentile(np.array(v), q))
    out = {"requests": n_requests, "rate_per_s": 200.0,
           "solves_per_s": n_requests / (last - specs[0].arrival),
           "p50_s": pct(lat, 50), "p99_s": pct(lat, 99),
           "latency": "completion - scheduled arrival (queueing included)",
           "batched_requests": batched, "slots": max_slots,
           "mean_server_queue_s": float(np.mean(queue)), "mean_setup_s": float(np.mean(setup)),
           "mean_solve_s": float(np.mean(solve_t)),
           "amg_method": "mixed AMG-PCG, Chebyshev degree 3 V-cycle",
           "producer": {"build_processes": procs, "window": window,
                        "submitted_after_arrival": len(inflight_at_late),
                        "min_in_flight_then": min(inflight_at_late) if inflight_at_late else None,
                        "note": "the server was never short of work when min_in_flight_then "
                                "exceeds the slots"}}
    if not compare_plain:
        return out
    # the plain path: one request at a time, FP64 everywhere
    B = _Builder(specs, 16, procs)
    svc = []
    try:
        for i, sp in enumerate(specs):
            r = B.get(i)
            s = r.system
            b = torch.tensor(s.b, device="cuda")
            torch.cuda.synchronize()
            ts = time.perf_counter()
            A = capi.DeviceMatrix(s)
            x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            if r.method == "amg_mixed":
                G = capi.DeviceAmg(A, precision=0, rel_tol=1e-8, max_iter=2000,
                                   smoother=1, cheby_degree=3, cheby_from=0, eig_ratio=30.0)
                st = G.solve(x, b)
                G.close()
            else:
                st = A.krylov_solve(0 if r.method == "pcg_dic" else 1,
                                    2 if r.method == "pcg_dic" else 3, x, b, rel_tol=1e-8,
                                    max_iter=2000)
            _ = x.cpu()
            A.close()
            svc.append(time.perf_counter() - ts)
            if not st["converged"]:
                raise RuntimeError(f"plain request did not converge: {st}")
    finally:
        B.close()
    c, qlat = 0.0, []
    for sp, dt in zip(specs, svc):
        c = max(c, sp.arrival) + dt
        qlat.append(c - sp.arrival)
    out["one_at_a_time_fp64"] = {
        "solves_per_s": n_requests / (c - specs[0].arrival),
        "p50_s": pct(qlat, 50), "p99_s": pct(qlat, 99),
        "latency": "first-in first-out on the same arrival schedule: completion - scheduled "
                   "arrival, from each request's measured service time",
        "service_p50_s": pct(svc, 50), "service_p99_s": pct(svc, 99),
        "amg_method": "FP64 AMG-PCG, Chebyshev degree 3 V-cycle"}
    return out


def krylov_case(args):
    """One solve of a Krylov config (c1 or c3) through the reference's method,
    timed with CUDA events after `--warmup` solves (the small case for the
    whole-solve launch's profile); `--team-shape T,C` forces the launch
    shape of the whole-solve launch (c1's size)."""
    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    torch.cuda.set_device(0)
    name = args.krylov_config
    cfg = CONFIGS[name]
    if cfg["kind"] != "krylov":
        raise SystemExit(f"{name} is not a Krylov config")
    if args.team_shape:
        t, c = (int(v) for v in args.team_shape.split(","))
        capi.force_team_shape(t, c)
    s = W.config(name, args.scale, seed=0)
    A = capi.DeviceMatrix(s)
    b = torch.tensor(s.b, device="cuda")
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup + 1):
        x.zero_()
        st = A.krylov_solve(cfg["method"], cfg["precond"], x, b, rel_tol=cfg["rel_tol"],
                            max_iter=5000)
    print(json.dumps({"config": name, "cells": s.n, "iterations": st["nIterations"],
                      "seconds": st["seconds"], "shape": capi.team_shape(s.n, 1)}), flush=True)
    A.close()


def kernels_case(args):
    """Finest-level kernels of the workload's matrix, each launched on its own
    and timed with CUDA events (SpMV, DIC/DILU, Gauss-Seidel sweeps FP64 and
    FP32, residual).  No AMG hierarchy is built, so the device holds only the
    matrix and a few vectors."""
    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    torch.cuda.set_device(0)
    s = W.config(args.workload, args.scale, seed=0)
    A = capi.DeviceMatrix(s)
    prof = A.profile(reps=args.reps)
    print(json.dumps({"workload": args.workload, "scale": args.scale, "cells": s.n,
                      "faces": s.nf, "ms": prof, **A.info()}), flush=True)
    A.close()


def smoother_case(args):
    """One smoothing launch group (a Chebyshev step, or a Gauss-Seidel sweep)
    on AMG level `--smoother-level` of the workload's hierarchy, timed with
    CUDA events after one warm-up (the small case for kernel profiles)."""
    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    torch.cuda.set_device(0)
    wl = WORKLOADS[args.workload]
    s = W.config(args.workload, args.scale, seed=0)
    A = capi.DeviceMatrix(s)
    G = capi.DeviceAmg(A, precision=wl["precision"], rel_tol=wl["rel_tol"], n_coarsest=1000,
                       **amg_kwargs(wl))
    sizes = G.level_sizes()
    k = args.smoother_level
    ms, by, launches = G.profile_smoother(k, reps=args.reps)
    print(json.dumps({"workload": args.workload, "scale": args.scale, "level": k,
                      "rows": sizes[k][0], "faces": sizes[k][1], "ms": ms,
                      "algorithmic_bytes": by, "launches": launches,
                      "achieved_gbs": by / (ms * 1e-3) / 1e9}), flush=True)
    G.close()
    A.close()


def textio_case(args):
    """Host text I/O of the workload's matrix in the reference's LDU dump
    format: print it, read it back (both through the C ABI, from a pool of
    host threads), and, where the reference build oracle/_ref loads (the x86
    host it was compiled on), the reference's own reader and printer on the
    same file.  No GPU work."""
    import shutil
    import tempfile
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    s = W.config(args.workload, args.scale, seed=0)
    h0 = capi.ldumatrixcreat(s)
    d = tempfile.mkdtemp(prefix="unap_textio_")
    out = {"mode": "textio", "workload": args.workload, "scale": args.scale, "cells": s.n,
           "faces": s.nf, "threads": os.cpu_count()}
    try:
        t = time.perf_counter()
        f = capi.print_ldu_matrix(h0, os.path.join(d, "A"))
        out["print_s"] = time.perf_counter() - t
        out["file_mb"] = os.path.getsize(f) / 1e6
        t = time.perf_counter()
        h = capi.read_ldu_matrix(f)
        out["read_s"] = time.perf_counter() - t
        m = capi.handle_ldu(h)
        out["read_matches_print"] = bool(np.array_equal(m["upper_addr"], s.upper_addr))
        capi.sw_matrix_destroy(h)
        ref = None
        try:
            sys.path.insert(0, os.path.join(ROOT, "tests"))
            from oracle_lib import Oracle, ref_available
            ref = Oracle("ref").lib if ref_available() else None
        except OSError as e:  # an x86 build on another host
            out["reference"] = f"unavailable: {e}"
        if ref is not None:
            import ctypes
            ref.ref_read_ldu.restype = ctypes.c_void_p
            ref.ref_read_ldu.argtypes = [ctypes.c_char_p]
            ref.ref_print_ldu.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
            ref.ref_ldu_destroy.argtypes = [ctypes.c_void_p]
            t = time.perf_counter()
            A = ref.ref_read_ldu(os.fsencode(f))
            rr = time.perf_counter() - t
            t = time.perf_counter()
            ref.ref_print_ldu(A, os.fsencode(os.path.join(d, "B")))
            rp = time.perf_counter() - t
            ref.ref_ldu_destroy(A)
            same = open(f, "rb").read() == open(os.path.join(d, "B_0.txt"), "rb").read()
            out["reference"] = {"read_s": rr, "print_s": rp, "cores": 1,
                                "files_byte_identical": same}
        elif "reference" not in out:
            out["reference"] = "unavailable: oracle/_ref not built on this host"
    finally:
        capi.sw_matrix_destroy(h0)
        shutil.rmtree(d, ignore_errors=True)
    print(json.dumps(out), flush=True)


def setup_case(args):
    """Setup of the workload's matrix and mixed AMG hierarchy, built by the
    device kernels (the default) and by the host loops, wall-clock timed
    with the device synchronized; the two must give the same internal order
    and hierarchy."""
    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    torch.cuda.set_device(0)
    s = W.config(args.workload, args.scale, seed=0)
    wl = WORKLOADS[args.workload]
    out = {"mode": "setup", "workload": args.workload, "scale": args.scale, "cells": s.n,
           "faces": s.nf}
    layouts = {}
    for name, min_cells in (("device", 32768), ("host", -1)):
        old = capi.set_device_setup(min_cells)
        bracket = args.profile_solve and name == "device"
        try:
            torch.cuda.synchronize()
            if bracket:
                torch.cuda.profiler.start()
            t0 = time.perf_counter()
            A = capi.DeviceMatrix(s)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            G = capi.DeviceAmg(A, precision=wl["precision"], rel_tol=1e-10, n_coarsest=1000)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            if bracket:
                torch.cuda.profiler.stop()
        finally:
            capi.set_device_setup(old)
        info = G.info()
        layouts[name] = (A.layout()[0], info["cells"])
        out[name] = {"matrix_s": t1 - t0, "amg_s": t2 - t1, "levels": info["n_levels"]}
        G.close()
        A.close()
    out["same_order_and_hierarchy"] = bool(
        np.array_equal(layouts["device"][0], layouts["host"][0])
        and layouts["device"][1] == layouts["host"][1])
    out["speedup"] = ((out["host"]["matrix_s"] + out["host"]["amg_s"])
                      / (out["device"]["matrix_s"] + out["device"]["amg_s"]))
    print(json.dumps(out), flush=True)


def smoother_roofline(G, info, mixed: bool, peak: float, deg: int, sweeps: int):
    """Per-level smoother launch groups of the V-cycle timed with CUDA events
    (unap_cuda_amg_profile_smoother), and the kernel family with the largest
    device time per V-cycle: Chebyshev steps (2 deg - 1 launches per level
    and V-cycle: the first pre-smoothing step runs inside the restriction)
    or Gauss-Seidel sweeps (`sweeps` = nPre + nPost per level)."""
    fam = {"cheb": {"ms": 0.0, "bytes": 0.0, "levels": []},
           "gs_fine": {"ms": 0.0, "bytes": 0.0, "levels": []},
           "gs_coarse": {"ms": 0.0, "bytes": 0.0, "levels": []}}
    lam = G.eigenvalues()
    per_level = []
    for k in range(info["n_levels"] - 1):
        ms, by, launches = G.profile_smoother(k, reps=10)
        cheb = lam[k] > 0
        reps = (2 * deg - 1) if cheb else sweeps
        f = "cheb" if cheb else ("gs_fine" if k == 0 else "gs_coarse")
        fam[f]["ms"] += reps * ms
        fam[f]["bytes"] += reps * by
        fam[f]["levels"].append(k)
        per_level.append({"level": k, "smoother": "chebyshev" if cheb else "gauss-seidel",
                          "ms": ms, "launches": launches, "algorithmic_bytes": by,
                          "achieved_gbs": by / (ms * 1e-3) / 1e9})
    names = {"cheb": "cheb_step_kernel<%s>" % ("float" if mixed else "double"),
             "gs_fine": "gs_kernel<%s>" % ("float" if mixed else "double"),
             "gs_coarse": "gs_packed_kernel<%s>" % ("float" if mixed else "double")}
    groups = {}
    for f, v in fam.items():
        if v["ms"] > 0:
            ach = v["bytes"] / (v["ms"] * 1e-3) / 1e9
            groups[f] = {"kernel": names[f], "levels": v["levels"], "ms_per_vcycle": v["ms"],
                         "algorithmic_bytes_per_vcycle": v["bytes"], "achieved": ach,
                         "frac": ach / peak}
    top = max(groups, key=lambda f: groups[f]["ms_per_vcycle"])
    return top, groups, per_level


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c4", choices=sorted(WORKLOADS))
    ap.add_argument("--scale", type=float, default=1.0, help="grid edge scale (testing)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the c1-c3 blocks")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the all-Gauss-Seidel V-cycle comparison")
    ap.add_argument("--ref-iters", type=int, default=1,
                    help="PCG iterations per reference-arm sample")
    ap.add_argument("--serve", type=int, default=2000,
                    help="also serve this many requests of the c5 stream (rank 0 of a "
                         "1-GPU run; 0: skip)")
    ap.add_argument("--serve-slots", type=int, default=12,
                    help="concurrent large-request slots of the server")
    ap.add_argument("--kernels", action="store_true",
                    help="only time the finest-level kernels one launch at a time "
                         "(the small case for kernel profiles) and exit")
    ap.add_argument("--reps", type=int, default=5, help="repetitions for --kernels")
    ap.add_argument("--krylov-config", default="", choices=["", "c1", "c3"],
                    help="only run one solve of this Krylov config (after --warmup) and exit")
    ap.add_argument("--team-shape", default="",
                    help="with --krylov-config: force the whole-solve launch shape 'T,C'")
    ap.add_argument("--profile-solve", action="store_true",
                    help="bracket one extra mixed solve after the timed ones (with --setup: "
                         "the device setup) with cudaProfilerStart/Stop, for ncu "
                         "--profile-from-start off")
    ap.add_argument("--smoother-level", type=int, default=-1,
                    help="only time one smoothing launch group on this AMG level (the small "
                         "case for kernel profiles) and exit")
    ap.add_argument("--setup", action="store_true",
                    help="only time the matrix and hierarchy setup, device vs host, and exit")
    ap.add_argument("--textio", action="store_true",
                    help="only time the LDU text dump printer and reader (host) and exit")
    args = ap.parse_args()
    if args.textio:
        textio_case(args)
        return
    if args.setup:
        setup_case(args)
        return
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.kernels:
        kernels_case(args)
        return
    if args.krylov_config:
        krylov_case(args)
        return
    if args.smoother_level >= 0:
        smoother_case(args)
        return
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
    mixed = wl["precision"] == 1
    kw = amg_kwargs(wl)
    G = capi.DeviceAmg(A, precision=wl["precision"], rel_tol=wl["rel_tol"], n_coarsest=1000, **kw)
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
    if args.profile_solve:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        solve(G)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    dev_s = [st["seconds"] for st in stats]
    per_solve = max_over_ranks(statistics.mean(dev_s), dist, device)
    iters = stats[-1]["nIterations"]
    true_rel = stats[-1]["trueResidual"] / stats[-1]["initialResidual"]
    x_head = x.clone()

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

    # roofline: the smoother kernel family with the largest device time per
    # V-cycle, from per-level launch groups timed with CUDA events
    peak, peak_kind = hbm_peak()
    peak_src = ("measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s")
    deg = kw.get("cheby_degree", 3)
    top, groups, per_level = smoother_roofline(G, info, mixed, peak, deg,
                                               kw.get("n_pre", 2) + kw.get("n_post", 2))
    vprof = G.profile_vcycle(reps=10)
    mprof = A.profile(reps=10)
    spmv = {"kernel": "spmv_kernel<double>", "ms": mprof["spmv"],
            "achieved": spmv64_bytes(s.n, s.nf) / (mprof["spmv"] * 1e-3) / 1e9}
    spmv["frac"] = spmv["achieved"] / peak
    solve_bytes = stats[-1].get("algorithmicBytes", 0.0)
    whole = None
    if solve_bytes > 0:
        whole = {"algorithmic_bytes": solve_bytes, "s": statistics.mean(dev_s),
                 "achieved": solve_bytes / statistics.mean(dev_s) / 1e9}
        whole["frac"] = whole["achieved"] / peak
    tg = groups[top]
    ratio = TRAFFIC_RATIO.get(tg["kernel"])
    roofline = {"bound": "hbm", "achieved": tg["achieved"], "peak": peak, "unit": "GB/s",
                "frac": tg["achieved"] / peak,
                "traffic": ratio[0] * tg["algorithmic_bytes_per_vcycle"] if ratio else None,
                "traffic_basis": ratio[1] if ratio else None,
                "kernel": tg["kernel"], "levels": tg["levels"],
                "launch_group": ("every launch of this kernel in one V-cycle, each level's "
                                 "launch group timed alone with CUDA events on the matrix's "
                                 "stream (inputs larger than L2 on the largest levels)"),
                "ms_per_vcycle": tg["ms_per_vcycle"],
                "algorithmic_bytes_per_vcycle": tg["algorithmic_bytes_per_vcycle"],
                "peak_source": peak_src, "groups": groups, "per_level": per_level,
                "vcycle_ms": vprof["vcycle_ms"], "vcycle_level_ms": vprof["level_ms"],
                "spmv64": spmv, "whole_solve": whole}

    # the same V-cycle in FP64, and the all-Gauss-Seidel V-cycle in both
    # precisions (the metric's "mixed vs FP64")
    fp64 = None
    smoothers = {}
    variants = []
    if mixed:
        variants.append(("fp64", 0, kw))
    if not args.no_compare and kw.get("smoother", 0) == 1:
        variants += [("gs_mixed", 1, {}), ("gs_fp64", 0, {})] if mixed else [("gs_fp64", 0, {})]
    x_fp64 = None
    for name, prec, vkw in variants:
        H = capi.DeviceAmg(A, precision=prec, rel_tol=wl["rel_tol"], n_coarsest=1000, **vkw)
        nsteps = args.steps if name == "fp64" else 2
        for _ in range(args.warmup if name == "fp64" else 1):
            solve(H)
        sts = [solve(H) for _ in range(nsteps)]
        t = max_over_ranks(statistics.mean(q["seconds"] for q in sts), dist, device)
        vp = H.profile_vcycle(reps=5)
        smoothers[name] = {"value": t, "unit": "s", "iterations": sts[-1]["nIterations"],
                           "precision": "fp32 V-cycle" if prec else "fp64",
                           "smoother": "chebyshev" if vkw.get("smoother") else "gauss-seidel",
                           "vcycle_ms": vp["vcycle_ms"], "level_ms": vp["level_ms"]}
        if name == "fp64":
            x_fp64 = x.clone()
        H.close()
    if mixed:
        f = smoothers.pop("fp64")
        rel = float(torch.linalg.vector_norm(x_head - x_fp64) / torch.linalg.vector_norm(x_fp64))
        fp64 = {"value": f["value"], "unit": "s", "iterations": f["iterations"],
                "speedup_mixed_vs_fp64": f["value"] / per_solve,
                "mixed_solution_rel_diff_vs_fp64": rel,
                "fp64_pinned_by": "the FP64 GPU AMG-PCG matches the oracle at full 128^3 (c2, "
                                  "+-1 iteration, solution within 1e-10 at relTol 1e-13) in "
                                  "tests/test_gpu_fullsize.py",
                "vcycle_ms": f["vcycle_ms"]}
    smoothers["headline"] = {"value": per_solve, "unit": "s", "iterations": iters,
                             "precision": "fp32 V-cycle" if mixed else "fp64",
                             "smoother": "chebyshev" if kw.get("smoother") else "gauss-seidel",
                             "vcycle_ms": vprof["vcycle_ms"], "level_ms": vprof["level_ms"]}
    gpu_iters64 = fp64["iterations"] if fp64 else iters
    G.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = oracle_amg_sample(s, wl, gpu_iters64)
        except Exception as e:  # reported, never fatal
            cpu = {"value": None, "unit": "s", "cores": 1, "kind": "port",
                   "sample": f"failed: {e}"}
    matrix_bytes = A.info()["device_bytes"]
    A.close()
    del b, x, x_head, x_fp64
    torch.cuda.empty_cache()

    configs = None
    if rank == 0 and world == 1 and not args.no_configs and args.workload == "c4":
        configs = {}
        for name in ("c1", "c2", "c3"):
            try:
                configs[name] = config_block(name, args.steps, args.warmup,
                                             cpu=not args.no_cpu_baseline)
            except Exception as e:  # reported in the line, never fatal
                configs[name] = {"error": str(e)}
            torch.cuda.empty_cache()

    serving = None
    if args.serve > 0 and rank == 0 and world == 1:
        try:
            serving = serve_bench(args.serve, seed=rank, max_slots=args.serve_slots)
        except Exception as e:  # reported in the line, never fatal
            serving = {"error": str(e)}

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
        "dtype": "f64 outer PCG + f32 V-cycle" if mixed else "f64",
        "data": "synthetic (seeded generator; the reference ships no data sets)",
        "config": {"workload": f"{args.workload}: {wl['desc']}", "cells": s.n, "faces": s.nf,
                   "levels": info["n_levels"], "level_cells": info["cells"],
                   "coarsest": info["cells"][-1], "iterations": iters,
                   "true_relative_residual": true_rel, "vcycle": kw,
                   "l2": f"inputs larger than L2: matrix {matrix_bytes / 1e9:.2f} GB on device "
                         f"> {L2_BYTES / 1e6:.0f} MB",
                   "setup_s": info["setup_s"], "wall_s_per_step": t_wall / args.steps,
                   "parallelism": f"replicas x{world}"},
        "fp64": fp64,
        "smoothers": smoothers,
        "configs": configs,
        "serving": serving,
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": 2 * 8 * s.n,
                "d2h_bytes_per_step": 8 * s.n},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
