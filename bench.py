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

A 1-GPU run also serves the seeded 200-request stream of config c5
(`serving`: solves/s and p50/p99 latency beside the one-at-a-time FP64
path; `--serve 0` skips it).

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
# DRAM bytes / algorithmic bytes of a whole FP32 Gauss-Seidel sweep, measured
# in situ (no cache flush) with ncu on the 192^3 log-normal matrix
SWEEP_TRAFFIC_RATIO = 1.29
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
    # The GPU path's FP64 iteration count is not known here, and a full
    # solve at 256^3 takes the oracle about 20 minutes: the warm-up measures
    # the convergence rate between the residuals after 1 and 6 iterations
    # (at 128^3 it predicts 51 iterations to 1e-10 where the solve takes
    # 53), the timed steps the time per iteration, and each sample is scaled
    # to the iterations that rate needs.
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle, OracleAmg
    orc = Oracle("orc")
    samples = []
    # the hierarchy is built once, outside the timed samples (as the GPU arm's)
    O = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=1e-10, max_iter=1)
    _, s1 = O.solve(s.b)
    O.set_max_iter(6)
    _, s6 = O.solve(s.b)
    iters_needed = s6["n_iter"]
    if not s6["converged"] and s1["n_iter"] == 1 and s6["n_iter"] == 6:
        rate = (s6["final_res"] / s1["final_res"]) ** 0.2
        if 0 < rate < 1:
            more = np.log(1e-10 * s6["init_res"] / s6["final_res"]) / np.log(rate)
            iters_needed = 6 + max(0, int(np.ceil(more)))
    O.set_max_iter(args.ref_iters)
    for step in range(max(args.warmup - 2, 0) + args.steps):
        t0 = time.perf_counter()
        _, st = O.solve(s.b)
        dt = time.perf_counter() - t0
        if step >= args.warmup - 2:
            samples.append(dt / st["n_iter"] * iters_needed)
    O.close()
    value = statistics.mean(samples)
    line = {"impl": "reference", "metric": "amg_pcg_time_to_1e-10", "value": value, "unit": "s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{args.workload}: {wl['desc']} (CPU: FP64 V-cycle)",
                       "cells": s.n, "faces": s.nf},
            "cpu_baseline": {"value": value, "unit": "s", "cores": 1, "kind": "port",
                             "sample": (f"each step: oracle FP64 AMG-PCG, {args.ref_iters} PCG "
                                        f"iteration(s) timed, scaled to the {iters_needed} "
                                        f"iterations to 1e-10 that its convergence rate "
                                        f"between iterations 1 and 6 gives; hierarchy setup "
                                        f"untimed")},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def serve_bench(n_requests: int, seed: int = 0, max_slots: int = 4, compare_plain: bool = True):
    """Config c5 served: a seeded Poisson request stream (200 req/s, sizes
    log-uniform 8k-2M cells, 60% mixed AMG-PCG / 25% PCG+DIC / 15%
    PBiCGStab+DILU, tol 1e-8) submitted on its arrival schedule to the
    continuous-batching server, then the same requests one at a time with
    the plain FP64 path (FP64 AMG-PCG instead of mixed) on the same GPU.
    Latency = completion - scheduled arrival."""
    import torch
    from unap_gb300 import capi
    from unap_gb300 import workloads as W

    reqs = W.serving_requests(count=n_requests, rate=200.0, seed=seed)
    srv = capi.Server(max_slots=max_slots)
    t0 = time.perf_counter()
    ids = []
    for r in reqs:
        dt = r.arrival - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(r.system, r.method, rel_tol=1e-8, max_iter=2000))
    lat, batched, setup, solve_t, queue = [], 0, [], [], []
    for r, rid in zip(reqs, ids):
        _, info = srv.wait(rid, r.system.n)
        if not info["converged"]:
            raise RuntimeError(f"served request did not converge: {info}")
        lat.append(info["latencySeconds"])
        setup.append(info["setupSeconds"])
        solve_t.append(info["solveSeconds"])
        queue.append(info["queueSeconds"])
        batched += info["batched"]
    span = time.perf_counter() - t0
    srv.close()

    pct = lambda v, q: float(np.percentile(np.array(v), q))
    out = {"requests": n_requests, "rate_per_s": 200.0,
           "solves_per_s": n_requests / span, "p50_s": pct(lat, 50), "p99_s": pct(lat, 99),
           "batched_requests": batched, "slots": max_slots,
           "mean_queue_s": float(np.mean(queue)), "mean_setup_s": float(np.mean(setup)),
           "mean_solve_s": float(np.mean(solve_t))}
    if not compare_plain:
        return out
    # the plain path: one request at a time, FP64 everywhere
    seq_lat = []
    t1 = time.perf_counter()
    for r in reqs:
        ts = time.perf_counter()
        s = r.system
        A = capi.DeviceMatrix(s)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        b = torch.tensor(s.b, device="cuda")
        if r.method == "amg_mixed":
            G = capi.DeviceAmg(A, precision=0, rel_tol=1e-8, max_iter=2000)
            G.solve(x, b)
            G.close()
        else:
            A.krylov_solve(0 if r.method == "pcg_dic" else 1, 2 if r.method == "pcg_dic" else 3,
                           x, b, rel_tol=1e-8, max_iter=2000)
        _ = x.cpu()
        A.close()
        seq_lat.append(time.perf_counter() - ts)
    seq_span = time.perf_counter() - t1
    out["one_at_a_time_fp64"] = {"solves_per_s": n_requests / seq_span,
                                 "p50_s": pct(seq_lat, 50), "p99_s": pct(seq_lat, 99),
                                 "latency": "solve time alone, no queueing"}
    return out


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c4", choices=sorted(WORKLOADS))
    ap.add_argument("--scale", type=float, default=1.0, help="grid edge scale (testing)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-iters", type=int, default=1,
                    help="PCG iterations per reference-arm sample")
    ap.add_argument("--serve", type=int, default=200,
                    help="also serve this many requests of the c5 stream (rank 0 of a "
                         "1-GPU run; 0: skip)")
    ap.add_argument("--serve-slots", type=int, default=12,
                    help="concurrent large-request slots of the server")
    ap.add_argument("--kernels", action="store_true",
                    help="only time the finest-level kernels one launch at a time "
                         "(the small case for kernel profiles) and exit")
    ap.add_argument("--reps", type=int, default=5, help="repetitions for --kernels")
    ap.add_argument("--profile-solve", action="store_true",
                    help="bracket one extra mixed solve after the timed ones (with --setup: "
                         "the device setup) with cudaProfilerStart/Stop, for ncu "
                         "--profile-from-start off")
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
    tail_rows, single_rows = capi.get_tail_rows(wl["precision"])
    tail_info = {"cluster_ctas": capi.tail_cluster_size(), "tail_rows": tail_rows,
                 "single_cta_rows": single_rows,
                 "levels_in_tail": sum(1 for c in info["cells"][:-1] if c <= tail_rows)}
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

    # FP64 AMG-PCG on the same matrix (the metric's "mixed vs FP64")
    fp64 = None
    if G64 is not G:
        x_mixed = x.clone()
        for _ in range(args.warmup):
            solve(G64)
        st64 = [solve(G64) for _ in range(args.steps)]
        t64 = max_over_ranks(statistics.mean(st["seconds"] for st in st64), dist, device)
        # the mixed solution against the FP64 one (both to a 1e-10 residual)
        rel = float(torch.linalg.vector_norm(x_mixed - x) / torch.linalg.vector_norm(x))
        fp64 = {"value": t64, "unit": "s", "iterations": st64[-1]["nIterations"],
                "speedup_mixed_vs_fp64": t64 / per_solve,
                "mixed_solution_rel_diff_vs_fp64": rel}
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

    # roofline of the dominant kernel: the FP32 (FP64) Gauss-Seidel sweep of
    # the finest level, all wavefront launches of one sweep timed with CUDA
    # events on the matrix's stream.  The whole solve's algorithmic bytes
    # (the library's per-step bookkeeping) over its device time are reported
    # beside it, with the FP64 SpMV.
    prof = A.profile(reps=10)
    peak, peak_kind = hbm_peak()
    peak_src = ("measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s")
    mixed = wl["precision"] == 1
    sweep_bytes = gs32_sweep_bytes(s.n, s.nf) if mixed else 32 * s.n + 16 * s.nf
    sweep_ms = prof["gs_fwd32"] if mixed else prof["gs_fwd"]
    achieved = sweep_bytes / (sweep_ms * 1e-3) / 1e9
    spmv = {"kernel": "spmv_kernel<double>", "ms": prof["spmv"],
            "achieved": spmv64_bytes(s.n, s.nf) / (prof["spmv"] * 1e-3) / 1e9}
    solve_bytes = stats[-1].get("algorithmicBytes", 0.0)
    whole = None
    if solve_bytes > 0:
        whole = {"algorithmic_bytes": solve_bytes, "s": statistics.mean(dev_s),
                 "achieved": solve_bytes / statistics.mean(dev_s) / 1e9}
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": SWEEP_TRAFFIC_RATIO * sweep_bytes if mixed else None,
                "traffic_source": "in-situ DRAM bytes of a whole FP32 sweep measured by ncu "
                                  "on the 192^3 case (profiles/gs_kernel_float_c4_192cube_"
                                  "waves.md), ratio 1.29 to algorithmic, scaled to this sweep"
                                  if mixed else None,
                "kernel": "gs_kernel<float>" if mixed else "gs_kernel<double>",
                "launch_group": f"one forward sweep of the finest level "
                                f"({A.info()['n_wavefronts']} wavefront launches)",
                "algorithmic_bytes_per_sweep": sweep_bytes, "sweep_ms": sweep_ms,
                "peak_source": peak_src, "spmv64": spmv, "whole_solve": whole}

    # the kernels with the largest share of device time: the V-cycle's
    # sweeps on levels 1..L-1 (row-packed, one launch per wavefront; the
    # smallest levels run in the one-CTA tail), from the per-level profile
    # of a graph-captured V-cycle; algorithmic bytes per level = 4 sweeps and
    # one residual of (16 N + 12 F) for FP32 rows (8 x 4 bytes for FP64)
    prof = G.profile_vcycle(reps=10)
    lsz = G.level_sizes()
    lvl_ms = prof["level_ms"]
    cb, fb = (16.0, 12.0) if mixed else (32.0, 16.0)
    coarse_bytes = sum(5 * (cb * n + fb * f) for (n, f, _) in lsz[1:-1])
    coarse_ms = sum(lvl_ms[1:len(lsz) - 1]) + (lvl_ms[len(lsz) - 1] if len(lvl_ms) >= len(lsz)
                                               else 0.0)
    coarse_gbs = coarse_bytes / (coarse_ms * 1e-3) / 1e9 if coarse_ms > 0 else None
    roofline["coarse_levels"] = {
        "kernel": "gs_packed_kernel<float>" if mixed else "gs_packed_kernel<double>",
        "levels": f"1-{len(lsz) - 1} (with the coarsest dense solve)",
        "share_of_vcycle": coarse_ms / prof["vcycle_ms"] if prof["vcycle_ms"] else None,
        "vcycle_ms": prof["vcycle_ms"], "level_ms": lvl_ms[:len(lsz)],
        "wavefronts_per_level": [w for (_, _, w) in lsz],
        "algorithmic_bytes": coarse_bytes, "ms": coarse_ms,
        "achieved": coarse_gbs, "unit": "GB/s",
        "frac": coarse_gbs / peak if coarse_gbs else None,
        "bound": "latency: one dependent launch per wavefront (about 2,000 per V-cycle)"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(s, gpu_iters64)
        except Exception as e:  # reported, never fatal
            cpu = {"value": None, "unit": "s", "cores": 1, "kind": "port",
                   "sample": f"failed: {e}"}

    serving = None
    if args.serve > 0 and rank == 0 and world == 1:
        try:
            serving = serve_bench(args.serve, seed=rank, max_slots=args.serve_slots)
        except Exception as e:  # reported in the line, never fatal
            serving = {"error": str(e)}

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
                   "vcycle_tail": tail_info,
                   "parallelism": f"replicas x{world}"},
        "fp64": fp64,
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
    G.close()
    if G64 is not G:
        G64.close()
    A.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
