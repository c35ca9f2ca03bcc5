"""The continuous-batching solve server: requests that arrive while others
are on the GPU are admitted as slots and memory free up, small ones are
batched into one launch, and every result is the same as the same solve run
alone (within the solver tolerance: +-1 iteration, 2.2 relTol ||r0|| in
residual space), including under a memory budget that forces queueing."""
import threading
import time

import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def alone(torch, s, method, rel_tol):
    """The same solve outside the server, with the server's method: AMG
    requests on a matrix without wavefronts, Chebyshev degree 3 on every
    level ([lambda/30, 1.1 lambda]), coarsest level of 200 cells."""
    amg = method in ("amg_mixed", "amg_fp64")
    old = capi.set_matrix_wavefronts(not amg)
    try:
        A = capi.DeviceMatrix(s)
    finally:
        capi.set_matrix_wavefronts(old)
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    b = torch.tensor(s.b, device="cuda")
    if amg:
        G = capi.DeviceAmg(A, precision=1 if method == "amg_mixed" else 0, rel_tol=rel_tol,
                           max_iter=1000, n_coarsest=200, smoother=1, cheby_degree=3,
                           cheby_from=0, eig_ratio=30.0)
        st = G.solve(x, b)
        G.close()
    else:
        st = A.krylov_solve(0 if method == "pcg_dic" else 1, 2 if method == "pcg_dic" else 3,
                            x, b, rel_tol=rel_tol, max_iter=1000)
    A.close()
    return x.cpu().numpy(), st


@pytest.mark.parametrize("budget", [0, 40 << 20])
def test_results_same_alone_and_in_the_mix(cuda, orc, budget):
    torch = cuda
    reqs = W.serving_requests(count=14, rate=400.0, min_cells=2_000, max_cells=120_000, seed=3)
    srv = capi.Server(memory_budget=budget, max_slots=3, small_cells=20_000)
    ids = {}
    lock = threading.Lock()

    def client():
        t0 = time.perf_counter()
        for i, r in enumerate(reqs):
            dt = r.arrival - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            rid = srv.submit(r.system, r.method, rel_tol=1e-8)
            with lock:
                ids[i] = rid

    th = threading.Thread(target=client)
    th.start()
    th.join()
    batched = 0
    for i, r in enumerate(reqs):
        x, info = srv.wait(ids[i], r.system.n)
        assert info["status"] == 0 and info["converged"], (r.method, info)
        batched += info["batched"]
        xa, sta = alone(torch, r.system, r.method, 1e-8)
        assert abs(info["nIterations"] - sta["nIterations"]) <= 1, (r.method, info, sta)
        d = orc.spmv(r.system, x - xa)
        assert np.linalg.norm(d) <= 2.2e-8 * sta["initialResidual"], r.method
        assert info["latencySeconds"] >= info["solveSeconds"] >= 0
    assert batched >= 1
    srv.close()
