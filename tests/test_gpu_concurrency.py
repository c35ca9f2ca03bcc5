"""Device-pointer solves from several host threads at once.

Each thread owns its matrix (and so its stream), fills its initial guess on
the default stream and calls the solver right away: the call must order
itself after that fill (the initial residual is ||b||, not the residual of
the previous solution), and every solve must match the same solve done
alone.
"""
import threading

import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _run_threads(fn, n):
    errors = []

    def wrap(i):
        try:
            fn(i)
        except Exception as e:  # reported in the main thread
            errors.append(e)

    th = [threading.Thread(target=wrap, args=(i,)) for i in range(n)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    if errors:
        raise errors[0]


def test_concurrent_amg_solves_match_alone(cuda):
    torch = cuda
    N = 8
    systems = [W.lognormal(30, 28, 26, seed=200 + i, permute=True, sigma=2.0) for i in range(N)]
    old = capi.set_matrix_wavefronts(False)
    try:
        mats = [capi.DeviceMatrix(s) for s in systems]
    finally:
        capi.set_matrix_wavefronts(old)
    amgs = [capi.DeviceAmg(A, precision=1, rel_tol=1e-8, max_iter=300, smoother=1,
                           cheby_degree=3, cheby_from=0, eig_ratio=30.0) for A in mats]
    bs = [torch.tensor(s.b, device="cuda") for s in systems]
    xs = [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s in systems]
    alone = []
    for G, x, b in zip(amgs, xs, bs):
        x.fill_(1.0)
        x.zero_()
        alone.append((G.solve(x, b), x.cpu().numpy().copy()))
    out = [None] * N

    def work(i):
        res = []
        for _ in range(3):
            xs[i].fill_(1.0)  # a stale guess the solve must not see
            xs[i].zero_()
            st = amgs[i].solve(xs[i], bs[i])
            res.append((st, xs[i].cpu().numpy().copy()))
        out[i] = res

    _run_threads(work, N)
    for i in range(N):
        st0, x0 = alone[i]
        assert st0["converged"]
        assert np.isclose(st0["initialResidual"], np.linalg.norm(systems[i].b), rtol=1e-12)
        for st, x in out[i]:
            assert st["converged"], (i, st)
            assert st["initialResidual"] == st0["initialResidual"], (i, st, st0)
            assert st["nIterations"] == st0["nIterations"], (i, st, st0)
            assert np.array_equal(x, x0), i
    for G in amgs:
        G.close()
    for A in mats:
        A.close()


def test_concurrent_krylov_solves_match_alone(cuda):
    torch = cuda
    N = 6
    systems = [W.laplace(40, 38, 36, seed=300 + i, permute=True, rhs="normal", shift=0.1)
               for i in range(N)]
    mats = [capi.DeviceMatrix(s) for s in systems]
    bs = [torch.tensor(s.b, device="cuda") for s in systems]
    xs = [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s in systems]
    alone = []
    for A, x, b in zip(mats, xs, bs):
        x.zero_()
        alone.append(A.krylov_solve(0, 2, x, b, rel_tol=1e-9, max_iter=2000))
    out = [None] * N

    def work(i):
        res = []
        for _ in range(2):
            xs[i].fill_(1.0)
            xs[i].zero_()
            res.append(mats[i].krylov_solve(0, 2, xs[i], bs[i], rel_tol=1e-9, max_iter=2000))
        out[i] = res

    _run_threads(work, N)
    for i in range(N):
        for st in out[i]:
            assert st["converged"], (i, st)
            assert st["initialResidual"] == alone[i]["initialResidual"], (i, st, alone[i])
            assert st["nIterations"] == alone[i]["nIterations"], (i, st, alone[i])
    for A in mats:
        A.close()
