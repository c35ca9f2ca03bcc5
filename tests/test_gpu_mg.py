"""GPU parity of the reference MGSolver (V-cycle iteration) against the
oracle: same hierarchy (the reference's agglomeration and stop rule),
iteration count within +-1, final residual agreement, and the C ABI's
mgsolversolve_ / handle calls."""
import ctypes

import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def weights(s):
    return np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))


CASES = [
    lambda: W.laplace(10, 9, 8, seed=21, permute=True, rhs="normal"),
    lambda: W.lognormal(10, seed=22, permute=True, sigma=1.0),
    lambda: W.convdiff(9, 8, 7, seed=23, permute=True, pe=2.0),
]


@pytest.mark.parametrize("smoother", [1, 2])
@pytest.mark.parametrize("opts", [dict(), dict(n_pre=2), dict(scale_corr=0)])
def test_mg_parity(cuda, orc, smoother, opts):
    torch = cuda
    for make in CASES:
        s = make()
        w = weights(s)
        A = capi.DeviceMatrix(s)
        G = capi.DeviceMG(A, weights=w, smoother=smoother, n_coarsest=12, rel_tol=1e-8,
                          max_iter=60, **opts)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, torch.tensor(s.b, device="cuda"))
        x_ref, st_ref = orc.mg(s, s.b, w, n_coarsest=12, smoother=smoother, rel_tol=1e-8,
                               max_iter=60, **opts)
        assert len(G.levels()) - 1 == st_ref["n_levels"], s.name
        assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (s.name, st, st_ref)
        assert st["converged"] == st_ref["converged"]
        assert np.isclose(st["initialResidual"], st_ref["init_res"], rtol=1e-12)
        if st["converged"]:
            d = orc.spmv(s, x.cpu().numpy() - x_ref)
            assert np.linalg.norm(d) <= 2.2e-8 * st_ref["init_res"], s.name
        G.close()
        A.close()


def test_mgsolversolve_oneshot(cuda, orc):
    s = W.laplace(8, 7, 6, seed=24, permute=True, rhs="normal")
    h = capi.ldumatrixcreat(s)
    lib = capi.load()
    x = np.zeros(s.n)
    b = np.ascontiguousarray(s.b)
    it = ctypes.c_int(0)
    res = ctypes.c_double(0)
    args = [ctypes.c_int(v) for v in (s.n, 1, 1)]
    lib.mgsolversolve_(x.ctypes.data_as(capi._dp), ctypes.byref(ctypes.c_long(h)),
                       b.ctypes.data_as(capi._dp), ctypes.byref(args[0]),
                       ctypes.byref(args[1]), ctypes.byref(args[2]),
                       ctypes.byref(ctypes.c_double(0.0)), ctypes.byref(ctypes.c_double(1e-8)),
                       ctypes.byref(ctypes.c_int(100)), ctypes.byref(ctypes.c_int(0)),
                       ctypes.byref(it), ctypes.byref(res), None)
    x_ref, st = orc.mg(s, s.b, weights(s), smoother=1, n_pre=0, rel_tol=1e-8, max_iter=100)
    assert abs(it.value - st["n_iter"]) <= 1
    assert np.isclose(res.value, st["final_res"], rtol=1e-3)


def test_mg_handle_api(cuda, orc):
    s = W.lognormal(8, seed=25, permute=True, sigma=1.0)
    lib = capi.load()
    A = ctypes.c_long(capi.ldumatrixcreat(s))
    mg = ctypes.c_long(0)
    agg = ctypes.c_long(0)
    w = weights(s)
    lib.contruct_solver_mg__(ctypes.byref(mg), ctypes.byref(A), ctypes.byref(agg),
                             w.ctypes.data_as(capi._dp), ctypes.byref(ctypes.c_int(2)),
                             ctypes.byref(ctypes.c_int(50)), ctypes.byref(ctypes.c_int(10)))
    assert mg.value != 0
    lib.sw_solver_mg_set_reltol__(ctypes.byref(mg), ctypes.byref(ctypes.c_double(1e-8)))
    lib.sw_solver_mg_set_maxiter__(ctypes.byref(mg), ctypes.byref(ctypes.c_int(80)))
    for _ in range(2):  # initSmoothers before each solve: same answer twice
        x = np.zeros(s.n)
        res = ctypes.c_double(0)
        lib.sw_solve_mg__(ctypes.byref(mg), ctypes.byref(A), x.ctypes.data_as(capi._dp),
                          np.ascontiguousarray(s.b).ctypes.data_as(capi._dp), ctypes.byref(res))
        assert res.value <= 1e-8 * np.linalg.norm(s.b) * 1.01
    x_ref, st = orc.mg(s, s.b, w, n_coarsest=10, smoother=2, rel_tol=1e-8, max_iter=80)
    assert np.linalg.norm(orc.spmv(s, x - x_ref)) <= 2.2e-8 * st["init_res"]
    lib.sw_solver_destroy_mg__(ctypes.byref(mg))
    lib.sw_matrix_destroy__(ctypes.byref(A))
