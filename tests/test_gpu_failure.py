"""Failure detection without a GPU fault.

The persistent executor's grid barriers wait with an iteration bound; when a
bound runs out the launch unwinds and reports a timeout status instead of
hanging.  The self-test makes a wait run out on purpose (one CTA sleeps in a
bounded loop past a tiny bound) and checks the status and that the context
still runs the next launch.  Solver-level failures are reported as status
and flags: a singular system stops with `singular`, an exhausted iteration
budget returns converged = 0, bad handles and sizes are errors.
"""
import ctypes

import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_barrier_wait_bound_reports_timeout(cuda):
    t = ctypes.c_int(-1)
    r = ctypes.c_int(-1)
    capi.check(capi.load().unap_cuda_selftest_barrier_timeout(ctypes.byref(t), ctypes.byref(r)))
    assert t.value == 1
    assert r.value == 1


def test_singular_system_is_reported(cuda, executor):
    torch = cuda
    # zero right-hand side: w.r = 0 at the first iteration (PCG.cpp:107-117)
    s = W.laplace(6, seed=1, shift=1.0)
    A = capi.DeviceMatrix(s)
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    st = A.krylov_solve(0, 2, x, torch.zeros(s.n, dtype=torch.float64, device="cuda"))
    assert st["singular"] == 1 and st["nIterations"] == 0
    assert not torch.isnan(x).any()
    A.close()


def test_iteration_budget_exhausted(cuda, executor):
    torch = cuda
    s = W.lognormal(10, seed=2)
    A = capi.DeviceMatrix(s)
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    st = A.krylov_solve(0, 0, x, torch.tensor(s.b, device="cuda"), rel_tol=1e-14, max_iter=5)
    assert st["nIterations"] == 5 and st["converged"] == 0
    A.close()


def test_nan_input_does_not_hang(cuda, executor):
    torch = cuda
    s = W.laplace(6, seed=3)
    b = s.b.copy()
    b[3] = np.nan
    A = capi.DeviceMatrix(s)
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    st = A.krylov_solve(0, 2, x, torch.tensor(b, device="cuda"), rel_tol=1e-8, max_iter=50)
    # NaN fails every comparison: singular (|w.r| > SMALL is false)
    assert st["singular"] == 1 or st["converged"] == 0
    A.close()


def test_size_mismatch_is_an_error(cuda):
    s = W.laplace(4, seed=4)
    h = capi.ldumatrixcreat(s)
    x = np.zeros(s.n + 1)
    lib = capi.load()
    it = ctypes.c_int(0)
    res = ctypes.c_double(0)
    n = ctypes.c_int(s.n + 1)
    b = np.zeros(s.n + 1)
    lib.pcgsolversolve_(x.ctypes.data_as(capi._dp), ctypes.byref(ctypes.c_long(h)),
                        b.ctypes.data_as(capi._dp), ctypes.byref(n), ctypes.byref(ctypes.c_int(2)),
                        ctypes.byref(ctypes.c_double(0)), ctypes.byref(ctypes.c_double(1e-6)),
                        ctypes.byref(ctypes.c_int(10)), ctypes.byref(ctypes.c_int(0)),
                        ctypes.byref(it), ctypes.byref(res))
    assert it.value == -1 and np.isnan(res.value)
