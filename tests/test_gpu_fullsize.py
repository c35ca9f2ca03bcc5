"""The benchmark configurations at their full sizes.

Where the oracle is linear in the matrix size it runs at full size too, so
those kernels are checked bit for bit (SpMV, DIC/DILU application,
Gauss-Seidel sweeps, one AMG V-cycle at 128^3); the solves are checked
through properties that hold at any size: convergence to the stated
tolerance in the true residual (b - A x computed by the oracle's SpMV), the
same iteration count and the same solution bits from the device and host
structure builds, and mixed precision agreeing with FP64.

c1  32^3 natural-order Laplacian, PCG+DIC, tol 1e-8 (also solved by the oracle)
c2  128^3 permuted Laplacian, FP64 AMG-PCG, tol 1e-10 (also solved by the oracle)
c3  200^3 permuted convection-diffusion Pe=5, PBiCGStab+DILU, tol 1e-9
c4  256^3 permuted log-normal (sigma 2) Poisson, mixed vs FP64 AMG-PCG, tol 1e-10
"""
import numpy as np
import pytest

from oracle_lib import OracleAmg
from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def true_rel(orc, s, x):
    return np.linalg.norm(s.b - orc.spmv(s, x)) / np.linalg.norm(s.b)


def test_c1_full_parity(cuda, orc):
    torch = cuda
    s = W.config("c1")
    A = capi.DeviceMatrix(s)
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    st = A.krylov_solve(0, 2, x, dev(torch, s.b), rel_tol=1e-8, max_iter=1000)
    x_ref, st_ref = orc.pcg(s, 2, s.b, rel_tol=1e-8, max_iter=1000)
    assert st["converged"] and abs(st["nIterations"] - st_ref["n_iter"]) <= 1
    xg = x.cpu().numpy()
    assert np.linalg.norm(orc.spmv(s, xg - x_ref)) <= 2.2e-8 * st_ref["init_res"]
    assert true_rel(orc, s, xg) <= 1.0001e-8
    A.close()


def test_c2_full(cuda, orc):
    torch = cuda
    s = W.config("c2")
    A = capi.DeviceMatrix(s)
    rng = np.random.default_rng(2)
    v = rng.standard_normal(s.n)
    y = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    A.spmv(dev(torch, v), y)
    assert np.array_equal(y.cpu().numpy(), orc.spmv(s, v))
    xg = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    A.gauss_seidel(xg, dev(torch, s.b), 2)
    assert np.array_equal(xg.cpu().numpy(), orc.gs(s, np.zeros(s.n), s.b, 2))
    G = capi.DeviceAmg(A, n_coarsest=1000, precision=0, rel_tol=1e-10)
    O = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=1e-10)
    assert G.info()["cells"] == O.level_sizes()
    z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    G.vcycle(dev(torch, v), z)
    assert np.array_equal(z.cpu().numpy(), O.vcycle(v))
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    st = G.solve(x, dev(torch, s.b))
    assert st["converged"]
    xg = x.cpu().numpy()
    x64 = xg.copy()  # the FP64 GPU solve at relTol 1e-10
    assert true_rel(orc, s, xg) <= 1.0001e-10
    # the oracle's own FP64 AMG-PCG at full size: the same iteration count
    # +-1 and agreement in residual space at relTol 1e-10, and solutions
    # within 1e-10 relative 2-norm at relTol 1e-13
    x_ref, st_ref = O.solve(s.b)
    assert st_ref["converged"] and abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (st, st_ref)
    assert np.linalg.norm(orc.spmv(s, xg - x_ref)) <= 2.2e-10 * st_ref["init_res"]
    O.close()
    G.close()
    G = capi.DeviceAmg(A, n_coarsest=1000, precision=0, rel_tol=1e-13)
    O = OracleAmg(orc, s, n_coarsest=1000, precision=0, rel_tol=1e-13)
    x.zero_()
    st = G.solve(x, dev(torch, s.b))
    x_ref, st_ref = O.solve(s.b)
    assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (st, st_ref)
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - x_ref) <= 1e-10 * np.linalg.norm(x_ref)
    O.close()
    G.close()
    # the mixed-precision solve (FP32 V-cycle, FP64 outer PCG, the
    # benchmark's smoothers) against the FP64 oracle's solution (relTol
    # 1e-13): at relTol 1e-10 its error is the convergence tolerance's, as
    # large as the FP64 solve's at the same tolerance and not more
    G = capi.DeviceAmg(A, n_coarsest=1000, precision=1, rel_tol=1e-10, smoother=1,
                       cheby_degree=3, cheby_from=2, eig_ratio=60.0, n_pre=1, n_post=1)
    x.zero_()
    st = G.solve(x, dev(torch, s.b))
    assert st["converged"]
    xm = x.cpu().numpy()
    assert true_rel(orc, s, xm) <= 1.0001e-10
    nref = np.linalg.norm(x_ref)
    err_mixed = np.linalg.norm(xm - x_ref) / nref
    err_fp64 = np.linalg.norm(x64 - x_ref) / nref
    print(f"c2 error against the FP64 oracle: mixed {err_mixed:.3e}, FP64 {err_fp64:.3e}")
    assert err_mixed <= 10 * err_fp64 + 1e-12, (err_mixed, err_fp64)
    G.close()
    A.close()


def test_c3_full(cuda, orc):
    torch = cuda
    s = W.config("c3")
    A = capi.DeviceMatrix(s)
    rng = np.random.default_rng(3)
    r = rng.standard_normal(s.n)
    w = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    A.precondition(3, dev(torch, r), w)
    assert np.array_equal(w.cpu().numpy(), orc.precond(3, s, r)[0])
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    st = A.krylov_solve(1, 3, x, dev(torch, s.b), rel_tol=1e-9, max_iter=2000)
    assert st["converged"]
    assert true_rel(orc, s, x.cpu().numpy()) <= 1.0001e-9
    A.close()


def test_c4_full(cuda, orc):
    torch = cuda
    s = W.config("c4")
    b = dev(torch, s.b)
    A = capi.DeviceMatrix(s)
    rng = np.random.default_rng(4)
    v = rng.standard_normal(s.n)
    y = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    A.spmv(dev(torch, v), y)
    assert np.array_equal(y.cpu().numpy(), orc.spmv(s, v))
    w = torch.zeros_like(y)
    A.precondition(2, dev(torch, v), w)
    assert np.array_equal(w.cpu().numpy(), orc.precond(2, s, v)[0])
    sols = {}
    for prec in (1, 0):
        G = capi.DeviceAmg(A, n_coarsest=1000, precision=prec, rel_tol=1e-10)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, b)
        assert st["converged"], (prec, st)
        xh = x.cpu().numpy()
        assert true_rel(orc, s, xh) <= 1.0001e-10, prec
        sols[prec] = (st["nIterations"], xh)
        G.close()
    # both meet the same 1e-10 residual; the log-normal matrix's condition
    # number lets the solutions differ by far less than 1e-6
    d = np.linalg.norm(sols[1][1] - sols[0][1]) / np.linalg.norm(sols[0][1])
    assert d <= 1e-6, d
    assert abs(sols[1][0] - sols[0][0]) <= 5, (sols[1][0], sols[0][0])
    A.close()


def test_c4_headline_vcycle(cuda, orc):
    """The benchmark's V-cycle (Gauss-Seidel 1/1 on levels 0-1, Chebyshev
    degree 3 on [lambda/60, 1.1 lambda] below) at full 256^3: the mixed and
    FP64 solves both reach a 1e-10 true relative residual (b - A x by the
    oracle's SpMV) and agree within 1e-8."""
    torch = cuda
    s = W.config("c4")
    b = dev(torch, s.b)
    A = capi.DeviceMatrix(s)
    kw = dict(smoother=1, cheby_degree=3, cheby_from=2, eig_ratio=60.0, n_pre=1, n_post=1)
    sols = {}
    for prec in (1, 0):
        G = capi.DeviceAmg(A, n_coarsest=1000, precision=prec, rel_tol=1e-10, **kw)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, b)
        assert st["converged"], (prec, st)
        xh = x.cpu().numpy()
        assert true_rel(orc, s, xh) <= 1.0001e-10, prec
        sols[prec] = (st["nIterations"], xh)
        G.close()
    d = np.linalg.norm(sols[1][1] - sols[0][1]) / np.linalg.norm(sols[0][1])
    assert d <= 1e-8, d
    assert abs(sols[1][0] - sols[0][0]) <= 3, (sols[1][0], sols[0][0])
    A.close()
