"""GPU parity of the Chebyshev-smoothed AMG V-cycle and AMG-PCG against the
oracle (the smoother of chebySmoother.cpp:44-148 on every level from
chebyFrom down, its eigenvalue estimate of eigenDiagPCG.cpp:11-361 taken
once at setup).

* The per-level eigenvalue estimates agree with the oracle's to within the
  bisection band of the Sturm search (1e-5): the diagonal-PCG dot products
  sum in a different order on the device, which moves the Lanczos matrix in
  the last bits only.
* With the device's estimates given to the oracle, one V-cycle is
  bit-identical to the oracle's in FP64 and FP32, for several degrees and
  first Chebyshev levels, with and without programmatic dependent launch,
  and whatever CTA size the step launches use.
* AMG-PCG with the Chebyshev V-cycle matches the oracle's iteration count
  within +-1 and reaches the true relative residual it claims, with both
  executors; at relTol 1e-13 the FP64 solutions agree within 1e-10.
"""
import numpy as np
import pytest

from oracle_lib import OracleAmg
from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# half-width of the Sturm bisection's final band (eigenDiagPCG.cpp:259-276)
EIG_TOL = 1e-5


def spd_systems():
    return [W.lognormal(14, 12, 10, seed=5, permute=True),
            W.laplace(12, 11, 10, seed=6, permute=True, rhs="normal"),
            W.lognormal(20, seed=8, permute=True, sigma=1.0)]


def dev(torch, a):
    return torch.tensor(np.asarray(a, dtype=np.float64), device="cuda")


CASES = [dict(cheby_from=0, cheby_degree=3, eig_ratio=30.0),
         dict(cheby_from=1, cheby_degree=3, eig_ratio=30.0),
         dict(cheby_from=0, cheby_degree=2, eig_ratio=1.5),
         dict(cheby_from=2, cheby_degree=1, eig_ratio=4.0),
         dict(cheby_from=0, cheby_degree=4, eig_ratio=30.0)]


def _pair(orc, s, precision, case, **kw):
    A = capi.DeviceMatrix(s)
    G = capi.DeviceAmg(A, n_coarsest=40, precision=precision, smoother=1, **case, **kw)
    O = OracleAmg(orc, s, n_coarsest=40, precision=precision, smoother=1, flexible=precision,
                  **case, **kw)
    return A, G, O


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_cheby_eigenvalues_and_vcycle_bit_exact(cuda, orc, precision, case):
    torch = cuda
    for s in spd_systems():
        A, G, O = _pair(orc, s, precision, CASES[case])
        assert G.info()["cells"] == O.level_sizes(), s.name
        lam_g = G.eigenvalues()
        lam_o = O.eigs()
        assert lam_g.shape == lam_o.shape
        assert np.all(np.abs(lam_g - lam_o) <= EIG_TOL), (s.name, lam_g, lam_o)
        # levels above chebyFrom use Gauss-Seidel and carry no estimate
        frm = CASES[case]["cheby_from"]
        assert np.all(lam_g[:frm] == 0) and np.all(lam_g[frm:] > 0), lam_g
        O.set_eigs(lam_g)
        r = np.random.default_rng(s.n).standard_normal(s.n)
        z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        for pdl in (True, False):
            old = capi.set_wave_pdl(pdl)
            try:
                G.vcycle(dev(torch, r), z)
            finally:
                capi.set_wave_pdl(old)
            assert np.array_equal(z.cpu().numpy(), O.vcycle(r)), (s.name, precision, pdl)
        G.close()
        O.close()
        A.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", [0, 1, 4])
def test_cheby_cluster_tail_bit_exact(cuda, orc, precision, case):
    """The coarse Chebyshev levels in one cluster launch (from the first
    Chebyshev level below 1,000 rows, or from level 1): the same V-cycle
    bits as the oracle's, and the same solve as with a launch per step."""
    torch = cuda
    for rows in (1000, 1 << 30):
        old = capi.set_cheby_tail_rows(rows)
        try:
            for s in spd_systems():
                A, G, O = _pair(orc, s, precision, CASES[case])
                O.set_eigs(G.eigenvalues())
                r = np.random.default_rng(s.n).standard_normal(s.n)
                z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
                G.vcycle(dev(torch, r), z)
                assert np.array_equal(z.cpu().numpy(), O.vcycle(r)), (s.name, precision, rows)
                prof = G.profile_vcycle(reps=2)  # the tail's first level holds its time
                assert prof["vcycle_ms"] > 0 and min(prof["level_ms"]) >= 0
                G.close()
                O.close()
                A.close()
        finally:
            capi.set_cheby_tail_rows(old)
    s = W.lognormal(30, 28, 26, seed=19, permute=True)
    A = capi.DeviceMatrix(s)
    b = dev(torch, s.b)
    res = []
    for rows in (0, 5000):
        old = capi.set_cheby_tail_rows(rows)
        try:
            G = capi.DeviceAmg(A, n_coarsest=100, precision=precision, smoother=1,
                               rel_tol=1e-9, **CASES[case])
        finally:
            capi.set_cheby_tail_rows(old)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, b)
        res.append((st["nIterations"], x.cpu().numpy()))
        G.close()
    assert res[0][0] == res[1][0] and np.array_equal(res[0][1], res[1][1])
    A.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_cheby_launch_geometry_same_bits(cuda, precision):
    """One-warp or 256-thread CTAs and 8- or 16-entry load chunks for the
    Chebyshev steps: same bits."""
    torch = cuda
    s = W.lognormal(24, 20, 18, seed=11, permute=True)
    A = capi.DeviceMatrix(s)
    G = capi.DeviceAmg(A, n_coarsest=60, precision=precision, smoother=1)
    r = dev(torch, np.random.default_rng(3).standard_normal(s.n))
    out = []
    for rows, chunk in ((0, 0), (1 << 30, 0), (0, 8), (1 << 30, 16)):
        old = capi.set_cheby_small_rows(rows)
        oldc = capi.set_cheby_chunk(chunk)
        try:
            z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            G.vcycle(r, z)
            out.append(z.cpu().numpy())
        finally:
            capi.set_cheby_small_rows(old)
            capi.set_cheby_chunk(oldc)
    for o in out[1:]:
        assert np.array_equal(out[0], o)
    with pytest.raises(capi.UnapCudaError):
        capi.set_cheby_chunk(5)
    G.close()
    A.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_cheby_amg_pcg_parity(cuda, orc, precision, executor):
    torch = cuda
    for s in spd_systems():
        A, G, O = _pair(orc, s, precision, CASES[0], rel_tol=1e-10)
        O.set_eigs(G.eigenvalues())
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, dev(torch, s.b))
        x_ref, st_ref = O.solve(s.b)
        xg = x.cpu().numpy()
        assert st["converged"] and st_ref["converged"]
        assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (s.name, st, st_ref)
        assert (np.linalg.norm(orc.spmv(s, xg - x_ref))
                <= 2.2e-10 * st_ref["init_res"]), s.name
        true_rel = np.linalg.norm(s.b - orc.spmv(s, xg)) / np.linalg.norm(s.b)
        assert true_rel <= 1.0001e-10, (s.name, true_rel)
        G.close()
        O.close()
        A.close()


def test_cheby_amg_pcg_solution_tight(cuda, orc, executor):
    """FP64 Chebyshev AMG-PCG to relTol 1e-13: GPU and oracle solutions agree
    within 1e-10 relative 2-norm."""
    torch = cuda
    for s in (W.laplace(12, 11, 10, seed=6, permute=True, rhs="normal", shift=0.5),
              W.lognormal(16, seed=8, permute=True, sigma=1.0, shift=0.1)):
        A, G, O = _pair(orc, s, 0, CASES[0], rel_tol=1e-13)
        O.set_eigs(G.eigenvalues())
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, dev(torch, s.b))
        x_ref, st_ref = O.solve(s.b)
        assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (s.name, st, st_ref)
        xg = x.cpu().numpy()
        assert np.linalg.norm(xg - x_ref) <= 1e-10 * np.linalg.norm(x_ref), s.name
        G.close()
        O.close()
        A.close()


def test_cheby_rejects_bad_parameters(cuda):
    s = W.lognormal(8, seed=2, permute=True)
    A = capi.DeviceMatrix(s)
    for kw, msg in ((dict(smoother=2), "smoother"), (dict(smoother=1, cheby_degree=0), "degree"),
                    (dict(smoother=1, cheby_degree=17), "degree"),
                    (dict(smoother=1, eig_ratio=0.5), "ratio")):
        with pytest.raises(capi.UnapCudaError, match=msg):
            capi.DeviceAmg(A, **kw)
    A.close()


def test_reference_cheby_smoother_c_abi(cuda, orc):
    """chebySmoother::smooth through unap_cuda_cheby_smooth_host (the
    reference's smoother, chebySmoother.cpp:13-149): the first call's
    eigenvalue estimate (eigenDiagPCG.cpp:11-361) equals the oracle's within
    the bisection band and leaves x as the oracle's 10 diagonal-PCG
    iterations do, up to dot-product summation order (1e-12 relative); the
    next call's Chebyshev sweeps equal the oracle's chain bit for bit from
    the device's state; on symmetric and asymmetric matrices."""
    import ctypes
    lib = capi.load()
    for s in (W.lognormal(14, 12, 10, seed=5, permute=True),
              W.convdiff(10, 9, 8, seed=3, permute=True, pe=2.0),
              W.laplace(12, seed=4, permute=False, rhs="normal")):
        h = capi.ldumatrixcreat(s)
        x0 = np.random.default_rng(s.n).standard_normal(s.n)
        b = np.ascontiguousarray(s.b)
        x = x0.copy()
        lam = ctypes.c_double(0.0)
        est = ctypes.c_int(0)
        capi.check(lib.unap_cuda_cheby_smooth_host(h, x.ctypes.data, b.ctypes.data, 3,
                                                   ctypes.byref(lam), ctypes.byref(est)))
        assert est.value == 1
        lam_ref, x_ref = orc.eigen(s, x0, b)
        assert abs(lam.value - lam_ref) <= EIG_TOL, (s.name, lam.value, lam_ref)
        assert np.linalg.norm(x - x_ref) <= 1e-12 * np.linalg.norm(x_ref), s.name
        x1 = x.copy()
        capi.check(lib.unap_cuda_cheby_smooth_host(h, x.ctypes.data, b.ctypes.data, 3,
                                                   ctypes.byref(lam), ctypes.byref(est)))
        assert np.array_equal(x, orc.cheby_chain(s, x1, b, lam.value, 1.5, 3)), s.name
        capi.sw_matrix_destroy(h)


@pytest.mark.parametrize("precision", [0, 1])
def test_matrix_without_wavefronts(cuda, orc, precision):
    """Matrices built in locality order only (unap_cuda_set_matrix_wavefronts
    (0)): one row range, the same order from the device and the host build,
    SpMV and the all-Chebyshev V-cycle bit-identical to the oracle, the
    Krylov solve without a preconditioner within 10% of the oracle's
    iteration count; the sweeps (DIC, Gauss-Seidel, AMG with Gauss-Seidel
    on the finest level) refused."""
    torch = cuda
    old = capi.set_matrix_wavefronts(False)
    try:
        for s in (W.lognormal(14, 12, 10, seed=5, permute=True),
                  W.lognormal(40, 36, 30, seed=9, permute=True)):
            A = capi.DeviceMatrix(s)
            perm, waves = A.layout()
            assert len(waves) == 2 and waves[-1] == s.n
            oldd = capi.set_device_setup(-1)
            try:
                H = capi.DeviceMatrix(s)
                assert np.array_equal(H.layout()[0], perm)
                H.close()
            finally:
                capi.set_device_setup(oldd)
            v = np.random.default_rng(s.n).standard_normal(s.n)
            y = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            A.spmv(dev(torch, v), y)
            assert np.array_equal(y.cpu().numpy(), orc.spmv(s, v))
            with pytest.raises(capi.UnapCudaError, match="wavefronts"):
                A.precondition(2, dev(torch, v), y)
            with pytest.raises(capi.UnapCudaError, match="wavefronts"):
                A.gauss_seidel(y, dev(torch, v), 1)
            with pytest.raises(capi.UnapCudaError, match="wavefronts"):
                capi.DeviceAmg(A, n_coarsest=40, precision=precision)
            G = capi.DeviceAmg(A, n_coarsest=40, precision=precision, smoother=1, cheby_from=0)
            O = OracleAmg(orc, s, n_coarsest=40, precision=precision, smoother=1, cheby_from=0,
                          eig_ratio=30.0)
            O.set_eigs(G.eigenvalues())
            z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            G.vcycle(dev(torch, v), z)
            assert np.array_equal(z.cpu().numpy(), O.vcycle(v)), (s.name, precision)
            G.close()
            O.close()
            x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            st = A.krylov_solve(0, 0, x, dev(torch, s.b), rel_tol=1e-6, max_iter=3000)
            x_ref, st_ref = orc.pcg(s, 0, s.b, rel_tol=1e-6, max_iter=3000)
            # unpreconditioned CG amplifies summation-order rounding
            assert abs(st["nIterations"] - st_ref["n_iter"]) <= max(1, st_ref["n_iter"] // 10)
            A.close()
    finally:
        capi.set_matrix_wavefronts(old)
