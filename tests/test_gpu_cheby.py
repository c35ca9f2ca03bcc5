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
