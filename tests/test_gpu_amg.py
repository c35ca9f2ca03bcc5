"""GPU parity of AMG-PCG (FP64 and FP32 V-cycle) against the oracle.

The hierarchy is the reference's pairwise agglomeration (exact integer
equality of the level sizes), one V-cycle is bit-identical to the oracle's in
both precisions (every kernel keeps the oracle's per-row order, the coarsest
inverse is computed by the same Cholesky steps), and a full AMG-PCG solve
matches the oracle's iteration count within +-1, its solution within 1e-10
relative 2-norm, and reaches the true relative residual it claims.
"""
import numpy as np
import pytest

from oracle_lib import OracleAmg
from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def spd_systems():
    return [W.lognormal(14, 12, 10, seed=5, permute=True),
            W.laplace(12, 11, 10, seed=6, permute=True, rhs="normal"),
            W.laplace(10, seed=7, permute=False),
            W.lognormal(20, seed=8, permute=True, sigma=1.0)]


def dev(torch, a):
    return torch.tensor(np.asarray(a, dtype=np.float64), device="cuda")


@pytest.mark.parametrize("precision", [0, 1])
def test_hierarchy_and_vcycle_bit_exact(cuda, orc, precision, tail_mode):
    torch = cuda
    for s in spd_systems():
        A = capi.DeviceMatrix(s)
        G = capi.DeviceAmg(A, n_coarsest=40, precision=precision)
        O = OracleAmg(orc, s, n_coarsest=40, precision=precision)
        info = G.info()
        assert info["cells"] == O.level_sizes(), s.name
        r = np.random.default_rng(s.n).standard_normal(s.n)
        z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        G.vcycle(dev(torch, r), z)
        assert np.array_equal(z.cpu().numpy(), O.vcycle(r)), (s.name, precision)
        G.close()
        O.close()
        A.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_amg_pcg_parity(cuda, orc, precision, executor):
    torch = cuda
    for s in spd_systems():
        A = capi.DeviceMatrix(s)
        G = capi.DeviceAmg(A, n_coarsest=40, precision=precision, rel_tol=1e-10)
        O = OracleAmg(orc, s, n_coarsest=40, precision=precision, flexible=precision,
                      rel_tol=1e-10)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, dev(torch, s.b))
        x_ref, st_ref = O.solve(s.b)
        xg = x.cpu().numpy()
        assert st["converged"] and st_ref["converged"]
        assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (s.name, st, st_ref)
        # both meet ||b - A x|| <= 1e-10 ||b||: they agree within that in
        # residual space (dot-product summation order differs)
        assert (np.linalg.norm(orc.spmv(s, xg - x_ref))
                <= 2.2e-10 * st_ref["init_res"]), s.name
        true_rel = np.linalg.norm(s.b - orc.spmv(s, xg)) / np.linalg.norm(s.b)
        assert true_rel <= 1.0001e-10, (s.name, true_rel)
        # the host-array entry point gives the same bits as the device one
        xh = np.zeros(s.n)
        st_h = G.solve_host(xh, np.ascontiguousarray(s.b))
        assert st_h["nIterations"] == st["nIterations"]
        assert np.array_equal(xh, xg)
        G.close()
        O.close()
        A.close()


def test_amg_pcg_solution_tight(cuda, orc, executor):
    """FP64 AMG-PCG to relTol 1e-13 on well-conditioned systems: the GPU and
    oracle solutions agree within 1e-10 relative 2-norm."""
    torch = cuda
    for s in (W.laplace(12, 11, 10, seed=6, permute=True, rhs="normal", shift=0.5),
              W.lognormal(16, seed=8, permute=True, sigma=1.0, shift=0.1)):
        A = capi.DeviceMatrix(s)
        G = capi.DeviceAmg(A, n_coarsest=40, precision=0, rel_tol=1e-13)
        O = OracleAmg(orc, s, n_coarsest=40, precision=0, rel_tol=1e-13)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, dev(torch, s.b))
        x_ref, st_ref = O.solve(s.b)
        assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (s.name, st, st_ref)
        xg = x.cpu().numpy()
        assert np.linalg.norm(xg - x_ref) <= 1e-10 * np.linalg.norm(x_ref), s.name
        G.close()
        O.close()
        A.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_amg_pcg_same_bits_in_every_tail_mode(cuda, precision):
    """The V-cycle is bit-identical wherever its coarse levels run, so whole
    AMG-PCG solves are too: same iteration count, same solution bits."""
    from conftest import TAIL_MODES
    torch = cuda
    s = W.lognormal(24, 20, 18, seed=11, permute=True)
    A = capi.DeviceMatrix(s)
    b = dev(torch, s.b)
    modes = ["per-wavefront", "sell-sweeps", "packed-narrow", "packed-wide"] + (
        ["cluster", "one-cta", "split"] if capi.tail_cluster_size() > 0 else [])
    results = {}
    old = capi.set_tail_rows(*TAIL_MODES["per-wavefront"])
    try:
        for m in modes:
            # "sell-sweeps" / "packed-narrow": per-wavefront launches reading
            # the SELL-32 rows, or the row-packed copy with a 16/8-entry window
            capi.set_packed_sweeps({"sell-sweeps": 0, "packed-narrow": 2,
                                    "packed-wide": 3}.get(m, 1))
            capi.set_tail_rows(*TAIL_MODES[m if m in TAIL_MODES else "per-wavefront"])
            G = capi.DeviceAmg(A, n_coarsest=60, precision=precision, rel_tol=1e-10)
            x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            st = G.solve(x, b)
            results[m] = (st["nIterations"], x.cpu().numpy())
            G.close()
    finally:
        capi.set_packed_sweeps(1)
        capi.restore_tail_rows(old)
        A.close()
    it0, x0 = results["per-wavefront"]
    for m, (it, xm) in results.items():
        assert it == it0, (m, it, it0)
        assert np.array_equal(xm, x0), m


def test_amg_rejects_nonsymmetric(cuda):
    s = W.convdiff(6, seed=1)
    A = capi.DeviceMatrix(s)
    with pytest.raises(capi.UnapCudaError, match="symmetric"):
        capi.DeviceAmg(A)
    A.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_device_coarsest_inverse_bit_exact(cuda, orc, precision):
    """Coarsest levels of 128 cells or more are inverted on the device; the
    V-cycle stays bit-identical to the oracle's, with coarse levels and with
    none (the matrix itself is the coarsest, in its own internal order)."""
    torch = cuda
    for s, nco in ((W.lognormal(18, 16, 14, seed=12, permute=True), 700),
                   (W.laplace(8, 8, 6, seed=13, permute=True, rhs="normal"), 1000)):
        A = capi.DeviceMatrix(s)
        G = capi.DeviceAmg(A, n_coarsest=nco, precision=precision)
        O = OracleAmg(orc, s, n_coarsest=nco, precision=precision)
        cells = G.info()["cells"]
        assert cells == O.level_sizes(), s.name
        assert cells[-1] >= 128, cells
        r = np.random.default_rng(s.n).standard_normal(s.n)
        z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        G.vcycle(dev(torch, r), z)
        assert np.array_equal(z.cpu().numpy(), O.vcycle(r)), (s.name, precision)
        G.close()
        O.close()
        A.close()
