"""Batched solves: many systems of uneven size in one fused launch.

Each system's result in the batch must be the same as solved alone (and as
the oracle's) within the solver tolerance: iteration count within +-1 and
agreement within 2.2 relTol ||r0|| in residual space.  The batch mixes PCG
(none/Diag/DIC) on symmetric and PBiCGStab+DILU on nonsymmetric systems, and
one system above the fused-launch size limit.
"""
import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def make_batch():
    rng = np.random.default_rng(41)
    out = []
    for i in range(24):
        e = int(rng.integers(4, 14))
        kind = i % 4
        if kind == 0:
            s = W.laplace(e, e + 1, e + 2, seed=i, permute=True, rhs="normal", shift=0.1)
            out.append((s, 0, 2))
        elif kind == 1:
            s = W.lognormal(e, e, e + 1, seed=i, permute=True, sigma=1.0, shift=0.01)
            out.append((s, 0, 1))
        elif kind == 2:
            s = W.convdiff(e, e, e, seed=i, permute=True, pe=3.0)
            out.append((s, 1, 3))
        else:
            s = W.laplace(e + 2, e, e, seed=i, permute=False, shift=0.5)
            out.append((s, 0, 0))
    out.append((W.lognormal(44, 40, 40, seed=99, permute=True, sigma=1.0, shift=0.01), 0, 2))
    return out


def test_batch_matches_individual_and_oracle(cuda, orc):
    torch = cuda
    cases = make_batch()
    mats = [capi.DeviceMatrix(s) for s, _, _ in cases]
    xs = [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s, _, _ in cases]
    bs = [torch.tensor(s.b, device="cuda") for s, _, _ in cases]
    B = capi.Batch()
    items = [dict(matrix=m, method=meth, precond=pc, x=x, b=b, rel_tol=1e-9, max_iter=2000)
             for m, (s, meth, pc), x, b in zip(mats, cases, xs, bs)]
    stats, threads = B.solve(items)
    assert threads in (128, 256, 512, 1024)
    for (s, meth, pc), m, x, b, st in zip(cases, mats, xs, bs, stats):
        x_alone = torch.zeros_like(x)
        st_alone = m.krylov_solve(meth, pc, x_alone, b, rel_tol=1e-9, max_iter=2000)
        fn = orc.pcg if meth == 0 else orc.pbicgstab
        x_ref, st_ref = fn(s, pc, s.b, rel_tol=1e-9, max_iter=2000)
        assert st["converged"] and st_alone["converged"], (s.name, st)
        for other in (st_alone["nIterations"], st_ref["n_iter"]):
            assert abs(st["nIterations"] - other) <= 1, (s.name, st, st_alone, st_ref)
        xb = x.cpu().numpy()
        for other in (x_alone.cpu().numpy(), x_ref):
            d = orc.spmv(s, xb - other)
            assert np.linalg.norm(d) <= 2.2e-9 * st_ref["init_res"], s.name
    # a second batch reuses the tuned CTA size and cached factors
    for x in xs:
        x.zero_()
    stats2, threads2 = B.solve(items)
    assert threads2 == threads
    assert [s["nIterations"] for s in stats2] == [s["nIterations"] for s in stats]
    B.close()
    for m in mats:
        m.close()


def test_batch_factor_cache_after_matrix_replaced(cuda, orc):
    """A matrix destroyed and a new one created (the allocator may hand back
    the same address) must not reuse the old matrix's cached DIC factor."""
    torch = cuda
    B = capi.Batch()
    for seed in range(4):
        s = W.lognormal(14, 13, 12, seed=100 + seed, permute=True, sigma=1.5, shift=0.01)
        m = capi.DeviceMatrix(s)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        b = torch.tensor(s.b, device="cuda")
        (st,), _ = B.solve([dict(matrix=m, method=0, precond=2, x=x, b=b, rel_tol=1e-9,
                                 max_iter=2000)])
        _, st_ref = orc.pcg(s, 2, s.b, rel_tol=1e-9, max_iter=2000)
        assert st["converged"], (seed, st)
        assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (seed, st, st_ref)
        m.close()
    B.close()


def team_cases():
    return [(W.laplace(20, 18, 16, seed=51, permute=True, rhs="normal", shift=0.1), 0, 2),
            (W.laplace(24, 24, 24, seed=52, permute=False, rhs="uniform"), 0, 2),
            (W.lognormal(16, 15, 14, seed=53, permute=True, sigma=1.0, shift=0.01), 0, 1),
            (W.convdiff(18, 17, 16, seed=54, permute=True, pe=4.0), 1, 3),
            (W.convdiff(12, 12, 30, seed=55, permute=False, pe=2.0), 1, 3),
            (W.laplace(15, 14, 13, seed=56, permute=True, shift=0.5), 0, 0)]


@pytest.mark.parametrize("threads,cluster", [(128, 1), (1024, 1), (256, 2), (512, 4),
                                             (128, 8), (1024, 8), (256, 16), (1024, 16)])
def test_team_shapes_match_oracle(cuda, orc, threads, cluster):
    """Every launch shape of the whole-solve kernel (one CTA, or a cluster of
    2-16 CTAs whose block sums meet in distributed shared memory) gives the
    oracle's iterations within one and its solution in residual space, and
    a repeated launch of the same shape is bit-identical."""
    torch = cuda
    if cluster > 1 and capi.load().unap_cuda_force_team_shape(threads, cluster) != 0:
        pytest.skip("device cannot schedule this cluster")
    capi.force_team_shape(threads, cluster)
    try:
        cases = team_cases()
        mats = [capi.DeviceMatrix(s) for s, _, _ in cases]
        bs = [torch.tensor(s.b, device="cuda") for s, _, _ in cases]
        B = capi.Batch()
        runs = []
        for rep in range(2):
            xs = [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s, _, _ in cases]
            items = [dict(matrix=m, method=meth, precond=pc, x=x, b=b, rel_tol=1e-9,
                          max_iter=2000)
                     for m, (s, meth, pc), x, b in zip(mats, cases, xs, bs)]
            stats, _ = B.solve(items)
            assert B.last_shape() == (threads, cluster)
            runs.append(([x.cpu().numpy() for x in xs], stats))
        for (s, meth, pc), st, xb, xb2 in zip(cases, runs[0][1], runs[0][0], runs[1][0]):
            fn = orc.pcg if meth == 0 else orc.pbicgstab
            x_ref, st_ref = fn(s, pc, s.b, rel_tol=1e-9, max_iter=2000)
            assert st["converged"], (s.name, st)
            assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1, (s.name, st, st_ref)
            d = orc.spmv(s, xb - x_ref)
            assert np.linalg.norm(d) <= 2.2e-9 * st_ref["init_res"], s.name
            assert np.array_equal(xb, xb2), s.name
        # single solves through the Krylov driver take the same launch
        s, meth, pc = cases[1]
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = mats[1].krylov_solve(meth, pc, x, bs[1], rel_tol=1e-9, max_iter=2000)
        assert np.array_equal(x.cpu().numpy(), runs[0][0][1])
        assert st["nIterations"] == runs[0][1][1]["nIterations"]
        B.close()
        for m in mats:
            m.close()
    finally:
        capi.force_team_shape(0, 0)


def test_team_shape_autotuner(cuda):
    """The autotuner picks a launchable shape per (size class, count class)
    and reuses it."""
    torch = cuda
    s = W.laplace(22, 21, 20, seed=61, permute=True, rhs="normal", shift=0.1)
    m = capi.DeviceMatrix(s)
    b = torch.tensor(s.b, device="cuda")
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    m.krylov_solve(0, 2, x, b, rel_tol=1e-9, max_iter=2000)
    t, c = capi.team_shape(s.n, 1)
    assert t in (128, 256, 512, 1024) and c in (1, 2, 4, 8, 16)
    x.zero_()
    m.krylov_solve(0, 2, x, b, rel_tol=1e-9, max_iter=2000)
    assert capi.team_shape(s.n, 1) == (t, c)
    m.close()


def test_large_systems_batch(cuda, orc):
    """Systems above the whole-solve size: the autotuner picks one group
    launch (clusters of 16 CTAs) or one solve after another; either way each
    result matches the oracle, and the next batch of that class keeps the
    choice."""
    torch = cuda
    cases = [(W.laplace(44, 42, 40, seed=71, permute=True, rhs="normal", shift=0.1), 0, 2),
             (W.convdiff(42, 42, 40, seed=72, permute=True, pe=3.0), 1, 3),
             (W.lognormal(46, 40, 40, seed=73, permute=True, sigma=1.0, shift=0.01), 0, 1)]
    assert all(s.n > 65536 for s, _, _ in cases)
    mats = [capi.DeviceMatrix(s) for s, _, _ in cases]
    bs = [torch.tensor(s.b, device="cuda") for s, _, _ in cases]
    B = capi.Batch()
    modes = []
    for rep in range(2):
        xs = [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s, _, _ in cases]
        items = [dict(matrix=m, method=meth, precond=pc, x=x, b=b, rel_tol=1e-9, max_iter=3000)
                 for m, (s, meth, pc), x, b in zip(mats, cases, xs, bs)]
        stats, _ = B.solve(items)
        modes.append(B.large_mode())
        for (s, meth, pc), st, x in zip(cases, stats, xs):
            fn = orc.pcg if meth == 0 else orc.pbicgstab
            x_ref, st_ref = fn(s, pc, s.b, rel_tol=1e-9, max_iter=3000)
            assert st["converged"], (s.name, st)
            assert abs(st["nIterations"] - st_ref["n_iter"]) <= 1 or pc == 1, (s.name, st, st_ref)
            d = orc.spmv(s, x.cpu().numpy() - x_ref)
            assert np.linalg.norm(d) <= 2.2e-9 * st_ref["init_res"], s.name
    assert modes[0] in (0, 1) and modes[1] == modes[0]
    B.close()
    for m in mats:
        m.close()
