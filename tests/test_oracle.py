"""The C restatement (oracle/unap_oracle.c) against the reference.

* against tests/golden/reference_small.npz (outputs of the reference library
  on seeded systems; runs on every host);
* against the reference's own known answers (test/ex2.cpp, test/ex3.cpp);
* against the reference library itself on freshly generated systems, where
  oracle/_ref was built on this host.

Every comparison is bit-exact: both codes run the same loops with the same
operation order and no fused multiply-adds.
"""
import numpy as np
import pytest

import golden_cases
from unap_gb300 import workloads as W


def _eq(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and np.array_equal(a, b)


@pytest.fixture(scope="module")
def golden():
    return golden_cases.load()


def test_golden_kernels(orc, golden):
    for s, g in golden:
        x = g["x"]
        assert _eq(orc.spmv(s, x), g["spmv"]), s.name
        for t in (1, 2, 3):
            w, rD = orc.precond(t, s, x)
            assert _eq(w, g[f"precond{t}_w"]) and _eq(rD, g[f"precond{t}_rD"]), (s.name, t)
        assert _eq(orc.gs(s, x, s.b, 3), g["gs3"]), s.name
        assert _eq(orc.cheby(s, x, s.b, 3, 3), g["cheby3x3"]), s.name
        e, xe = orc.eigen(s, x, s.b)
        assert e == float(g["eig"]) and _eq(xe, g["eig_x"]), s.name


def test_golden_krylov(orc, golden):
    for s, g in golden:
        for t in (0, 1, 2, 3):
            x, st = orc.pcg(s, t, s.b, rel_tol=1e-8)
            ref = g[f"pcg{t}_stats"]
            assert _eq(x, g[f"pcg{t}_x"]), (s.name, "pcg", t)
            assert st["n_iter"] == int(ref[0]) and st["final_res"] == ref[2]
            x, st = orc.pbicgstab(s, t, s.b, rel_tol=1e-8)
            ref = g[f"bicg{t}_stats"]
            assert _eq(x, g[f"bicg{t}_x"]), (s.name, "bicg", t)
            assert st["n_iter"] == int(ref[0]) and st["final_res"] == ref[2]


def test_golden_hierarchy_and_mg(orc, golden):
    for s, g in golden:
        w = np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))
        levels = orc.hierarchy(s, w, n_coarsest=8)
        assert len(levels) == int(g["nlevels"]), s.name
        for li, L in enumerate(levels):
            for key in ("restrict", "face_restrict", "lower_addr", "upper_addr", "diag", "upper",
                        "lower"):
                if key == "lower" and s.symm:
                    continue
                assert _eq(L[key], g[f"L{li}_{key}"]), (s.name, li, key)
        for sm in (1, 2):
            x, st = orc.mg(s, s.b, w, n_coarsest=8, smoother=sm, rel_tol=1e-8, max_iter=60)
            ref = g[f"mg{sm}_stats"]
            assert _eq(x, g[f"mg{sm}_x"]), (s.name, sm)
            assert st["n_iter"] == int(ref[0]) and st["n_levels"] == int(ref[4])


def test_known_answer_ex2_spmv(orc):
    # test/ex2.cpp: 10-cell ring, diag 4, off-diagonals -1, x = (i + 0.2)/0.4;
    # the reference prints Apsi = (-24, 6, 11, 16, 21, 26, 31, 36, 41, 71)
    n = 10
    lo_addr = np.array([i if i < n - 1 else 0 for i in range(n)], np.int32)
    up_addr = np.array([i + 1 if i < n - 1 else n - 1 for i in range(n)], np.int32)
    s = W.LduSystem(n, lo_addr, up_addr, np.full(n, -1.0), np.full(n, 4.0), np.full(n, -1.0),
                    np.zeros(n))
    y = orc.spmv(s, (np.arange(n) + 0.2) / 0.4)
    assert np.allclose(y, [-24, 6, 11, 16, 21, 26, 31, 36, 41, 71], rtol=0, atol=1e-12)


def test_known_answer_ex3_pcg(orc):
    # test/ex3.cpp: A = [[3,2],[2,6]], b = (2,-8), PCG+DIC -> x = (2,-2) in 1 iteration
    s = W.LduSystem(2, np.array([0], np.int32), np.array([1], np.int32), np.array([2.0]),
                    np.array([3.0, 6.0]), np.array([2.0]), np.array([2.0, -8.0]))
    x, st = orc.pcg(s, 2, s.b)
    assert st["n_iter"] == 1
    assert np.allclose(x, [2.0, -2.0], atol=1e-14)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_against_reference_library(orc, ref, seed):
    cases = [W.laplace(5, 6, 4, seed=seed, permute=True, rhs="normal"),
             W.convdiff(5, 5, 5, seed=seed, permute=True, pe=3.0 + seed),
             W.lognormal(7, 6, 5, seed=seed, permute=True)]
    for s in cases:
        x = np.random.default_rng(seed).standard_normal(s.n)
        assert _eq(orc.spmv(s, x), ref.spmv(s, x))
        for a, b in zip(orc.losort(s), ref.losort(s)):
            assert _eq(a, b)
        for t in (1, 2, 3):
            assert all(_eq(a, b) for a, b in zip(orc.precond(t, s, x), ref.precond(t, s, x)))
        assert _eq(orc.gs(s, x, s.b, 2), ref.gs(s, x, s.b, 2))
        assert _eq(orc.cheby(s, x, s.b, 4, 2), ref.cheby(s, x, s.b, 4, 2))
        for t in (0, 2, 3):
            a, b = orc.pcg(s, t, s.b, rel_tol=1e-9), ref.pcg(s, t, s.b, rel_tol=1e-9)
            assert _eq(a[0], b[0]) and a[1] == b[1]
            a, b = orc.pbicgstab(s, t, s.b, rel_tol=1e-9), ref.pbicgstab(s, t, s.b, rel_tol=1e-9)
            assert _eq(a[0], b[0]) and a[1] == b[1]
        w = np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))
        h1, h2 = orc.hierarchy(s, w, n_coarsest=6), ref.hierarchy(s, w, n_coarsest=6)
        assert len(h1) == len(h2)
        for L1, L2 in zip(h1, h2):
            for k in ("restrict", "face_restrict", "lower_addr", "upper_addr", "diag", "upper"):
                assert _eq(L1[k], L2[k]), k
        for sm in (1, 2):
            a = orc.mg(s, s.b, w, n_coarsest=6, smoother=sm, rel_tol=1e-8, max_iter=40)
            b = ref.mg(s, s.b, w, n_coarsest=6, smoother=sm, rel_tol=1e-8, max_iter=40)
            assert _eq(a[0], b[0]) and a[1] == b[1]


def test_mg_options_against_reference(orc, ref):
    # pre-smoothing, no correction scaling, maxLevels limit
    s = W.laplace(6, 6, 5, seed=7, permute=True, rhs="normal")
    w = np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))
    for kw in (dict(n_pre=2), dict(scale_corr=0), dict(max_levels=3, n_post=1, n_finest=3)):
        for sm in (1, 2):
            a = orc.mg(s, s.b, w, n_coarsest=5, smoother=sm, rel_tol=1e-8, max_iter=30, **kw)
            b = ref.mg(s, s.b, w, n_coarsest=5, smoother=sm, rel_tol=1e-8, max_iter=30, **kw)
            assert _eq(a[0], b[0]) and a[1] == b[1], kw


def test_amg_pcg_oracle_converges(orc):
    # NEW component (no reference counterpart): AMG-PCG with SGS, dense coarsest
    from oracle_lib import OracleAmg
    s = W.lognormal(12, seed=3)
    for prec in (0, 1):
        A = OracleAmg(orc, s, n_coarsest=60, precision=prec, flexible=prec, rel_tol=1e-10)
        sizes = A.level_sizes()
        assert sizes[-1] <= 60 and sizes[0] == s.n
        x, st = A.solve(s.b)
        assert st["converged"]
        r = s.b - orc.spmv(s, x)
        assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(s.b)
        inv = A.coarse_inverse()
        assert np.allclose(inv, inv.T, rtol=0, atol=0)
        A.close()


def test_amg_iteration_cap_can_change(orc):
    """The reference arm's sampling: one hierarchy, solves capped at 1, 6
    and then unlimited iterations; the capped runs restart from x = 0 and
    the residuals decrease with the cap."""
    from oracle_lib import OracleAmg
    s = W.lognormal(12, seed=4)
    A = OracleAmg(orc, s, n_coarsest=60, precision=0, rel_tol=1e-10, max_iter=1)
    _, s1 = A.solve(s.b)
    A.set_max_iter(6)
    _, s6 = A.solve(s.b)
    A.set_max_iter(500)
    _, sf = A.solve(s.b)
    assert (s1["n_iter"], s6["n_iter"]) == (1, 6)
    assert s1["init_res"] == s6["init_res"] == sf["init_res"]
    assert sf["converged"] and sf["n_iter"] > 6
    assert s1["final_res"] > s6["final_res"] > sf["final_res"]
    A.close()


def test_cheby_chain_is_the_reference_smoother(orc, golden):
    """The AMG levels' Chebyshev chain (a step from x, then degree - 1 more)
    is chebySmoother::smooth after its first, estimating call: from the
    reference's eigenvalue and the x its estimate leaves, two chains of 3
    steps with the reference's ratio 1.5 give the reference's
    3-sweep-x-3-call result bit for bit (golden vectors printed by the
    reference library)."""
    for s, g in golden:
        x1 = g["eig_x"]
        lam = float(g["eig"])
        x2 = orc.cheby_chain(s, x1, s.b, lam, 1.5, 3)
        x3 = orc.cheby_chain(s, x2, s.b, lam, 1.5, 3)
        assert _eq(x3, g["cheby3x3"]), s.name


def test_cheby_chain_against_reference_library(orc, ref):
    for seed in (0, 1):
        for s in (W.lognormal(7, 6, 5, seed=seed, permute=True),
                  W.laplace(6, 5, 5, seed=seed, permute=True, rhs="normal")):
            x = np.random.default_rng(seed).standard_normal(s.n)
            for deg in (1, 2, 4):
                lam, x1 = ref.eigen(s, x, s.b)
                want = ref.cheby(s, x, s.b, deg, 2)
                assert _eq(orc.cheby_chain(s, x1, s.b, lam, 1.5, deg), want), (s.name, deg)
            # the chain from x = 0 equals the chain from a zero vector
            z = orc.cheby_chain(s, x, s.b, 1.9, 30.0, 3, from_zero=True)
            assert _eq(z, orc.cheby_chain(s, np.zeros(s.n), s.b, 1.9, 30.0, 3)), s.name


def test_eig_start_vector(orc):
    """splitmix64 start vector: deterministic, in [-1, 1), mean near 0."""
    v = orc.eig_start(4096)
    assert np.all(v >= -1.0) and np.all(v < 1.0)
    assert abs(v.mean()) < 0.05 and v.std() > 0.5
    assert len(np.unique(v)) == v.size


def test_cheby_amg_oracle(orc):
    """AMG-PCG with the Chebyshev V-cycle (new component): per-level
    eigenvalue estimates of D^-1 A are within the spectrum's upper end, the
    FP64 V-cycle is a symmetric operator, and the solve converges to the
    true relative residual it claims, in FP64 and FP32."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from oracle_lib import OracleAmg
    s = W.lognormal(12, 11, 10, seed=3, permute=True)
    for prec in (0, 1):
        for frm in (0, 1):
            A = OracleAmg(orc, s, n_coarsest=60, precision=prec, flexible=prec, rel_tol=1e-10,
                          smoother=1, cheby_degree=3, cheby_from=frm, eig_ratio=30.0)
            lam = A.eigs()
            assert np.all(lam[:frm] == 0) and np.all(lam[frm:] > 0)
            if frm == 0 and prec == 0:
                M = sp.coo_matrix((np.concatenate([s.upper, s.upper, s.diag]),
                                   (np.concatenate([s.lower_addr, s.upper_addr, np.arange(s.n)]),
                                    np.concatenate([s.upper_addr, s.lower_addr, np.arange(s.n)]))),
                                  shape=(s.n, s.n)).tocsr()
                Dh = sp.diags(1.0 / np.sqrt(s.diag))
                top = spla.eigsh(Dh @ M @ Dh, k=1, which="LA", return_eigenvectors=False)[0]
                # Lanczos from 10 iterations approaches lambda_max from below
                assert 0.8 * top <= lam[0] <= top * (1 + 1e-6), (lam[0], top)
                rng = np.random.default_rng(1)
                r1, r2 = rng.standard_normal(s.n), rng.standard_normal(s.n)
                a, b = np.dot(A.vcycle(r1), r2), np.dot(r1, A.vcycle(r2))
                assert abs(a - b) <= 1e-12 * abs(a), (a, b)
            x, st = A.solve(s.b)
            assert st["converged"], (prec, frm, st)
            r = s.b - orc.spmv(s, x)
            assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(s.b)
            A.close()


_DEGENERATE_EIGEN = r"""
import sys
import numpy as np
sys.path[:0] = [{root!r}, {tests!r}]
from oracle_lib import Oracle
from unap_gb300 import workloads as W
orc = Oracle("orc")
out = []
for s in (W.convdiff(2, 1, 1, seed=3, permute=True, pe=2.0),
          W.laplace(2, 1, 1, seed=3, permute=True),
          W.laplace(3, 1, 1, seed=4, permute=True, shift=0.5)):
    x0 = np.random.default_rng(1).standard_normal(s.n)
    e, _ = orc.eigen(s, x0, s.b, 10)
    out.append(e)
print(repr(out))
"""


def test_eigen_estimate_ends_when_the_diagonal_pcg_stops_early():
    """The two-cell convection-diffusion system stops the diagonal PCG after
    two iterations; the reference builds its tridiagonal matrix from all ten
    (zero alphas, infinite entries) and its bisection never ends.  The
    oracle's (like the CUDA path's) uses the iterations that ran and returns
    a finite estimate; the tiny Laplacians beside it end either way.  Run in
    a child process so that a regression fails instead of stalling the
    suite."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = _DEGENERATE_EIGEN.format(root=root, tests=os.path.join(root, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr[-2000:]
    vals = eval(r.stdout.strip().splitlines()[-1])
    assert len(vals) == 3 and all(np.isfinite(v) for v in vals), vals


def test_eigen_estimate_of_one_cell_is_one_over_alpha(orc):
    """A one-cell system: the diagonal PCG solves it in its first iteration
    (alpha_0 = 1) and stops; the estimate is 1 / alpha_0 from the one
    iteration that ran (the reference bisects over infinite entries and
    returns 0.99999237), and the iterate is the exact solution b / d."""
    s = W.laplace(1, 1, 1, seed=3, permute=True)
    assert s.n == 1 and s.nf == 0
    e, x = orc.eigen(s, np.array([0.7]), s.b, 10)
    assert e == 1.0
    assert np.allclose(x, s.b / s.diag, rtol=1e-15)


def test_tiny_eigen_estimates_against_reference_library(orc, ref):
    """Two- and three-cell Laplacians, on which the reference's estimate
    ends: the oracle's estimate and iterate are the reference's, bit for
    bit."""
    for s in (W.laplace(2, 1, 1, seed=3, permute=True),
              W.laplace(3, 1, 1, seed=4, permute=True, shift=0.5)):
        x0 = np.random.default_rng(1).standard_normal(s.n)
        a, xa = orc.eigen(s, x0, s.b, 10)
        b, xb = ref.eigen(s, x0, s.b, 10)
        assert a == b and _eq(xa, xb), (a, b)


def test_mg_without_coarse_levels(orc):
    """A matrix already at or below nCellsCoarsest gets no coarse level (the
    reference's MGSolver then dereferences a missing level and crashes).
    The oracle, like the CUDA MgSolver, runs the V-cycle without coarse
    levels: nothing is prolongated into the finest correction, so without
    correction scaling Gauss-Seidel MG is plain Gauss-Seidel iteration (with
    it, the scaling's Jacobi update still acts)."""
    s = W.laplace(1, 1, 7, seed=5, permute=True, rhs="normal")
    w = np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))
    assert orc.hierarchy(s, w, n_coarsest=8) == []
    x, st = orc.mg(s, s.b, w, n_coarsest=8, smoother=1, rel_tol=1e-8, max_iter=3, n_finest=2,
                   scale_corr=0)
    assert st["n_levels"] == 0 and st["n_iter"] == 3
    assert _eq(x, orc.gs(s, np.zeros(s.n), s.b, 6))
    x, st = orc.mg(s, s.b, w, n_coarsest=8, smoother=1, rel_tol=1e-8, max_iter=40)
    assert st["n_levels"] == 0 and np.all(np.isfinite(x))


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 1, 1), (1, 1, 7), (1, 3, 2), (3, 3, 1),
                                   (2, 2, 5)])
def test_tiny_and_thin_systems_against_reference_library(orc, ref, shape):
    """Edge shapes: one cell and no face, two cells, a chain, thin slabs.
    SpMV, the three preconditioners, Gauss-Seidel, and PCG / PBiCGStab with
    every preconditioner code (1 Diag, 2 DIC, 3 DILU, 0 none) are the
    reference library's bit for bit, iteration counts and residuals
    included."""
    for gen, kw in (("laplace", {}), ("lognormal", {}), ("convdiff", {"pe": 2.0})):
        s = getattr(W, gen)(*shape, seed=3, permute=True, **kw)
        x = np.random.default_rng(1).standard_normal(s.n)
        assert _eq(orc.spmv(s, x), ref.spmv(s, x))
        for t in (1, 2, 3):
            assert all(_eq(a, b) for a, b in zip(orc.precond(t, s, x), ref.precond(t, s, x)))
        assert _eq(orc.gs(s, x, s.b, 2), ref.gs(s, x, s.b, 2))
        for t in (0, 1, 2, 3):
            if s.symm:
                a, b = (o.pcg(s, t, s.b, rel_tol=1e-9, max_iter=200) for o in (orc, ref))
                assert _eq(a[0], b[0]) and a[1] == b[1], (gen, shape, t)
            a, b = (o.pbicgstab(s, t, s.b, rel_tol=1e-9, max_iter=200) for o in (orc, ref))
            assert _eq(a[0], b[0]) and a[1] == b[1], (gen, shape, t)


def test_golden_fixture_is_what_its_generator_writes(ref):
    """tests/golden/reference_small.npz holds exactly what
    tests/golden/make_golden.py computes with the reference library built
    here: every array, bit for bit."""
    import importlib.util
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(here, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    fresh = mod.generate(ref)
    with np.load(os.path.join(here, "golden", "reference_small.npz")) as z:
        assert sorted(z.files) == sorted(fresh)
        for k in z.files:
            assert _eq(z[k], fresh[k]), k
