"""The reference's C++ class API (include/unap/) on the GPU.

* tests/cxx/known_answers.cpp: the reference examples' known answers through
  the C++ classes -- the 2x2 system of test/ex3.cpp solved to x = (2, -2) in
  one PCG iteration with DIC (and with Diag, and by PBiCGStab+DILU), and the
  COO -> LDU arrays of test/ex8.cpp.
* tests/cxx/api_driver.cpp: every numerical call of the classes on one
  system, compared with the oracle: SpMV, the DIC preconditioner and its rD,
  Gauss-Seidel sweeps bit for bit; the Chebyshev smoother's eigenvalue
  within the Sturm bisection band and its sweeps bit for bit from the
  device's state; PCG+DIC, PBiCGStab+DILU and MGSolver (Gauss-Seidel and
  Chebyshev) within +-1 iteration and in residual-space agreement; the
  agglomeration's level sizes exactly.
"""
import os
import subprocess

import numpy as np
import pytest

from cxx_util import CXX_DIR, compile_program, compiler
from unap_gb300 import workloads as W

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(compiler() is None, reason="no C++ compiler")]


def _build(name, tmp_path):
    exe = str(tmp_path / name)
    rc, err = compile_program(os.path.join(CXX_DIR, f"{name}.cpp"), exe)
    assert rc == 0, err[-3000:]
    return exe


def test_known_answers(cuda, tmp_path):
    exe = _build("known_answers", tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "pcg_dic iterations 1 x0 2 x1 -2" in r.stdout, r.stdout
    assert "ALL OK" in r.stdout


def test_api_driver_against_oracle(cuda, orc, tmp_path):
    nx, ny, nz, shift = 12, 10, 8, 1e-3
    s = W.laplace(nx, ny, nz, seed=3, permute=False, shift=shift, rhs="normal")
    n = s.n
    rng = np.random.default_rng(9)
    b = np.ascontiguousarray(s.b)
    x0 = rng.standard_normal(n)
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    np.concatenate([b, x0]).tofile(inp)
    exe = _build("api_driver", tmp_path)
    r = subprocess.run([exe, str(nx), str(ny), str(nz), repr(shift), str(inp), str(outp)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(outp)
    pos = [0]

    def take(k):
        v = out[pos[0]:pos[0] + k]
        pos[0] += k
        return v

    assert np.array_equal(take(n), orc.spmv(s, x0))
    w_ref, rD_ref = orc.precond(2, s, b)
    assert np.array_equal(take(n), w_ref)
    assert np.array_equal(take(n), rD_ref)
    assert np.array_equal(take(n), orc.gs(s, x0, b, 2))
    lam = take(1)[0]
    lam_ref, x_est_ref = orc.eigen(s, x0, b)
    assert abs(lam - lam_ref) <= 1e-5, (lam, lam_ref)
    x_est = take(n)
    # the estimate's diagonal-PCG dot products sum in another order
    assert np.linalg.norm(x_est - x_est_ref) <= 1e-12 * np.linalg.norm(x_est_ref)
    assert np.array_equal(take(n), orc.cheby_chain(s, x_est, b, lam, 1.5, 3))
    for method, precond, fn in ((0, 2, orc.pcg), (1, 3, orc.pbicgstab)):
        it = int(take(1)[0])
        xs = take(n)
        x_ref, st = fn(s, precond, b, rel_tol=1e-10)
        assert abs(it - st["n_iter"]) <= 1, (method, it, st)
        assert np.linalg.norm(orc.spmv(s, xs - x_ref)) <= 2.2e-10 * st["init_res"]
    nl = int(take(1)[0])
    sizes = take(nl).astype(int).tolist()
    weights = np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))
    assert sizes == [L["n"] for L in orc.hierarchy(s, weights, n_coarsest=50)]
    for smoother in (1, 2):
        it = int(take(1)[0])
        xs = take(n)
        x_ref, st = orc.mg(s, b, weights, n_coarsest=50, smoother=smoother, rel_tol=1e-8)
        assert abs(it - st["n_iter"]) <= 1, (smoother, it, st)
        assert np.linalg.norm(orc.spmv(s, xs - x_ref)) <= 2.2e-8 * st["init_res"]
    assert pos[0] == out.size
