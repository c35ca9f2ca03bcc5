"""The seeded workload generators (unap_gb300/workloads.py): every matrix
keeps the reference's LDU preconditions (faces oriented lowerAddr <
upperAddr and sorted by owner, then neighbour: lduMatrix.cpp:269-296,
lduDICPrecond.cpp:63-76), the matrix families follow their definitions, the
benchmark configurations have the stated sizes, and the serving stream has
its stated mix.  Host only."""
import numpy as np
import pytest

from unap_gb300 import workloads as W


def _faces_ok(s):
    l = s.lower_addr.astype(np.int64)
    u = s.upper_addr.astype(np.int64)
    assert s.lower_addr.dtype == np.int32 and s.upper_addr.dtype == np.int32
    assert np.all(l < u) and l.min(initial=0) >= 0 and u.max(initial=-1) < s.n
    key = l * s.n + u
    assert np.all(np.diff(key) > 0), "faces sorted by (owner, neighbour), no repeats"


def _grid_faces(nx, ny, nz):
    return 3 * nx * ny * nz - (ny * nz + nx * nz + nx * ny)


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 1, 1), (5, 4, 3), (7, 1, 2), (6, 6, 6)])
@pytest.mark.parametrize("permute", [False, True])
def test_ldu_preconditions(shape, permute):
    for gen, kw in (("laplace", {}), ("lognormal", {}), ("convdiff", {"pe": 3.0})):
        s = getattr(W, gen)(*shape, seed=11, permute=permute, **kw)
        assert s.n == int(np.prod(shape))
        assert s.nf == _grid_faces(*shape)
        _faces_ok(s)
        assert s.diag.shape == (s.n,) and s.b.shape == (s.n,)


def test_permutation_relabels_the_grid():
    """A permuted matrix is the natural-order one with its cells renamed:
    the same diagonal multiset and, for the Laplacian, the same spectrum."""
    a = W.laplace(4, 3, 5, seed=2, permute=False)
    b = W.laplace(4, 3, 5, seed=2, permute=True)
    assert np.array_equal(np.sort(a.diag), np.sort(b.diag))
    ea = np.linalg.eigvalsh(a.dense())
    eb = np.linalg.eigvalsh(b.dense())
    assert np.allclose(ea, eb, rtol=0, atol=1e-12)


def test_family_definitions():
    # Laplacian: off-diagonals -1, diag = sum |offdiag| + shift
    s = W.laplace(5, 4, 3, seed=1, permute=True, shift=0.25)
    assert s.symm and np.all(s.upper == -1.0)
    off = np.abs(s.dense() - np.diag(np.diag(s.dense()))).sum(axis=1)
    assert np.allclose(s.diag, off + 0.25, rtol=0, atol=1e-14)
    # log-normal Poisson: symmetric, negative harmonic-mean coefficients,
    # diagonal dominance by the shift, a mean-free right-hand side
    s = W.lognormal(6, 5, 4, seed=3, permute=True, sigma=2.0)
    assert s.symm and np.all(s.upper < 0)
    off = np.abs(s.dense() - np.diag(np.diag(s.dense()))).sum(axis=1)
    assert np.allclose(s.diag - off, 1e-8, rtol=0, atol=1e-12 * s.diag.max())
    assert abs(s.b.mean()) < 1e-14
    # convection-diffusion: d = 1 on every face, upwinding on exactly one
    # side, diag = sum |offdiag| + 0.01
    s = W.convdiff(6, 5, 4, seed=4, permute=True, pe=5.0)
    assert not s.symm
    assert np.all(np.minimum(-s.upper, -s.lower) == 1.0)
    off = np.abs(s.dense() - np.diag(np.diag(s.dense()))).sum(axis=1)
    assert np.allclose(s.diag, off + 0.01, rtol=1e-14, atol=1e-14)


def test_seeds_reproduce():
    a = W.lognormal(5, 5, 5, seed=9)
    b = W.lognormal(5, 5, 5, seed=9)
    c = W.lognormal(5, 5, 5, seed=10)
    assert np.array_equal(a.upper, b.upper) and np.array_equal(a.b, b.b)
    assert np.array_equal(a.lower_addr, b.lower_addr)
    assert not np.array_equal(a.upper, c.upper)


def test_config_sizes():
    c1 = W.config("c1")
    assert (c1.n, c1.nf) == (32_768, 95_232)
    _faces_ok(c1)
    # natural order: the faces of a cell's +x/+y/+z neighbours
    assert np.array_equal(np.unique(c1.upper_addr - c1.lower_addr), [1, 32, 1024])
    for name, edge in (("c2", 128), ("c3", 200), ("c4", 256)):
        s = W.config(name, scale=8 / edge)
        assert (s.n, s.nf) == (512, _grid_faces(8, 8, 8)), name
        _faces_ok(s)
    assert _grid_faces(128, 128, 128) == 6_242_304
    assert _grid_faces(200, 200, 200) == 23_880_000
    assert _grid_faces(256, 256, 256) == 50_135_040
    with pytest.raises(ValueError):
        W.config("c9")


def test_serving_stream_mix():
    specs = W.serving_stream(count=2000, rate=200.0, seed=0)
    assert len(specs) == 2000
    t = np.array([s.arrival for s in specs])
    assert np.all(np.diff(t) > 0)
    # Poisson arrivals at 200/s: 2000 requests in about 10 s
    assert 9.0 < t[-1] < 11.0
    cells = np.array([np.prod(s.dims) for s in specs])
    assert cells.min() >= 4 ** 3 and cells.max() <= 2.6e6
    frac = {m: np.mean([s.method == m for s in specs])
            for m in ("amg_mixed", "pcg_dic", "bicgstab_dilu")}
    assert abs(frac["amg_mixed"] - 0.60) < 0.04
    assert abs(frac["pcg_dic"] - 0.25) < 0.04
    assert abs(frac["bicgstab_dilu"] - 0.15) < 0.04
    pe = [s.pe for s in specs if s.method == "bicgstab_dilu"]
    assert min(pe) >= 1.0 and max(pe) <= 10.0
    assert [s.seed for s in W.serving_stream(count=50, seed=0)] == [s.seed for s in specs[:50]]
    # a request's matrix is built by its own seed
    r = W.build_request(specs[0])
    _faces_ok(r.system)
    assert r.system.n == int(np.prod(specs[0].dims))
