"""Device-built matrix structure (internal order, wavefronts, SELL-32 layout,
values) against the host build, which is the specification: the same cell
order and wavefront boundaries exactly, and therefore the same bits from
every kernel and solve.  Covers many BFS levels (an unpermuted grid), several
connected components with runs of isolated cells, asymmetric values, and
AMG hierarchies whose coarse levels carry locality keys; shapes the device
build declines go to the host with the same result (a cell with more lower
neighbours than it takes, a chain with more wavefronts, more connected
components than it follows).
"""
import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def merged(parts, isolated_every=0, seed=0):
    """Block-diagonal system of `parts` with cells interleaved and, when
    isolated_every > 0, a cell without faces after every that many cells."""
    rng = np.random.default_rng(seed)
    n = sum(p.n for p in parts)
    owner = np.concatenate([np.full(p.n, k) for k, p in enumerate(parts)])
    rng.shuffle(owner)
    order = np.zeros(n, np.int64)
    nxt = [0] * len(parts)
    newid = [np.zeros(p.n, np.int64) for p in parts]
    pos = 0
    for i, k in enumerate(owner):
        if isolated_every and i % isolated_every == isolated_every - 1:
            pos += 1  # leave an isolated cell
        newid[k][nxt[k]] = pos
        nxt[k] += 1
        pos += 1
    N = pos + (1 if isolated_every else 0)
    l = np.concatenate([newid[k][p.lower_addr] for k, p in enumerate(parts)])
    u = np.concatenate([newid[k][p.upper_addr] for k, p in enumerate(parts)])
    up = np.concatenate([p.upper for p in parts])
    lo = np.concatenate([p.upper if p.symm else p.lower for p in parts])
    srt = np.lexsort((u, l))
    diag = np.full(N, 2.0)
    for k, p in enumerate(parts):
        diag[newid[k]] = p.diag
    b = rng.standard_normal(N)
    sym = all(p.symm for p in parts)
    return W.LduSystem(N, l[srt].astype(np.int32), u[srt].astype(np.int32),
                       None if sym else lo[srt], diag, up[srt], b, name=f"merged{N}")


def star(n_leaves=1500, seed=0):
    """Leaves 0..n-1 each joined to the hub n (the last cell): the hub has
    more lower-side faces than the device build handles."""
    rng = np.random.default_rng(seed)
    n = n_leaves + 1
    l = np.arange(n_leaves, dtype=np.int32)
    u = np.full(n_leaves, n_leaves, np.int32)
    up = -rng.random(n_leaves)
    diag = np.ones(n) + np.abs(up).sum() * (np.arange(n) == n_leaves)
    diag[:n_leaves] += np.abs(up)
    return W.LduSystem(n, l, u, None, diag, up, rng.standard_normal(n), name="star")


def chain(n=6000, seed=0):
    """A 1-D chain in natural order: n wavefronts, more than the device
    build takes (declined to the host, same result)."""
    rng = np.random.default_rng(seed)
    l = np.arange(n - 1, dtype=np.int32)
    u = l + 1
    up = -rng.random(n - 1) - 0.5
    diag = np.full(n, 3.0)
    return W.LduSystem(n, l, u, None, diag, up, rng.standard_normal(n), name="chain")


def systems():
    return [chain(),
            merged([W.laplace(3, 2, 2, seed=40 + k, permute=True) for k in range(70)], seed=2),
            W.lognormal(20, 18, 16, seed=3, permute=True),
            W.laplace(24, 20, 18, seed=4, permute=False),     # 60 wavefronts, deep BFS
            W.convdiff(16, 14, 12, seed=2, permute=True),     # asymmetric
            merged([W.laplace(9, 8, 7, seed=5, permute=True),
                    W.lognormal(10, 9, 8, seed=6, permute=True),
                    W.laplace(6, seed=7, permute=False)], isolated_every=37, seed=1),
            star()]


def built(s, min_cells):
    old = capi.set_device_setup(min_cells)
    try:
        A = capi.DeviceMatrix(s)
        A.layout()  # builds now, under this setting
    finally:
        capi.set_device_setup(old)
    return A


def test_device_layout_equals_host_layout(cuda):
    torch = cuda
    for s in systems():
        D, H = built(s, 1), built(s, -1)
        pd, wd = D.layout()
        ph, wh = H.layout()
        assert np.array_equal(pd, ph), s.name
        assert np.array_equal(wd, wh), s.name
        assert D.info() == H.info(), s.name
        x = torch.tensor(np.random.default_rng(1).standard_normal(s.n), device="cuda")
        yd = torch.zeros_like(x)
        yh = torch.zeros_like(x)
        D.spmv(x, yd)
        H.spmv(x, yh)
        assert torch.equal(yd, yh), s.name
        b = torch.tensor(s.b, device="cuda")
        for A, out in ((D, yd), (H, yh)):
            out.zero_()
            A.gauss_seidel(out, b, 2)
        assert torch.equal(yd, yh), s.name
        if s.symm:
            xs = []
            for A in (D, H):
                xv = torch.zeros_like(x)
                st = A.krylov_solve(0, 2, xv, b, rel_tol=1e-9, max_iter=400)
                xs.append((st["nIterations"], xv.cpu().numpy()))
            assert xs[0][0] == xs[1][0] and np.array_equal(xs[0][1], xs[1][1]), s.name
        D.close()
        H.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_device_built_amg_equals_host_built(cuda, precision):
    torch = cuda
    s = W.lognormal(28, 24, 22, seed=9, permute=True)
    out = []
    for mc in (1, -1):
        old = capi.set_device_setup(mc)
        try:
            A = capi.DeviceMatrix(s)
            G = capi.DeviceAmg(A, n_coarsest=60, precision=precision, rel_tol=1e-10)
        finally:
            capi.set_device_setup(old)
        lay = [G.level_layout(k) for k in range(len(G.info()["cells"]))]
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, torch.tensor(s.b, device="cuda"))
        out.append((lay, st["nIterations"], x.cpu().numpy()))
        G.close()
        A.close()
    (ld, itd, xd), (lh, ith, xh) = out
    assert len(ld) == len(lh)
    for k, ((pd, wd), (ph, wh)) in enumerate(zip(ld, lh)):
        assert np.array_equal(pd, ph), k
        assert np.array_equal(wd, wh), k
    assert itd == ith
    assert np.array_equal(xd, xh)


def coo_of(s, rng, shuffle_cols=True):
    """The system as 0-based COO, rows ascending, columns in random order
    inside each row (sorted when shuffle_cols is False)."""
    rows = np.concatenate([np.arange(s.n), s.lower_addr, s.upper_addr])
    cols = np.concatenate([np.arange(s.n), s.upper_addr, s.lower_addr])
    vals = np.concatenate([s.diag, s.upper, s.upper if s.symm else s.lower])
    key = rng.random(rows.shape[0]) if shuffle_cols else cols
    o = np.lexsort((key, rows))
    return vals[o], rows[o].astype(np.int32), cols[o].astype(np.int32)


def csr2ldu(vals, rows, cols, n, symm):
    import ctypes
    lib = capi.load()
    ptr = np.zeros(n + 1, np.int32)
    np.add.at(ptr, rows + 1, 1)
    ptr = np.cumsum(ptr).astype(np.int32)
    h = ctypes.c_long(0)
    v = np.ascontiguousarray(vals, np.float64)
    c = np.ascontiguousarray(cols, np.int32)
    lib.csr2ldumatrixcreat_(ctypes.byref(h), v.ctypes.data_as(capi._dp),
                            ptr.ctypes.data_as(capi._ip), c.ctypes.data_as(capi._ip),
                            ctypes.byref(ctypes.c_int(n)), ctypes.byref(ctypes.c_int(v.shape[0])),
                            ctypes.byref(ctypes.c_int(1 if symm else 0)))
    if not h.value:
        raise capi.UnapCudaError(lib.unap_cuda_last_error().decode())
    return h.value


def both_ways(make):
    out = []
    for mc in (1, -1):
        old = capi.set_device_setup(mc)
        try:
            h = make()
        finally:
            capi.set_device_setup(old)
        out.append(capi.handle_ldu(h))
        capi.sw_matrix_destroy(h)
    return out


def assert_same_ldu(a, b):
    assert (a["n"], a["nf"], a["symm"]) == (b["n"], b["nf"], b["symm"])
    for k in ("lower_addr", "upper_addr"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("diag", "upper", "lower"):
        assert np.array_equal(a[k].view(np.int64), b[k].view(np.int64)), k


def test_device_coo_and_csr_ingest_equal_host(cuda):
    rng = np.random.default_rng(4)
    for s in (W.convdiff(14, 12, 10, seed=2, permute=True),
              W.lognormal(16, seed=3, permute=True),
              merged([W.laplace(7, seed=1, permute=True), W.convdiff(6, seed=2)], seed=3)):
        v, r, c = coo_of(s, rng)
        d, h = both_ways(lambda: capi.coo2ldumatrixcreat(v, r + 1, c + 1, s.n, symm=s.symm))
        assert_same_ldu(d, h)
        # the ingest gives back the system itself
        assert np.array_equal(d["upper_addr"], s.upper_addr)
        assert np.array_equal(d["upper"], s.upper) and np.array_equal(d["diag"], s.diag)
        if not s.symm:
            assert np.array_equal(d["lower"], s.lower)
        v2, r2, c2 = coo_of(s, rng, shuffle_cols=False)
        dc, hc = both_ways(lambda: csr2ldu(v2, r2, c2, s.n, s.symm))
        assert_same_ldu(dc, hc)
        assert_same_ldu(dc, d)


def test_device_coo_ingest_errors_match_host(cuda):
    rng = np.random.default_rng(5)
    s = W.convdiff(8, 7, 6, seed=2, permute=True)
    v, r, c = coo_of(s, rng)
    lower = np.nonzero(c < r)[0]
    upper = np.nonzero(c > r)[0]
    # one lower entry moved to another column of its row: counts per column
    # no longer match the upper faces
    k = lower[len(lower) // 2]
    row_cols = set(c[r == r[k]].tolist())
    free = next(x for x in range(int(r[k])) if x not in row_cols)
    c_bad = c.copy()
    c_bad[k] = free
    order_bad = r.copy()
    order_bad[[upper[3], upper[-3]]] = order_bad[[upper[-3], upper[3]]]
    dup_c = c.copy()
    same_row = np.nonzero(r == r[upper[5]])[0]
    dup_c[same_row[0]], dup_c[same_row[1]] = dup_c[same_row[1]], dup_c[same_row[1]]
    cases = [(c_bad, r, "structurally symmetric"),
             (c, order_bad, "ascending row order"),
             (dup_c, r, "repeats an entry")]
    for cc, rr, msg in cases:
        for mc in (1, -1):
            old = capi.set_device_setup(mc)
            try:
                with pytest.raises(capi.UnapCudaError, match=msg):
                    capi.coo2ldumatrixcreat(v, rr + 1, cc + 1, s.n, symm=False)
            finally:
                capi.set_device_setup(old)


def test_device_agglomeration_matches_oracle(cuda, orc):
    """Agglomeration on the device (dependency rounds of the sequential
    greedy) gives the reference's hierarchy: level sizes and V-cycle bits
    equal to the oracle's."""
    from oracle_lib import OracleAmg
    torch = cuda
    old = capi.set_device_setup(1)
    try:
        for s in (W.lognormal(30, 26, 24, seed=21, permute=True),
                  W.laplace(28, seed=22, permute=True, rhs="normal"),
                  W.lognormal(16, 14, 12, seed=23, permute=False)):
            for precision in (0, 1):
                A = capi.DeviceMatrix(s)
                G = capi.DeviceAmg(A, n_coarsest=60, precision=precision)
                O = OracleAmg(orc, s, n_coarsest=60, precision=precision)
                assert G.info()["cells"] == O.level_sizes(), s.name
                r = np.random.default_rng(s.n).standard_normal(s.n)
                z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
                G.vcycle(torch.tensor(r, device="cuda"), z)
                assert np.array_equal(z.cpu().numpy(), O.vcycle(r)), (s.name, precision)
                G.close()
                O.close()
                A.close()
    finally:
        capi.set_device_setup(old)


def test_device_agglomeration_asymmetric_mg_same_bits(cuda):
    """The reference MGSolver on a convection-diffusion matrix (asymmetric
    coarse coefficients): device-built and host-built hierarchies give the
    same solve bit for bit."""
    torch = cuda
    s = W.convdiff(22, 20, 18, seed=24, permute=True, pe=2.0)
    w = np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))
    out = []
    for mc in (1, -1):
        old = capi.set_device_setup(mc)
        try:
            A = capi.DeviceMatrix(s)
            G = capi.DeviceMG(A, weights=w, smoother=1, n_coarsest=12, rel_tol=1e-8, max_iter=60)
        finally:
            capi.set_device_setup(old)
        x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
        st = G.solve(x, torch.tensor(s.b, device="cuda"))
        out.append((G.levels(), st["nIterations"], x.cpu().numpy()))
        G.close()
        A.close()
    assert out[0][0] == out[1][0]
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])
