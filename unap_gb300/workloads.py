"""Synthetic LDU workloads: seeded hex-grid matrices in UNAP's LDU layout.

The reference ships no data sets for its hot path (its examples read
OpenFOAM/Hypre dumps that are not in the repository), so every workload here
is generated from a seed.  A hex grid of nx*ny*nz cells gets one face per pair
of +x/+y/+z neighbours.  An optional seeded random cell permutation makes the
addressing unstructured; faces are then oriented lowerAddr < upperAddr and
sorted by (owner, neighbour), which is the precondition the reference's
Gauss-Seidel (ownerStart, lduMatrix.cpp:269-296) and DIC face-order sweep
(lduDICPrecond.cpp:63-76) rely on.

Matrix families (the LDU conventions of lduMatrixSpMV.cpp:83-92: row u gets
lower[f] at column l, row l gets upper[f] at column u):

* ``laplace``   7-point Laplacian, upper = lower = -1,
                diag = sum |offdiag| + shift (shift 1e-6 by default).
* ``convdiff``  convection-diffusion, face diffusion d = 1, flux F ~ N(0,1)*Pe,
                upper = -(d + max(0,-F)), lower = -(d + max(0,F)),
                diag = sum |offdiag| + 0.01.
* ``lognormal`` variable-coefficient Poisson, cell conductance
                kappa = exp(N(0, sigma^2)), face coefficient = harmonic mean
                2 ka kb / (ka + kb), negated off the diagonal,
                diag = sum |offdiag| + shift (1e-8).
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class LduSystem:
    """One LDU system A x = b (0-based int32 addressing, FP64 values)."""

    n: int
    lower_addr: np.ndarray  # int32[nf], owner
    upper_addr: np.ndarray  # int32[nf], neighbour
    lower: np.ndarray | None  # float64[nf]; None when symmetric
    diag: np.ndarray  # float64[n]
    upper: np.ndarray  # float64[nf]
    b: np.ndarray  # float64[n]
    name: str = ""

    @property
    def nf(self) -> int:
        return int(self.upper_addr.shape[0])

    @property
    def symm(self) -> bool:
        return self.lower is None

    @property
    def lower_or_upper(self) -> np.ndarray:
        return self.upper if self.lower is None else self.lower

    def dense(self) -> np.ndarray:
        """Dense copy (small cases only)."""
        a = np.diag(self.diag.copy())
        a[self.lower_addr, self.upper_addr] += self.upper
        a[self.upper_addr, self.lower_addr] += self.lower_or_upper
        return a


def grid_faces(nx: int, ny: int, nz: int) -> tuple[np.ndarray, np.ndarray]:
    """Face list (a, b) of an nx*ny*nz hex grid in natural cell order
    c = i + nx*(j + ny*k); faces come out sorted by (owner, neighbour): each
    cell's +x, +y, +z faces, cells in order."""
    n = nx * ny * nz
    c = np.arange(n, dtype=np.int64)
    i = c % nx
    j = (c // nx) % ny
    k = c // (nx * ny)
    nb = np.stack([c + 1, c + nx, c + nx * ny], axis=1)
    ok = np.stack([i < nx - 1, j < ny - 1, k < nz - 1], axis=1)
    a = np.broadcast_to(c[:, None], nb.shape)[ok]
    return a, nb[ok]


def permuted_grid_faces(nx: int, ny: int, nz: int, perm: np.ndarray):
    """The faces of an nx*ny*nz hex grid after the cell renumbering
    c -> perm[c], oriented l < u and sorted by (l, u), with each face's two
    cells in the natural numbering (a_old -> l, b_old -> u).  Same list as
    orienting and sorting grid_faces, built row by row (every cell has at
    most six neighbours) instead of by one sort over all faces."""
    n = nx * ny * nz
    perm = perm.astype(np.int32)
    inv = np.empty(n, dtype=np.int32)
    inv[perm] = np.arange(n, dtype=np.int32)
    # row r of the renumbered matrix is old cell inv[r]
    c = inv.astype(np.int64)
    i = c % nx
    j = (c // nx) % ny
    k = c // (nx * ny)
    big = np.int32(np.iinfo(np.int32).max)
    rows = np.arange(n, dtype=np.int32)
    key = np.full((n, 6), big, dtype=np.int32)
    for col, (ok, off) in enumerate(((i > 0, -1), (i < nx - 1, 1), (j > 0, -nx), (j < ny - 1, nx),
                                     (k > 0, -nx * ny), (k < nz - 1, nx * ny))):
        nb = perm[np.where(ok, c + off, 0)]
        key[:, col] = np.where(ok & (nb > rows), nb, big)
    key.sort(axis=1)
    valid = key != big
    u = key[valid]
    l = np.broadcast_to(rows[:, None], key.shape)[valid]
    return l, u, inv[l].astype(np.int64), inv[u].astype(np.int64)


def _orient_and_sort(n: int, a: np.ndarray, b: np.ndarray, perm: np.ndarray | None,
                     *face_data: np.ndarray):
    """Apply the cell permutation, orient l < u and sort faces by (l, u).
    Per-face data arrays are reordered alongside; the returned `flip` mask
    says which faces had their (a, b) orientation swapped."""
    if perm is not None:
        a = perm[a]
        b = perm[b]
    l = np.minimum(a, b)
    u = np.maximum(a, b)
    flip = a > b
    # (l, u) pairs are unique, so one sort of the combined key gives the
    # lexicographic order
    order = np.argsort(l.astype(np.int64) * max(n, 1) + u)
    out = [l[order].astype(np.int32), u[order].astype(np.int32), flip[order]]
    out += [d[order] for d in face_data]
    return out


def _grid_ldu(nx, ny, nz, perm):
    """(lowerAddr, upperAddr) of a grid, optionally renumbered by perm."""
    if perm is None:
        a, b = grid_faces(nx, ny, nz)
        return a.astype(np.int32), b.astype(np.int32)
    l, u, _, _ = permuted_grid_faces(nx, ny, nz, perm)
    return l, u


def _row_abs_sum(n: int, l: np.ndarray, u: np.ndarray, upper: np.ndarray,
                 lower: np.ndarray) -> np.ndarray:
    s = np.zeros(n)
    np.add.at(s, l, np.abs(upper))
    np.add.at(s, u, np.abs(lower))
    return s


def _fast_row_abs_sum(n, l, u, upper, lower):
    s = np.bincount(l, weights=np.abs(upper), minlength=n)
    s += np.bincount(u, weights=np.abs(lower), minlength=n)
    return s


def laplace(nx: int, ny: int | None = None, nz: int | None = None, *, seed: int = 0,
            permute: bool = False, shift: float = 1e-6, rhs: str = "uniform") -> LduSystem:
    """7-point Laplacian, upper = lower = -1, diag = sum|offdiag| + shift."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n = nx * ny * nz
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n).astype(np.int64) if permute else None
    l, u = _grid_ldu(nx, ny, nz, perm)
    upper = np.full(l.shape[0], -1.0)
    diag = _fast_row_abs_sum(n, l, u, upper, upper) + shift
    rhs_v = _rhs(rng, n, rhs)
    return LduSystem(n, l, u, None, diag, upper, rhs_v, name=f"laplace{nx}x{ny}x{nz}")


def convdiff(nx: int, ny: int | None = None, nz: int | None = None, *, seed: int = 0,
             permute: bool = True, pe: float = 5.0, d: float = 1.0,
             shift: float = 0.01) -> LduSystem:
    """Nonsymmetric convection-diffusion LDU."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n = nx * ny * nz
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n).astype(np.int64) if permute else None
    l, u = _grid_ldu(nx, ny, nz, perm)
    flux = rng.standard_normal(l.shape[0]) * pe
    upper = -(d + np.maximum(0.0, -flux))
    lower = -(d + np.maximum(0.0, flux))
    diag = _fast_row_abs_sum(n, l, u, upper, lower) + shift
    rhs_v = rng.uniform(0.0, 1.0, n)
    return LduSystem(n, l, u, lower, diag, upper, rhs_v, name=f"convdiff{nx}x{ny}x{nz}")


def lognormal(nx: int, ny: int | None = None, nz: int | None = None, *, seed: int = 0,
              permute: bool = True, sigma: float = 2.0, shift: float = 1e-8) -> LduSystem:
    """Variable-coefficient Poisson with log-normal cell conductances."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n = nx * ny * nz
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n).astype(np.int64) if permute else None
    kappa = np.exp(rng.standard_normal(n) * sigma)
    if perm is not None:
        l, u, a, b = permuted_grid_faces(nx, ny, nz, perm)
    else:
        a, b = grid_faces(nx, ny, nz)
        l, u = a.astype(np.int32), b.astype(np.int32)
    # the harmonic mean is symmetric in the two cells
    ka, kb = kappa[a], kappa[b]
    coef = 2.0 * ka * kb / (ka + kb)
    upper = -coef
    diag = _fast_row_abs_sum(n, l, u, upper, upper) + shift
    rhs_v = rng.standard_normal(n)
    rhs_v -= rhs_v.mean()
    return LduSystem(n, l, u, None, diag, upper, rhs_v, name=f"lognormal{nx}x{ny}x{nz}")


def _rhs(rng, n, kind):
    if kind == "uniform":
        return rng.uniform(-1.0, 1.0, n)
    if kind == "normal":
        return rng.standard_normal(n)
    if kind == "uniform01":
        return rng.uniform(0.0, 1.0, n)
    raise ValueError(kind)


@dataclasses.dataclass
class Request:
    arrival: float  # seconds after the stream starts
    system: LduSystem
    method: str     # amg_mixed | pcg_dic | bicgstab_dilu
    seed: int


def grid_for(cells: int, rng) -> tuple[int, int, int]:
    """A cubic or elongated (aspect up to 4:1:1) hex grid of about `cells`."""
    if rng.random() < 0.5:
        e = max(4, int(round(cells ** (1 / 3))))
        return e, e, e
    aspect = rng.uniform(2.0, 4.0)
    e = max(4, int(round((cells / aspect) ** (1 / 3))))
    dims = [max(4, int(round(e * aspect))), e, e]
    rng.shuffle(dims)
    return int(dims[0]), int(dims[1]), int(dims[2])


@dataclasses.dataclass
class RequestSpec:
    """One request of the serving stream before its matrix is built."""
    arrival: float
    dims: tuple[int, int, int]
    method: str
    seed: int
    pe: float = 0.0


def serving_stream(count: int = 2000, rate: float = 200.0, min_cells: int = 8_000,
                   max_cells: int = 2_000_000, seed: int = 0) -> list[RequestSpec]:
    """The serving stream (config c5) as request specifications: Poisson
    arrivals at `rate` per second, sizes log-uniform in [min_cells,
    max_cells] on cubic or elongated grids; 60% log-normal Poisson (mixed
    AMG-PCG), 25% Laplacian (PCG+DIC), 15% convection-diffusion with
    Pe ~ U[1, 10] (PBiCGStab+DILU).  `build_request` makes the matrix."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        cells = float(np.exp(rng.uniform(np.log(min_cells), np.log(max_cells))))
        dims = grid_for(int(cells), rng)
        u = rng.random()
        s_seed = int(rng.integers(1 << 31))
        if u < 0.60:
            out.append(RequestSpec(t, dims, "amg_mixed", s_seed))
        elif u < 0.85:
            out.append(RequestSpec(t, dims, "pcg_dic", s_seed))
        else:
            out.append(RequestSpec(t, dims, "bicgstab_dilu", s_seed, float(rng.uniform(1, 10))))
    return out


def build_request(spec: RequestSpec) -> Request:
    """The permuted LDU system of one stream request."""
    nx, ny, nz = spec.dims
    if spec.method == "amg_mixed":
        s = lognormal(nx, ny, nz, seed=spec.seed, permute=True, sigma=2.0)
    elif spec.method == "pcg_dic":
        s = laplace(nx, ny, nz, seed=spec.seed, permute=True, rhs="uniform")
    else:
        s = convdiff(nx, ny, nz, seed=spec.seed, permute=True, pe=spec.pe)
    return Request(spec.arrival, s, spec.method, spec.seed)


def serving_requests(count: int = 2000, rate: float = 200.0, min_cells: int = 8_000,
                     max_cells: int = 2_000_000, seed: int = 0) -> list[Request]:
    """The serving stream (config c5) with every matrix built (see
    serving_stream)."""
    return [build_request(sp) for sp in serving_stream(count, rate, min_cells, max_cells, seed)]


def config(name: str, scale: float = 1.0, seed: int = 0) -> LduSystem:
    """The benchmark configurations by name, optionally shrunk by `scale`
    (grid edge multiplied by scale, at least 4):

    c1  32^3 natural-order Laplacian, PCG+DIC, tol 1e-8
    c2  128^3 permuted Laplacian, FP64 AMG-PCG, tol 1e-10
    c3  200^3 permuted convection-diffusion Pe=5, PBiCGStab+DILU, tol 1e-9
    c4  256^3 permuted log-normal (sigma 2) Poisson, mixed AMG-PCG, tol 1e-10
    """
    def edge(e):
        return max(4, int(round(e * scale)))

    if name == "c1":
        return laplace(edge(32), seed=seed, permute=False, rhs="uniform")
    if name == "c2":
        return laplace(edge(128), seed=seed, permute=True, rhs="normal")
    if name == "c3":
        return convdiff(edge(200), seed=seed, permute=True, pe=5.0)
    if name == "c4":
        return lognormal(edge(256), seed=seed, permute=True, sigma=2.0)
    raise ValueError(name)
