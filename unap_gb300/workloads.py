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
    c = i + nx*(j + ny*k); faces come out sorted by (owner, neighbour)."""
    idx = np.arange(nx * ny * nz, dtype=np.int64).reshape(nz, ny, nx)
    parts_a, parts_b = [], []
    if nx > 1:
        parts_a.append(idx[:, :, :-1])
        parts_b.append(idx[:, :, 1:])
    if ny > 1:
        parts_a.append(idx[:, :-1, :])
        parts_b.append(idx[:, 1:, :])
    if nz > 1:
        parts_a.append(idx[:-1, :, :])
        parts_b.append(idx[1:, :, :])
    if not parts_a:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    a = np.concatenate([p.ravel() for p in parts_a])
    b = np.concatenate([p.ravel() for p in parts_b])
    order = np.lexsort((b, a))
    return a[order], b[order]


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
    order = np.lexsort((u, l))
    out = [l[order].astype(np.int32), u[order].astype(np.int32), flip[order]]
    out += [d[order] for d in face_data]
    return out


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
    a, b = grid_faces(nx, ny, nz)
    l, u, _ = _orient_and_sort(n, a, b, perm)
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
    a, b = grid_faces(nx, ny, nz)
    l, u, _ = _orient_and_sort(n, a, b, perm)
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
    a, b = grid_faces(nx, ny, nz)
    ka, kb = kappa[a], kappa[b]
    coef = 2.0 * ka * kb / (ka + kb)
    l, u, _, coef = _orient_and_sort(n, a, b, perm, coef)
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


def serving_requests(count: int = 2000, rate: float = 200.0, min_cells: int = 8_000,
                     max_cells: int = 2_000_000, seed: int = 0) -> list[Request]:
    """The serving stream (config c5): Poisson arrivals at `rate` per second,
    sizes log-uniform in [min_cells, max_cells], permuted LDU on cubic or
    elongated grids; 60% log-normal Poisson solved by mixed AMG-PCG, 25%
    Laplacian by PCG+DIC, 15% convection-diffusion (Pe ~ U[1, 10]) by
    PBiCGStab+DILU."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate)
        cells = float(np.exp(rng.uniform(np.log(min_cells), np.log(max_cells))))
        nx, ny, nz = grid_for(int(cells), rng)
        u = rng.random()
        s_seed = int(rng.integers(1 << 31))
        if u < 0.60:
            s = lognormal(nx, ny, nz, seed=s_seed, permute=True, sigma=2.0)
            method = "amg_mixed"
        elif u < 0.85:
            s = laplace(nx, ny, nz, seed=s_seed, permute=True, rhs="uniform")
            method = "pcg_dic"
        else:
            s = convdiff(nx, ny, nz, seed=s_seed, permute=True, pe=float(rng.uniform(1, 10)))
            method = "bicgstab_dilu"
        out.append(Request(t, s, method, s_seed))
    return out


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
