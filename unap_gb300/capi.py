"""ctypes binding of libunap_cuda.so (include/unap_cuda.h).

This is the Python-side mirror of UNAP's foreign interface: the reference's
Fortran-convention calls (``ldumatrixcreat_``, ``pcgsolversolve_`` ...) are
exposed under the same names with the same argument meaning, and the GB300
``unap_cuda_*`` entry points are wrapped for device-resident vectors (any
object with a ``data_ptr()`` such as a CUDA torch tensor, or a raw int).

The library must be built (``unap_gb300.build.build()``); importing a missing
library raises instead of falling back to anything.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_c_int = ctypes.c_int
_c_long = ctypes.c_long
_c_ll = ctypes.c_longlong
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)

_LIB = None


class UnapCudaError(RuntimeError):
    pass


class Stats(ctypes.Structure):
    _fields_ = [("nIterations", _c_int), ("converged", _c_int), ("singular", _c_int),
                ("status", _c_int), ("initialResidual", _c_dbl), ("finalResidual", _c_dbl),
                ("trueResidual", _c_dbl), ("seconds", _c_dbl), ("algorithmicBytes", _c_dbl)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# name -> (restype, argtypes); the exported C symbols of include/unap_cuda.h
SIGNATURES = {
    "ldumatrixcreat_": (None, [_lp, _ip, _ip, _ip, _ip, _dp, _dp, _dp]),
    "coo2ldumatrixcreat_": (None, [_lp, _dp, _ip, _ip, _ip, _ip, _ip]),
    "csr2ldumatrixcreat_": (None, [_lp, _dp, _ip, _ip, _ip, _ip, _ip]),
    "matrixinterfacescreat_": (None, [_lp, _ip, _ip, _ip, _ip, _dp]),
    "pcgsolversolve_": (None, [_dp, _lp, _dp, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _dp]),
    "pbicgstabsolversolve_": (None, [_dp, _lp, _dp, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _dp]),
    "contruct_sw_matrix__": (None, [_lp, _ip, _ip, _ip, _ip]),
    "contruct_sw_matrix_interfaces__": (None, [_lp, _ip, _ip, _ip, _ip]),
    "fill_sw_matrix_coefficients__": (None, [_lp, _dp, _dp, _dp]),
    "fill_sw_matrix_interfaces_coefficients__": (None, [_lp, _ip, _dp]),
    "contruct_solver_pbicgstab__": (None, [_lp]),
    "sw_solver_pbicgstab_set_maxiter__": (None, [_lp, _ip]),
    "sw_solver_pbicgstab_set_miniter__": (None, [_lp, _ip]),
    "sw_solver_pbicgstab_set_tol__": (None, [_lp, _dp]),
    "sw_solver_pbicgstab_set_reltol__": (None, [_lp, _dp]),
    "sw_solver_pbicgstab_set_precond__": (None, [_lp, _lp, _ip]),
    "sw_solve_pbicgstab__": (None, [_lp, _lp, _dp, _dp, _dp]),
    "sw_matrix_destroy__": (None, [_lp]),
    "sw_solver_destroy_pbicgstab__": (None, [_lp]),
    "reordercoo_": (None, [_dp, _ip, _ip, _ip, _ip]),
    "reorderuface__": (None, [_ip, _ip, _ip, _ip, _ip]),
    "reorderlface__": (None, [_ip, _ip, _ip, _ip, _ip]),
    "reordervalue__": (None, [_dp, _ip, _ip]),
    "unap_cuda_matrix_set_values": (_c_int, [_c_long, _vp, _vp, _vp]),
    "unap_cuda_spmv_host": (_c_int, [_c_long, _vp, _vp]),
    "unap_cuda_precondition_host": (_c_int, [_c_long, _c_int, _vp, _vp]),
    "unap_cuda_precond_rD": (_c_int, [_c_long, _c_int, _vp]),
    "unap_cuda_gauss_seidel_host": (_c_int, [_c_long, _vp, _vp, _c_int, _c_int]),
    "unap_cuda_cheby_smooth_host": (_c_int, [_c_long, _vp, _vp, _c_int, _vp, _vp]),
    "unap_cuda_krylov_solve_host": (_c_int, [_c_long, _c_int, _c_int, _c_dbl, _c_dbl, _c_int,
                                             _c_int, _vp, _vp, ctypes.POINTER(Stats)]),
    "unap_cuda_reorder_coo": (_c_int, [_vp, _vp, _vp, _c_int, _c_int]),
    "unap_cuda_reorder_uface": (_c_int, [_vp, _vp, _c_int, _c_int, _vp]),
    "unap_cuda_reorder_lface": (_c_int, [_vp, _vp, _c_int, _c_int, _vp]),
    "unap_cuda_reorder_value": (_c_int, [_vp, _vp, _c_int]),
    "unap_cuda_agglomeration_create": (_c_int, [_lp, _c_long, _vp, _c_int, _c_int]),
    "unap_cuda_agglomeration_size": (_c_int, [_c_long, _vp]),
    "unap_cuda_agglomeration_level": (_c_int, [_c_long, _c_int, _vp, _vp, _vp, _vp, _vp, _vp,
                                               _vp, _vp, _vp, _vp]),
    "unap_cuda_agglomeration_destroy": (_c_int, [_c_long]),
    "unap_cuda_mg_solve_host": (_c_int, [_c_long, _vp, _vp, ctypes.POINTER(Stats)]),
    "unap_cuda_mg_set": (_c_int, [_c_long, _c_int, _c_int, _c_int, _c_int, _c_dbl, _c_dbl,
                                  _c_int, _c_int]),
    "unap_cuda_last_error": (ctypes.c_char_p, []),
    "unap_cuda_version": (ctypes.c_char_p, []),
    "unap_cuda_device_synchronize": (_c_int, []),
    "unap_cuda_matrix_create": (_c_int, [_lp, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp]),
    "unap_cuda_matrix_destroy": (_c_int, [_c_long]),
    "unap_cuda_matrix_size": (_c_int, [_c_long, _ip, _ip, _ip]),
    "unap_cuda_matrix_get_ldu": (_c_int, [_c_long, _vp, _vp, _vp, _vp, _vp]),
    "unap_cuda_matrix_info": (_c_int, [_c_long, _ip, ctypes.POINTER(_c_ll),
                                       ctypes.POINTER(_c_ll)]),
    "unap_cuda_spmv": (_c_int, [_c_long, _vp, _vp]),
    "unap_cuda_spmv_noalloc": (_c_int, [_c_long, _vp, _vp]),
    "unap_cuda_profile_kernels": (_c_int, [_c_long, _c_int, _vp]),
    "unap_cuda_precondition": (_c_int, [_c_long, _c_int, _vp, _vp]),
    "unap_cuda_gauss_seidel": (_c_int, [_c_long, _vp, _vp, _c_int, _c_int]),
    "unap_cuda_krylov_solve": (_c_int, [_c_long, _c_int, _c_int, _c_dbl, _c_dbl, _c_int,
                                        _c_int, _vp, _vp, ctypes.POINTER(Stats)]),
    "unap_cuda_amg_default_params": (None, [_vp]),
    "unap_cuda_amg_create": (_c_int, [_lp, _c_long, _vp]),
    "unap_cuda_amg_info": (_c_int, [_c_long, _ip, _vp, _vp, _c_int, _dp,
                                    ctypes.POINTER(_c_ll)]),
    "unap_cuda_amg_vcycle": (_c_int, [_c_long, _vp, _vp]),
    "unap_cuda_amg_setup_phases": (_c_int, [_c_long, _vp]),
    "unap_cuda_amg_eigenvalues": (_c_int, [_c_long, _vp, _c_int, _vp]),
    "unap_cuda_amg_profile_smoother": (_c_int, [_c_long, _c_int, _c_int, _vp, _vp, _vp]),
    "unap_cuda_set_cheby_small_rows": (_c_int, [_c_int]),
    "unap_cuda_set_cheby_chunk": (_c_int, [_c_int]),
    "unap_cuda_set_matrix_wavefronts": (_c_int, [_c_int]),
    "unap_cuda_amg_profile_vcycle": (_c_int, [_c_long, _c_int, _vp, _c_int, _ip]),
    "unap_cuda_amg_solve": (_c_int, [_c_long, _vp, _vp, ctypes.POINTER(Stats)]),
    "unap_cuda_amg_solve_host": (_c_int, [_c_long, _vp, _vp, ctypes.POINTER(Stats)]),
    "unap_cuda_amg_destroy": (_c_int, [_c_long]),
    "unap_cuda_launch_count": (_c_ll, []),
    "unap_cuda_set_executor": (_c_int, [_c_int]),
    "unap_cuda_set_host_wait": (_c_int, [_c_int]),
    "unap_cuda_set_wave_pdl": (_c_int, [_c_int]),
    "unap_cuda_set_wave_grid": (_c_int, [_c_int]),
    "unap_cuda_set_packed_sweeps": (_c_int, [_c_int]),
    "unap_cuda_set_tail_rows": (_c_int, [_c_int, _c_ll, _c_ll, ctypes.POINTER(_c_ll),
                                         ctypes.POINTER(_c_ll)]),
    "unap_cuda_tail_cluster_size": (_c_int, [_ip]),
    "unap_cuda_selftest_barrier_timeout": (_c_int, [_ip, _ip]),
    "mgsolversolve_": (None, [_dp, _lp, _dp, _ip, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _dp, _dp]),
    "contruct_solver_mg__": (None, [_lp, _lp, _lp, _dp, _ip, _ip, _ip]),
    "sw_solver_mg_set_maxiter__": (None, [_lp, _ip]),
    "sw_solver_mg_set_miniter__": (None, [_lp, _ip]),
    "sw_solver_mg_set_tol__": (None, [_lp, _dp]),
    "sw_solver_mg_set_reltol__": (None, [_lp, _dp]),
    "sw_solver_mg_set_npresweeps__": (None, [_lp, _ip]),
    "sw_solver_mg_set_npostsweeps__": (None, [_lp, _ip]),
    "sw_solver_mg_set_nfinestsweeps__": (None, [_lp, _ip]),
    "sw_solve_mg__": (None, [_lp, _lp, _dp, _dp, _dp]),
    "sw_solver_destroy_mg__": (None, [_lp]),
    "unap_cuda_mg_create": (_c_int, [_lp, _c_long, _vp, _c_int, _c_int, _c_int, _c_int, _c_int,
                                     _c_int, _c_int, _c_dbl, _c_dbl, _c_int, _c_int]),
    "unap_cuda_mg_levels": (_c_int, [_c_long, _ip, _vp, _c_int]),
    "unap_cuda_mg_solve": (_c_int, [_c_long, _vp, _vp, ctypes.POINTER(Stats)]),
    "unap_cuda_mg_destroy": (_c_int, [_c_long]),
    "unap_cuda_batch_create": (_c_int, [_lp]),
    "unap_cuda_batch_solve": (_c_int, [_c_long, _c_int, _vp, _vp, _ip]),
    "unap_cuda_batch_destroy": (_c_int, [_c_long]),
    "unap_cuda_batch_last_shape": (_c_int, [_c_long, _ip, _ip]),
    "unap_cuda_batch_large_mode": (_c_int, [_c_long, _ip]),
    "unap_cuda_set_team_solve_cells": (_c_int, [_c_int]),
    "unap_cuda_team_shape": (_c_int, [_c_int, _c_int, _ip, _ip]),
    "unap_cuda_force_team_shape": (_c_int, [_c_int, _c_int]),
    "unap_cuda_set_server_graphs": (_c_int, [_c_int]),
    "unap_cuda_set_cheby_tail_rows": (_c_int, [_c_int]),
    "unap_cuda_set_server_team_cells": (_c_int, [_c_int]),
    "unap_cuda_set_server_amg": (_c_int, [_c_int, _c_dbl]),
    "unap_cuda_server_create": (_c_int, [_lp, _c_ll, _c_int, _c_int]),
    "unap_cuda_server_submit": (_c_int, [_c_long, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp,
                                         _c_int, _c_dbl, _c_int, ctypes.POINTER(_c_ll)]),
    "unap_cuda_server_wait": (_c_int, [_c_long, _c_ll, _vp, _vp]),
    "unap_cuda_server_destroy": (_c_int, [_c_long]),
    "unap_cuda_set_device_setup": (_c_int, [_c_ll, ctypes.POINTER(_c_ll)]),
    "unap_cuda_matrix_layout": (_c_int, [_c_long, _ip, _vp, _vp]),
    "unap_cuda_amg_level_layout": (_c_int, [_c_long, _c_int, _ip, ctypes.POINTER(_c_ll), _ip,
                                            _vp, _vp]),
    "unap_cuda_read_ldu_matrix": (_c_int, [ctypes.c_char_p, _lp]),
    "unap_cuda_read_vector": (_c_int, [ctypes.c_char_p, _c_ll, _vp]),
    "unap_cuda_read_interfaces": (_c_int, [ctypes.c_char_p, _ip, ctypes.POINTER(_c_ll), _vp, _vp,
                                           _vp, _vp]),
    "unap_cuda_print_ldu_matrix": (_c_int, [_c_long, ctypes.c_char_p]),
    "unap_cuda_print_vector": (_c_int, [ctypes.c_char_p, _c_ll, _vp]),
    "unap_cuda_print_interfaces": (_c_int, [ctypes.c_char_p, _c_int, _vp, _vp, _vp, _vp]),
}


class BatchItem(ctypes.Structure):
    _fields_ = [("matrix", _c_long), ("method", _c_int), ("precond", _c_int), ("tol", _c_dbl),
                ("relTol", _c_dbl), ("maxIter", _c_int), ("minIter", _c_int), ("x", _vp),
                ("b", _vp)]


class Batch:
    """Batched solves (``unap_cuda_batch_*``): many systems, one fused launch
    for the small ones."""

    def __init__(self):
        h = _c_long(0)
        check(load().unap_cuda_batch_create(ctypes.byref(h)))
        self.handle = h.value

    def solve(self, items):
        """items: list of dicts(matrix=DeviceMatrix, method, precond, x, b,
        rel_tol=1e-6, tol=0, max_iter=1000, min_iter=0)."""
        arr = (BatchItem * len(items))()
        for i, it in enumerate(items):
            arr[i] = BatchItem(it["matrix"].handle, it.get("method", 0), it.get("precond", 0),
                               it.get("tol", 0.0), it.get("rel_tol", 1e-6),
                               it.get("max_iter", 1000), it.get("min_iter", 0),
                               _ptr(it["x"]), _ptr(it["b"]))
        stats = (Stats * len(items))()
        threads = _c_int(0)
        check(load().unap_cuda_batch_solve(self.handle, len(items), arr, stats,
                                           ctypes.byref(threads)))
        return [s.as_dict() for s in stats], threads.value

    def large_mode(self):
        """Systems above the whole-solve size in the last batch: 1 one group
        launch, 0 one after another, -1 none."""
        m = ctypes.c_int(0)
        check(load().unap_cuda_batch_large_mode(self.handle, ctypes.byref(m)))
        return m.value

    def last_shape(self):
        """(CTA size, CTAs per system) of the last fused launch."""
        t, c = ctypes.c_int(0), ctypes.c_int(0)
        check(load().unap_cuda_batch_last_shape(self.handle, ctypes.byref(t), ctypes.byref(c)))
        return t.value, c.value

    def close(self):
        if self.handle:
            check(load().unap_cuda_batch_destroy(self.handle))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RequestInfo(ctypes.Structure):
    _fields_ = [("status", _c_int), ("batched", _c_int), ("nIterations", _c_int),
                ("converged", _c_int), ("initialResidual", _c_dbl), ("finalResidual", _c_dbl),
                ("queueSeconds", _c_dbl), ("setupSeconds", _c_dbl), ("solveSeconds", _c_dbl),
                ("latencySeconds", _c_dbl)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


SERVE_METHODS = {"amg_mixed": 0, "amg_fp64": 1, "pcg_dic": 2, "bicgstab_dilu": 3}


class Server:
    """Continuous-batching solve server (``unap_cuda_server_*``)."""

    def __init__(self, memory_budget=0, max_slots=4, small_cells=65536):
        h = _c_long(0)
        check(load().unap_cuda_server_create(ctypes.byref(h), memory_budget, max_slots,
                                             small_cells))
        self.handle = h.value
        self._cells = {}  # request id -> nCells (the size of x that wait() fills)

    def submit(self, system, method, rel_tol=1e-8, max_iter=1000):
        l = _i32(system.lower_addr)
        u = _i32(system.upper_addr)
        lo = None if system.symm else _f64(system.lower)
        d = _f64(system.diag)
        up = _f64(system.upper)
        b = _f64(system.b)
        rid = _c_ll(0)
        m = SERVE_METHODS[method] if isinstance(method, str) else method
        check(load().unap_cuda_server_submit(self.handle, system.n, system.nf, l.ctypes.data,
                                             u.ctypes.data,
                                             None if lo is None else lo.ctypes.data,
                                             d.ctypes.data, up.ctypes.data, b.ctypes.data, m,
                                             rel_tol, max_iter, ctypes.byref(rid)))
        self._cells[rid.value] = int(system.n)
        return rid.value

    def wait(self, rid, n=None):
        cells = self._cells.pop(rid, None)
        if n is not None and cells is not None and n != cells:
            self._cells[rid] = cells
            raise ValueError(f"request {rid} has {cells} cells, not {n}")
        if cells is None and n is None:
            raise ValueError(f"unknown request {rid}: pass its number of cells")
        x = np.zeros(cells if cells is not None else n)
        info = RequestInfo()
        check(load().unap_cuda_server_wait(self.handle, rid, x.ctypes.data, ctypes.byref(info)))
        return x, info.as_dict()

    def close(self):
        if self.handle:
            check(load().unap_cuda_server_destroy(self.handle))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceMG:
    """The reference's MGSolver on a DeviceMatrix (``unap_cuda_mg_*``)."""

    def __init__(self, matrix, weights=None, smoother=1, n_coarsest=-1, max_levels=-1,
                 n_pre=-1, n_post=-1, n_finest=-1, scale_corr=-1, tol=0.0, rel_tol=1e-6,
                 max_iter=1000, min_iter=0):
        lib = load()
        self._w = None if weights is None else _f64(weights)
        h = _c_long(0)
        check(lib.unap_cuda_mg_create(ctypes.byref(h), matrix.handle,
                                      None if self._w is None else self._w.ctypes.data,
                                      smoother, n_coarsest, max_levels, n_pre, n_post, n_finest,
                                      scale_corr, tol, rel_tol, max_iter, min_iter))
        self.handle = h.value

    def levels(self):
        n = _c_int()
        cells = np.zeros(64, np.int32)
        check(load().unap_cuda_mg_levels(self.handle, ctypes.byref(n), cells.ctypes.data, 64))
        return cells[:n.value + 1].tolist()

    def solve(self, x, b):
        st = Stats()
        check(load().unap_cuda_mg_solve(self.handle, _ptr(x), _ptr(b), ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        if self.handle:
            check(load().unap_cuda_mg_destroy(self.handle))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_executor(persistent: bool) -> bool:
    """Executor of PCG solves created afterwards; returns the previous one."""
    return bool(load().unap_cuda_set_executor(1 if persistent else 0))


def set_host_wait(mode: int) -> None:
    """How host threads wait for the GPU: 0 default, 1 spin, 2 yield, 3
    blocking; call before the first CUDA work of the process."""
    check(load().unap_cuda_set_host_wait(int(mode)))


def set_team_solve_cells(cells: int) -> int:
    """Systems of at most `cells` cells with an LDU preconditioner are solved
    by one whole-solve launch (0: never); returns the previous value."""
    return int(load().unap_cuda_set_team_solve_cells(int(cells)))


def set_cheby_tail_rows(rows: int) -> int:
    """Chebyshev V-cycles run their levels of at most `rows` rows (and all
    below) in one cluster launch (0: never), for AMG handles created
    afterwards; returns the previous value."""
    return int(load().unap_cuda_set_cheby_tail_rows(int(rows)))


def set_server_graphs(on: bool) -> bool:
    """Server slots replay Krylov iterations from CUDA graphs (default) or
    launch kernel by kernel; returns the previous setting."""
    return bool(load().unap_cuda_set_server_graphs(1 if on else 0))


def set_server_amg(n_coarsest: int = 200, eig_ratio: float = 30.0) -> None:
    """Server AMG requests: coarsest level target and Chebyshev ratio."""
    check(load().unap_cuda_set_server_amg(int(n_coarsest), float(eig_ratio)))


def set_server_team_cells(cells: int) -> int:
    """Server slots solve PCG/PBiCGStab requests of up to `cells` cells in
    one whole-solve launch (0: never); returns the previous value."""
    return int(load().unap_cuda_set_server_team_cells(int(cells)))


def force_team_shape(threads: int, cluster: int = 1) -> None:
    """Whole-solve launches use this shape from now on (threads 0: back to
    the autotuner)."""
    check(load().unap_cuda_force_team_shape(int(threads), int(cluster)))


def team_shape(cells: int, systems: int = 1):
    """The autotuner's cached (CTA size, CTAs per system) for `systems`
    systems of up to `cells` cells; (0, 0) when not tuned yet."""
    t, c = ctypes.c_int(0), ctypes.c_int(0)
    check(load().unap_cuda_team_shape(int(cells), int(systems), ctypes.byref(t), ctypes.byref(c)))
    return t.value, c.value


def set_wave_pdl(on: bool) -> bool:
    """Programmatic dependent launch of wavefront kernels; returns the previous value."""
    return bool(load().unap_cuda_set_wave_pdl(1 if on else 0))


def set_wave_grid(one_row_per_thread: bool) -> bool:
    """Wavefront kernel grids: one row per thread, or a capped grid-stride loop."""
    return bool(load().unap_cuda_set_wave_grid(1 if one_row_per_thread else 0))


def set_packed_sweeps(mode) -> int:
    """V-cycle sweeps on long-row levels from the row-packed copy: 1 (or True)
    register window by mean row length, 2 always 16/8 entries, 3 always
    24/12, 0 (or False) SELL-32 rows."""
    return int(load().unap_cuda_set_packed_sweeps(int(mode)))


def set_cheby_small_rows(rows: int) -> int:
    """Chebyshev-step launches on levels of at most `rows` rows use one-warp
    CTAs; returns the previous threshold."""
    return int(load().unap_cuda_set_cheby_small_rows(int(rows)))


def set_matrix_wavefronts(on: bool) -> bool:
    """Wavefront ranges for matrices created afterwards (False: locality
    order only, SpMV-shaped work only); returns the previous value."""
    return bool(load().unap_cuda_set_matrix_wavefronts(1 if on else 0))


def set_cheby_chunk(entries: int) -> int:
    """Entries per load round trip of the Chebyshev step (0 auto, 8, 16);
    returns the previous value."""
    rc = int(load().unap_cuda_set_cheby_chunk(int(entries)))
    if rc < 0:
        check(rc)
    return rc


def set_tail_rows(tail_rows: int, single_rows: int, precision: int | None = None):
    """Thresholds of the AMG V-cycle's cluster tail kernel (0 disables it) for
    the FP64 (0) or FP32 (1) V-cycle, or both (None).  Returns the previous
    settings as {precision: (tail_rows, single_rows)}, which
    restore_tail_rows() puts back."""
    old = {}
    for p in ((0, 1) if precision is None else (precision,)):
        ot, os_ = _c_ll(), _c_ll()
        check(load().unap_cuda_set_tail_rows(p, int(tail_rows), int(single_rows),
                                             ctypes.byref(ot), ctypes.byref(os_)))
        old[p] = (ot.value, os_.value)
    return old


def restore_tail_rows(old) -> None:
    """Put back settings returned by set_tail_rows()."""
    for p, (t, s) in old.items():
        check(load().unap_cuda_set_tail_rows(p, int(t), int(s), None, None))


def get_tail_rows(precision: int) -> tuple[int, int]:
    """Current (tail_rows, single_rows) of the FP64 (0) or FP32 (1) V-cycle."""
    old = set_tail_rows(0, 0, precision)
    restore_tail_rows(old)
    return old[precision]


def set_device_setup(min_cells: int) -> int:
    """Matrices and AMG levels of at least min_cells cells build their device
    structure with kernels (< 0: all on the host); returns the old value."""
    old = _c_ll()
    check(load().unap_cuda_set_device_setup(int(min_cells), ctypes.byref(old)))
    return old.value


def _layout(fn, *head):
    nw = _c_int()
    n = _c_int()
    if fn == "unap_cuda_matrix_layout":
        lib = load()
        check(lib.unap_cuda_matrix_layout(*head, ctypes.byref(nw), None, None))
        info = _c_int()
        size = _c_int()
        check(lib.unap_cuda_matrix_size(*head, ctypes.byref(size), ctypes.byref(info), None))
        perm = np.zeros(size.value, np.int32)
        ws = np.zeros(nw.value + 1, np.int32)
        check(lib.unap_cuda_matrix_layout(*head, ctypes.byref(nw), perm.ctypes.data,
                                          ws.ctypes.data))
        return perm, ws
    lib = load()
    check(lib.unap_cuda_amg_level_layout(*head, ctypes.byref(n), None, ctypes.byref(nw), None,
                                         None))
    perm = np.zeros(n.value, np.int32)
    ws = np.zeros(nw.value + 1, np.int32)
    check(lib.unap_cuda_amg_level_layout(*head, ctypes.byref(n), None, ctypes.byref(nw),
                                         perm.ctypes.data, ws.ctypes.data))
    return perm, ws


def tail_cluster_size() -> int:
    """CTAs per cluster of the tail kernel on the current device (0: none)."""
    c = _c_int()
    check(load().unap_cuda_tail_cluster_size(ctypes.byref(c)))
    return c.value


class AmgParams(ctypes.Structure):
    _fields_ = [("nCoarsest", _c_int), ("maxLevels", _c_int), ("nPreSweeps", _c_int),
                ("nPostSweeps", _c_int), ("precision", _c_int), ("flexible", _c_int),
                ("tol", _c_dbl), ("relTol", _c_dbl), ("maxIter", _c_int), ("minIter", _c_int),
                ("smoother", _c_int), ("chebyDegree", _c_int), ("chebyFrom", _c_int),
                ("eigRatio", _c_dbl), ("fusedOuter", _c_int)]


class DeviceAmg:
    """AMG-preconditioned PCG on a DeviceMatrix (``unap_cuda_amg_*``)."""

    def __init__(self, matrix: "DeviceMatrix", **kw):
        lib = load()
        self.params = AmgParams()
        lib.unap_cuda_amg_default_params(ctypes.byref(self.params))
        if kw.get("precision", 0) == 1 and "flexible" not in kw:
            kw["flexible"] = 1
        names = dict(n_coarsest="nCoarsest", max_levels="maxLevels", n_pre="nPreSweeps",
                     n_post="nPostSweeps", precision="precision", flexible="flexible",
                     tol="tol", rel_tol="relTol", max_iter="maxIter", min_iter="minIter",
                     smoother="smoother", cheby_degree="chebyDegree", cheby_from="chebyFrom",
                     eig_ratio="eigRatio", fused_outer="fusedOuter")
        for k, v in kw.items():
            setattr(self.params, names[k], v)
        h = _c_long(0)
        check(lib.unap_cuda_amg_create(ctypes.byref(h), matrix.handle, ctypes.byref(self.params)))
        self.handle = h.value
        self.matrix = matrix

    def info(self):
        n = _c_int()
        cells = np.zeros(64, np.int32)
        waves = np.zeros(64, np.int32)
        t = _c_dbl()
        b = _c_ll()
        check(load().unap_cuda_amg_info(self.handle, ctypes.byref(n), cells.ctypes.data,
                                        waves.ctypes.data, 64, ctypes.byref(t), ctypes.byref(b)))
        return dict(n_levels=n.value, cells=cells[:n.value].tolist(),
                    wavefronts=waves[:n.value].tolist(), setup_s=t.value, device_bytes=b.value)

    def level_layout(self, level: int):
        """(perm, waveStart) of AMG level `level` (0 = the matrix)."""
        return _layout("unap_cuda_amg_level_layout", self.handle, level)

    def level_sizes(self):
        """[(cells, faces, wavefronts)] of every level, finest first."""
        lib = load()
        out = []
        for k in range(self.info()["n_levels"]):
            n, nw, nf = _c_int(), _c_int(), _c_ll()
            check(lib.unap_cuda_amg_level_layout(self.handle, k, ctypes.byref(n), ctypes.byref(nf),
                                                 ctypes.byref(nw), None, None))
            out.append((n.value, nf.value, nw.value))
        return out

    def vcycle(self, r, z):
        check(load().unap_cuda_amg_vcycle(self.handle, _ptr(r), _ptr(z)))

    def profile_smoother(self, level: int, reps: int = 10):
        """(ms, algorithmic bytes, launches) of one smoothing launch group on
        `level` (see unap_cuda_amg_profile_smoother)."""
        ms, b, n = _c_dbl(), _c_dbl(), _c_int()
        check(load().unap_cuda_amg_profile_smoother(self.handle, level, reps, ctypes.byref(ms),
                                                    ctypes.byref(b), ctypes.byref(n)))
        return ms.value, b.value, n.value

    def setup_phases(self):
        """Host wall time (s) of the setup phases: agglomeration, levels,
        coarsest, vectors, packing, eigenvalues."""
        t = np.zeros(6)
        check(load().unap_cuda_amg_setup_phases(self.handle, t.ctypes.data))
        return dict(zip(["agglomerate", "levels", "coarsest", "vectors", "pack", "eigen"],
                        t.tolist()))

    def eigenvalues(self):
        """Chebyshev eigenvalue estimate of every level but the coarsest
        (0 on Gauss-Seidel levels)."""
        lam = np.zeros(64)
        w = _c_int()
        check(load().unap_cuda_amg_eigenvalues(self.handle, lam.ctypes.data, 64, ctypes.byref(w)))
        return lam[:w.value].copy()

    def profile_vcycle(self, reps=10):
        """Mean V-cycle ms and per-level ms (see unap_cuda_amg_profile_vcycle)."""
        ms = np.zeros(65)
        w = _c_int()
        check(load().unap_cuda_amg_profile_vcycle(self.handle, reps, ms.ctypes.data, 65,
                                                  ctypes.byref(w)))
        return {"vcycle_ms": float(ms[0]), "level_ms": ms[1:w.value].tolist()}

    def solve(self, x, b):
        st = Stats()
        check(load().unap_cuda_amg_solve(self.handle, _ptr(x), _ptr(b), ctypes.byref(st)))
        return st.as_dict()

    def solve_host(self, x, b):
        st = Stats()
        check(load().unap_cuda_amg_solve_host(self.handle, _ptr(x), _ptr(b), ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        if self.handle:
            check(load().unap_cuda_amg_destroy(self.handle))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libunap_cuda.so (building it first if it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise UnapCudaError(f"{path} is not built")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        msg = load().unap_cuda_last_error().decode(errors="replace")
        raise UnapCudaError(f"unap_cuda error {rc}: {msg}")


def _ptr(t) -> int | None:
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _as_ip(a):
    return a.ctypes.data_as(_ip)


def _as_dp(a):
    return a.ctypes.data_as(_dp)


class DeviceMatrix:
    """An LDU matrix resident on the GPU (``unap_cuda_matrix_create``)."""

    def __init__(self, system):
        lib = load()
        self._keep = (_i32(system.lower_addr), _i32(system.upper_addr),
                      None if system.symm else _f64(system.lower), _f64(system.diag),
                      _f64(system.upper))
        l, u, lo, d, up = self._keep
        h = _c_long(0)
        check(lib.unap_cuda_matrix_create(ctypes.byref(h), system.n, system.nf, l.ctypes.data,
                                          u.ctypes.data, None if lo is None else lo.ctypes.data,
                                          d.ctypes.data, up.ctypes.data))
        self.handle = h.value
        self.n = system.n
        self._keep = None

    def info(self):
        w = _c_int()
        e = _c_ll()
        b = _c_ll()
        check(load().unap_cuda_matrix_info(self.handle, ctypes.byref(w), ctypes.byref(e),
                                           ctypes.byref(b)))
        return dict(n_wavefronts=w.value, n_entries=e.value, device_bytes=b.value)

    def layout(self):
        """(perm, waveStart): internal row i holds cell perm[i]."""
        return _layout("unap_cuda_matrix_layout", self.handle)

    def spmv(self, x, y):
        check(load().unap_cuda_spmv(self.handle, _ptr(x), _ptr(y)))

    def precondition(self, ptype, r, w):
        check(load().unap_cuda_precondition(self.handle, ptype, _ptr(r), _ptr(w)))

    def gauss_seidel(self, x, b, n_sweeps, backward=False):
        check(load().unap_cuda_gauss_seidel(self.handle, _ptr(x), _ptr(b), n_sweeps,
                                            1 if backward else 0))

    def krylov_solve(self, method, precond, x, b, tol=0.0, rel_tol=1e-6, max_iter=1000,
                     min_iter=0):
        st = Stats()
        check(load().unap_cuda_krylov_solve(self.handle, method, precond, tol, rel_tol,
                                            max_iter, min_iter, _ptr(x), _ptr(b),
                                            ctypes.byref(st)))
        return st.as_dict()

    def profile(self, reps=20):
        ms = np.zeros(8)
        check(load().unap_cuda_profile_kernels(self.handle, reps, ms.ctypes.data))
        keys = ["spmv", "dic_apply", "dilu_apply", "gs_fwd", "gs_bwd", "spmv32", "gs_fwd32",
                "residual"]
        return dict(zip(keys, ms.tolist()))

    def close(self):
        if self.handle:
            check(load().unap_cuda_matrix_destroy(self.handle))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- the reference's Fortran-convention calls, host arrays ----------------

def ldumatrixcreat(system) -> int:
    """ldumatrixcreat_ (fortranInterface.cpp:31-71); returns the handle."""
    lib = load()
    h = _c_long(0)
    n = _c_int(system.n)
    nf = _c_int(system.nf)
    l = _i32(system.lower_addr)
    u = _i32(system.upper_addr)
    up = _f64(system.upper)
    lo = up if system.symm else _f64(system.lower)
    d = _f64(system.diag)
    lib.ldumatrixcreat_(ctypes.byref(h), ctypes.byref(n), ctypes.byref(nf), _as_ip(l), _as_ip(u),
                        _as_dp(lo), _as_dp(d), _as_dp(up))
    if not h.value:
        raise UnapCudaError(load().unap_cuda_last_error().decode())
    return h.value


def _krylov_oneshot(fn_name, x, handle, b, precond, tol, rel_tol, max_iter, min_iter):
    lib = load()
    x = _f64(x)
    b = _f64(b)
    h = _c_long(handle)
    n = _c_int(x.shape[0])
    it = _c_int(0)
    res = _c_dbl(0)
    getattr(lib, fn_name)(_as_dp(x), ctypes.byref(h), _as_dp(b), ctypes.byref(n),
                          ctypes.byref(_c_int(precond)), ctypes.byref(_c_dbl(tol)),
                          ctypes.byref(_c_dbl(rel_tol)), ctypes.byref(_c_int(max_iter)),
                          ctypes.byref(_c_int(min_iter)), ctypes.byref(it), ctypes.byref(res))
    return x, it.value, res.value


def pcgsolversolve(x, handle, b, precond, tol=0.0, rel_tol=1e-6, max_iter=1000, min_iter=0):
    """pcgsolversolve_ (fortranInterface.cpp:200-268).  Consumes the handle."""
    return _krylov_oneshot("pcgsolversolve_", x, handle, b, precond, tol, rel_tol, max_iter,
                           min_iter)


def pbicgstabsolversolve(x, handle, b, precond, tol=0.0, rel_tol=1e-6, max_iter=1000,
                         min_iter=0):
    """pbicgstabsolversolve_ (fortranInterface.cpp:271-346).  Consumes the handle."""
    return _krylov_oneshot("pbicgstabsolversolve_", x, handle, b, precond, tol, rel_tol,
                           max_iter, min_iter)


def handle_ldu(handle: int) -> dict:
    """Host copy of a matrix handle's LDU arrays (no GPU work)."""
    lib = load()
    n = _c_int()
    nf = _c_int()
    sy = _c_int()
    check(lib.unap_cuda_matrix_size(handle, ctypes.byref(n), ctypes.byref(nf), ctypes.byref(sy)))
    l = np.zeros(nf.value, np.int32)
    u = np.zeros(nf.value, np.int32)
    lo = np.zeros(nf.value)
    up = np.zeros(nf.value)
    d = np.zeros(n.value)
    check(lib.unap_cuda_matrix_get_ldu(handle, l.ctypes.data, u.ctypes.data, lo.ctypes.data,
                                       d.ctypes.data, up.ctypes.data))
    return dict(n=n.value, nf=nf.value, symm=bool(sy.value), lower_addr=l, upper_addr=u,
                lower=lo, diag=d, upper=up)


def coo2ldumatrixcreat(data, rows_1based, cols_1based, n_cells, symm) -> int:
    """coo2ldumatrixcreat_ (fortranInterface.cpp:74-120); returns the handle."""
    lib = load()
    h = _c_long(0)
    d = _f64(data)
    r = _i32(rows_1based)
    c = _i32(cols_1based)
    lib.coo2ldumatrixcreat_(ctypes.byref(h), _as_dp(d), _as_ip(r), _as_ip(c),
                            ctypes.byref(_c_int(n_cells)), ctypes.byref(_c_int(d.shape[0])),
                            ctypes.byref(_c_int(1 if symm else 0)))
    if not h.value:
        raise UnapCudaError(lib.unap_cuda_last_error().decode())
    return h.value


def sw_matrix_destroy(handle: int) -> None:
    load().sw_matrix_destroy__(ctypes.byref(_c_long(handle)))


# ---- text dumps in the reference's on-disk formats (host only)

def _path(p) -> bytes:
    return os.fsencode(p)


def read_ldu_matrix(file_name) -> int:
    """constructLDUMatrixFromOpenFOAM (readFromOpenFOAM.cpp:9-139): a matrix
    handle read from an LDU text dump (destroy with sw_matrix_destroy)."""
    lib = load()
    h = _c_long(0)
    check(lib.unap_cuda_read_ldu_matrix(_path(file_name), ctypes.byref(h)))
    return h.value


def read_vector(file_name, n: int) -> np.ndarray:
    """constructVectorFromOpenFOAM (readFromOpenFOAM.cpp:142-204) into a new
    array of n values; the file's count must equal n."""
    v = np.zeros(n)
    check(load().unap_cuda_read_vector(_path(file_name), n, v.ctypes.data))
    return v


def read_interfaces(file_name) -> dict:
    """constructLDUInterfacesFromOpenFOAM (readFromOpenFOAM.cpp:207-322):
    per-neighbour ranks and sizes, then every face's cell and (negated)
    coefficient."""
    lib = load()
    np_ = _c_int()
    nf = _c_ll()
    check(lib.unap_cuda_read_interfaces(_path(file_name), ctypes.byref(np_), ctypes.byref(nf),
                                        None, None, None, None))
    nb = np.zeros(np_.value, np.int32)
    sz = np.zeros(np_.value, np.int32)
    fc = np.zeros(nf.value, np.int32)
    co = np.zeros(nf.value)
    check(lib.unap_cuda_read_interfaces(_path(file_name), ctypes.byref(np_), ctypes.byref(nf),
                                        nb.ctypes.data, sz.ctypes.data, fc.ctypes.data,
                                        co.ctypes.data))
    return dict(neighbour=nb, size=sz, face_cells=fc, coeffs=co)


def print_ldu_matrix(handle: int, name) -> str:
    """printLDUMatrix (printUNAP.cpp:8-58); returns the file written."""
    check(load().unap_cuda_print_ldu_matrix(handle, _path(name)))
    return os.fsdecode(_path(name)) + "_0.txt"


def print_vector(v, name) -> str:
    """printVector (printUNAP.hpp:27-42); returns the file written."""
    a = _f64(v)
    check(load().unap_cuda_print_vector(_path(name), a.shape[0], a.ctypes.data))
    return os.fsdecode(_path(name)) + "_0.txt"


def print_interfaces(name, neighbour, size, face_cells, coeffs) -> str:
    """printInterfaces (printUNAP.cpp:61-87); returns the file written."""
    nb, sz, fc = _i32(neighbour), _i32(size), _i32(face_cells)
    co = _f64(coeffs)
    if int(sz.sum()) != fc.shape[0] or fc.shape[0] != co.shape[0] or nb.shape != sz.shape:
        raise ValueError("interface arrays disagree in size")
    check(load().unap_cuda_print_interfaces(_path(name), nb.shape[0], nb.ctypes.data,
                                            sz.ctypes.data, fc.ctypes.data, co.ctypes.data))
    return os.fsdecode(_path(name)) + "_0.txt"
