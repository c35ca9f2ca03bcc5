"""ctypes access to the two CPU oracles (test infrastructure).

* ``Oracle("orc")`` loads oracle/liboracle.so, the C restatement of the
  reference path (built by oracle/Makefile, on any host).
* ``Oracle("ref")`` loads oracle/_ref/libunap_ref.so, the reference UNAP
  sources compiled in place with a serial MPI shim.  It only exists where the
  reference tree was available at build time; `ref_available()` says so.

Both expose the same function signatures with a different prefix, so a test
can run the same call through either and compare.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORC_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libunap_ref.so")

_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p


def build_oracle() -> None:
    if not os.path.exists(ORC_SO) or os.path.getmtime(ORC_SO) < max(
            os.path.getmtime(os.path.join(ORACLE_DIR, f))
            for f in ("unap_oracle.c", "unap_oracle.h")):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(_vp)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    def __init__(self, prefix: str = "orc"):
        if prefix == "orc":
            build_oracle()
            self.lib = ctypes.CDLL(ORC_SO)
        else:
            self.lib = ctypes.CDLL(REF_SO)
        self.prefix = prefix
        # attribute access caches the function object, so restype sticks
        # (indexing, lib["name"], returns a new object on every call)
        getattr(self.lib, f"{prefix}_eigen").restype = _c_dbl
        getattr(self.lib, f"{prefix}_aggl_create" if prefix == "ref"
                else f"{prefix}_hier_create").restype = _vp
        if prefix == "ref":
            self.lib.ref_coo2ldu.restype = _vp
        else:
            self.lib.orc_amg_create.restype = _vp

    def _f(self, name):
        return getattr(self.lib, f"{self.prefix}_{name}")

    @staticmethod
    def _mat(s):
        lo = None if s.symm else _f64(s.lower)
        return [_c_int(s.n), _c_int(s.nf), _p(_i32(s.lower_addr)), _p(_i32(s.upper_addr)),
                _p(lo), _p(_f64(s.diag)), _p(_f64(s.upper)), _c_int(1 if s.symm else 0)]

    # keep numpy temporaries alive across the call
    def _call(self, name, s, *rest):
        l = _i32(s.lower_addr)
        u = _i32(s.upper_addr)
        lo = None if s.symm else _f64(s.lower)
        d = _f64(s.diag)
        up = _f64(s.upper)
        args = [_c_int(s.n), _c_int(s.nf), _p(l), _p(u), _p(lo), _p(d), _p(up),
                _c_int(1 if s.symm else 0)]
        return self._f(name)(*args, *rest)

    def spmv(self, s, x):
        y = np.zeros(s.n)
        x = _f64(x)
        self._call("spmv", s, _p(x), _p(y))
        return y

    def losort(self, s):
        los = np.zeros(s.nf, np.int32)
        os_ = np.zeros(s.n + 1, np.int32)
        lss = np.zeros(s.n + 1, np.int32)
        l = _i32(s.lower_addr)
        u = _i32(s.upper_addr)
        self._f("losort")(_c_int(s.n), _c_int(s.nf), _p(l), _p(u), _p(los), _p(os_), _p(lss))
        return los, os_, lss

    def precond(self, ptype, s, r):
        w = np.zeros(s.n)
        rD = np.zeros(s.n)
        r = _f64(r)
        l = _i32(s.lower_addr)
        u = _i32(s.upper_addr)
        lo = None if s.symm else _f64(s.lower)
        d = _f64(s.diag)
        up = _f64(s.upper)
        self._f("precond")(_c_int(ptype), _c_int(s.n), _c_int(s.nf), _p(l), _p(u), _p(lo),
                           _p(d), _p(up), _c_int(1 if s.symm else 0), _p(r), _p(w), _p(rD))
        return w, rD

    def gs(self, s, x, b, n_sweeps, backward=False):
        x = _f64(x).copy()
        b = _f64(b)
        self._call("gs_bwd" if backward else "gs", s, _p(x), _p(b), _c_int(n_sweeps))
        return x

    def cheby(self, s, x, b, n_sweeps, n_calls):
        x = _f64(x).copy()
        b = _f64(b)
        self._call("cheby", s, _p(x), _p(b), _c_int(n_sweeps), _c_int(n_calls))
        return x

    def cheby_chain(self, s, x, b, lam, ratio, degree, from_zero=False):
        """The AMG levels' Chebyshev chain (FP64, new component) on one
        matrix with a given eigenvalue estimate."""
        x = _f64(x).copy()
        b = _f64(b)
        self._call("cheby_chain", s, _c_dbl(lam), _c_dbl(ratio), _c_int(degree), _p(x), _p(b),
                   _c_int(1 if from_zero else 0))
        return x

    def eig_start(self, n):
        f = self.lib.orc_eig_start
        f.restype = _c_dbl
        f.argtypes = [ctypes.c_longlong]
        return np.array([f(c) for c in range(n)])

    def eigen(self, s, x, b, n_pcg=10):
        x = _f64(x).copy()
        b = _f64(b)
        e = self._call("eigen", s, _p(x), _p(b), _c_int(n_pcg))
        return e, x

    def _krylov(self, name, s, precond, b, x0=None, tol=0.0, rel_tol=1e-6, max_iter=1000,
                min_iter=0):
        x = np.zeros(s.n) if x0 is None else _f64(x0).copy()
        b = _f64(b)
        it = _c_int()
        ir = _c_dbl()
        fr = _c_dbl()
        cv = _c_int()
        sg = _c_int()
        self._call(name, s, _c_int(precond), _c_dbl(tol), _c_dbl(rel_tol), _c_int(max_iter),
                   _c_int(min_iter), _p(x), _p(b), ctypes.byref(it), ctypes.byref(ir),
                   ctypes.byref(fr), ctypes.byref(cv), ctypes.byref(sg))
        return x, dict(n_iter=it.value, init_res=ir.value, final_res=fr.value,
                       converged=bool(cv.value), singular=bool(sg.value))

    def pcg(self, s, precond, b, **kw):
        return self._krylov("pcg", s, precond, b, **kw)

    def pbicgstab(self, s, precond, b, **kw):
        return self._krylov("pbicgstab", s, precond, b, **kw)

    def hierarchy(self, s, weights, n_coarsest=50, max_levels=50, stop_rule=0):
        """List of coarse levels, each a dict of restrict/faceRestrict maps,
        coarse addressing and coefficients."""
        l = _i32(s.lower_addr)
        u = _i32(s.upper_addr)
        lo = None if s.symm else _f64(s.lower)
        d = _f64(s.diag)
        up = _f64(s.upper)
        w = _f64(weights)
        base = [_c_int(s.n), _c_int(s.nf), _p(l), _p(u), _p(lo), _p(d), _p(up),
                _c_int(1 if s.symm else 0), _p(w), _c_int(n_coarsest), _c_int(max_levels)]
        if self.prefix == "ref":
            h = self.lib.ref_aggl_create(*base)
            nl, nc, nfc = self.lib.ref_aggl_nlevels, self.lib.ref_aggl_ncells, self.lib.ref_aggl_nfaces
            addr, coeffs, destroy = (self.lib.ref_aggl_addressing, self.lib.ref_aggl_coeffs,
                                     self.lib.ref_aggl_destroy)
        else:
            h = self.lib.orc_hier_create(*base, _c_int(stop_rule))
            nl, nc, nfc = self.lib.orc_hier_nlevels, self.lib.orc_hier_ncells, self.lib.orc_hier_nfaces
            addr, coeffs, destroy = (self.lib.orc_hier_addressing, self.lib.orc_hier_coeffs,
                                     self.lib.orc_hier_destroy)
        h = _vp(h)
        levels = []
        n_fine, nf_fine = s.n, s.nf
        for k in range(nl(h)):
            n = nc(h, k)
            nf = nfc(h, k)
            ra = np.zeros(n_fine, np.int32)
            fr = np.zeros(nf_fine, np.int32)
            cl = np.zeros(nf, np.int32)
            cu = np.zeros(nf, np.int32)
            addr(h, _c_int(k), _p(ra), _p(fr), _p(cl), _p(cu))
            dg = np.zeros(n)
            upc = np.zeros(nf)
            loc = np.zeros(nf)
            coeffs(h, _c_int(k), _p(dg), _p(upc), _p(loc))
            levels.append(dict(n=n, nf=nf, restrict=ra, face_restrict=fr, lower_addr=cl,
                               upper_addr=cu, diag=dg, upper=upc, lower=loc))
            n_fine, nf_fine = n, nf
        destroy(h)
        return levels

    def mg(self, s, b, weights, x0=None, n_coarsest=50, max_levels=50, smoother=1, n_pre=-1,
           n_post=-1, n_finest=-1, scale_corr=-1, tol=0.0, rel_tol=1e-6, max_iter=1000,
           min_iter=0):
        x = np.zeros(s.n) if x0 is None else _f64(x0).copy()
        b = _f64(b)
        w = _f64(weights)
        it = _c_int()
        ir = _c_dbl()
        fr = _c_dbl()
        cv = _c_int()
        nl = _c_int()
        self._call("mg", s, _p(w), _c_int(n_coarsest), _c_int(max_levels), _c_int(smoother),
                   _c_int(n_pre), _c_int(n_post), _c_int(n_finest), _c_int(scale_corr),
                   _c_dbl(tol), _c_dbl(rel_tol), _c_int(max_iter), _c_int(min_iter), _p(x),
                   _p(b), ctypes.byref(it), ctypes.byref(ir), ctypes.byref(fr),
                   ctypes.byref(cv), ctypes.byref(nl))
        return x, dict(n_iter=it.value, init_res=ir.value, final_res=fr.value,
                       converged=bool(cv.value), n_levels=nl.value)


class AmgParams(ctypes.Structure):
    _fields_ = [("nCoarsest", _c_int), ("maxLevels", _c_int), ("nPre", _c_int),
                ("nPost", _c_int), ("precision", _c_int), ("flexible", _c_int),
                ("tol", _c_dbl), ("relTol", _c_dbl), ("maxIter", _c_int), ("minIter", _c_int),
                ("smoother", _c_int), ("chebyDegree", _c_int), ("chebyFrom", _c_int),
                ("eigRatio", _c_dbl)]


class OracleAmg:
    """The C oracle's AMG-PCG (new component; no reference counterpart)."""

    def __init__(self, orc: Oracle, s, n_coarsest=1000, max_levels=50, n_pre=2, n_post=2,
                 precision=0, flexible=0, tol=0.0, rel_tol=1e-10, max_iter=500, min_iter=0,
                 smoother=0, cheby_degree=3, cheby_from=0, eig_ratio=0.0):
        assert orc.prefix == "orc" and s.symm
        self.lib = orc.lib
        self.s = s
        self._keep = [_i32(s.lower_addr), _i32(s.upper_addr), _f64(s.diag), _f64(s.upper)]
        self.params = AmgParams(n_coarsest, max_levels, n_pre, n_post, precision, flexible,
                                tol, rel_tol, max_iter, min_iter, smoother, cheby_degree,
                                cheby_from, eig_ratio)
        l, u, d, up = self._keep
        self.h = _vp(self.lib.orc_amg_create(_c_int(s.n), _c_int(s.nf), _p(l), _p(u), _p(d),
                                             _p(up), ctypes.byref(self.params)))

    @property
    def n_levels(self):
        return self.lib.orc_amg_nlevels(self.h)

    def level_sizes(self):
        return [self.lib.orc_amg_ncells(self.h, _c_int(k)) for k in range(self.n_levels)]

    def vcycle(self, r):
        z = np.zeros(self.s.n)
        r = _f64(r)
        self.lib.orc_amg_vcycle(self.h, _p(r), _p(z))
        return z

    def coarse_inverse(self):
        nc = self.level_sizes()[-1]
        inv = np.zeros((nc, nc))
        self.lib.orc_amg_coarse_inverse(self.h, _p(inv))
        return inv

    def solve(self, b, x0=None):
        x = np.zeros(self.s.n) if x0 is None else _f64(x0).copy()
        b = _f64(b)
        it = _c_int()
        ir = _c_dbl()
        fr = _c_dbl()
        tr = _c_dbl()
        cv = _c_int()
        self.lib.orc_amg_pcg(self.h, _p(x), _p(b), ctypes.byref(it), ctypes.byref(ir),
                             ctypes.byref(fr), ctypes.byref(tr), ctypes.byref(cv))
        return x, dict(n_iter=it.value, init_res=ir.value, final_res=fr.value,
                       true_res=tr.value, converged=bool(cv.value))

    def eigs(self):
        """Per-level eigenvalue estimates of the Chebyshev smoother (0 where
        a level uses Gauss-Seidel), levels 0 .. n_levels - 2."""
        lam = np.zeros(max(self.n_levels - 1, 1))
        self.lib.orc_amg_eigs(self.h, _p(lam))
        return lam[:self.n_levels - 1]

    def set_eigs(self, lam) -> None:
        lam = _f64(np.resize(np.asarray(lam, dtype=np.float64), max(self.n_levels - 1, 1)))
        self.lib.orc_amg_set_eigs(self.h, _p(lam))

    def set_max_iter(self, k: int) -> None:
        self.lib.orc_amg_set_max_iter(self.h, _c_int(k))

    def close(self):
        if self.h:
            self.lib.orc_amg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
