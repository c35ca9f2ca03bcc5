"""Generate tests/golden/reference_small.npz from the reference build.

Runs the reference UNAP library itself (oracle/_ref/libunap_ref.so, the x86
sources compiled in place by ``make -C oracle ref``) on small seeded LDU
systems and stores inputs and outputs, so the C restatement and the GPU path
can be pinned against reference results on hosts where the reference tree is
absent.  Re-run with ``python tests/golden/make_golden.py`` after
``make -C oracle ref``.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle_lib import Oracle, ref_available  # noqa: E402
from unap_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "reference_small.npz")


def cases():
    return [
        W.laplace(6, 5, 4, seed=11, permute=False),
        W.laplace(7, 6, 5, seed=12, permute=True, rhs="normal"),
        W.convdiff(6, 5, 4, seed=13, permute=True, pe=5.0),
        W.lognormal(8, seed=14, permute=True, sigma=2.0),
    ]


def mg_weights(s):
    return np.abs(s.upper) / np.sqrt(np.sum(s.upper ** 2))


def generate(ref):
    """Every fixture array, computed by the reference library `ref`."""
    out = {}
    for ci, s in enumerate(cases()):
        k = f"c{ci}/"
        rng = np.random.default_rng(100 + ci)
        x = rng.standard_normal(s.n)
        out[k + "n"] = np.array(s.n)
        out[k + "lower_addr"] = s.lower_addr
        out[k + "upper_addr"] = s.upper_addr
        out[k + "upper"] = s.upper
        out[k + "lower"] = s.upper if s.symm else s.lower
        out[k + "symm"] = np.array(1 if s.symm else 0)
        out[k + "diag"] = s.diag
        out[k + "b"] = s.b
        out[k + "x"] = x
        out[k + "spmv"] = ref.spmv(s, x)
        for t in (1, 2, 3):
            w, rD = ref.precond(t, s, x)
            out[k + f"precond{t}_w"] = w
            out[k + f"precond{t}_rD"] = rD
        out[k + "gs3"] = ref.gs(s, x, s.b, 3)
        out[k + "cheby3x3"] = ref.cheby(s, x, s.b, 3, 3)
        e, xe = ref.eigen(s, x, s.b)
        out[k + "eig"] = np.array(e)
        out[k + "eig_x"] = xe
        for t in (0, 1, 2, 3):
            xs, st = ref.pcg(s, t, s.b, rel_tol=1e-8)
            out[k + f"pcg{t}_x"] = xs
            out[k + f"pcg{t}_stats"] = np.array([st["n_iter"], st["init_res"], st["final_res"],
                                                 st["converged"], st["singular"]])
            xs, st = ref.pbicgstab(s, t, s.b, rel_tol=1e-8)
            out[k + f"bicg{t}_x"] = xs
            out[k + f"bicg{t}_stats"] = np.array([st["n_iter"], st["init_res"], st["final_res"],
                                                  st["converged"], st["singular"]])
        w = mg_weights(s)
        levels = ref.hierarchy(s, w, n_coarsest=8)
        out[k + "nlevels"] = np.array(len(levels))
        for li, L in enumerate(levels):
            for key in ("restrict", "face_restrict", "lower_addr", "upper_addr", "diag", "upper",
                        "lower"):
                out[k + f"L{li}_{key}"] = L[key]
        for sm in (1, 2):
            xs, st = ref.mg(s, s.b, w, n_coarsest=8, smoother=sm, rel_tol=1e-8, max_iter=60)
            out[k + f"mg{sm}_x"] = xs
            out[k + f"mg{sm}_stats"] = np.array([st["n_iter"], st["init_res"], st["final_res"],
                                                 st["converged"], st["n_levels"]])
    return out


def main():
    if not ref_available():
        raise SystemExit("build the reference first: make -C oracle ref")
    np.savez_compressed(OUT, **generate(Oracle("ref")))
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
