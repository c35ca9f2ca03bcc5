"""Loader for tests/golden/reference_small.npz (outputs of the reference
library on small seeded systems, see tests/golden/make_golden.py)."""
from __future__ import annotations

import os

import numpy as np

from unap_gb300.workloads import LduSystem

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_small.npz")


def load():
    z = np.load(PATH)
    n_cases = len({k.split("/")[0] for k in z.files})
    out = []
    for ci in range(n_cases):
        k = f"c{ci}/"
        symm = bool(z[k + "symm"])
        s = LduSystem(int(z[k + "n"]), z[k + "lower_addr"], z[k + "upper_addr"],
                      None if symm else z[k + "lower"], z[k + "diag"], z[k + "upper"],
                      z[k + "b"], name=f"golden{ci}")
        res = {key[len(k):]: z[key] for key in z.files if key.startswith(k)}
        out.append((s, res))
    return out
