"""Generate the text-dump fixtures under tests/golden/textio/ from the
reference build.

The reference's own reader and printers (readFromOpenFOAM.cpp,
printUNAP.cpp, compiled in place into oracle/_ref/libunap_ref.so by
``make -C oracle ref``) read a small matrix, a vector with awkward values
and an interfaces file written here in their input format, and print them
back; the printed files are committed, so the library's reader and printers
can be pinned against them on hosts where the reference tree is absent.
Re-run with ``python tests/golden/make_textio_golden.py``.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "textio")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle_lib import Oracle, ref_available  # noqa: E402
from unap_gb300 import workloads as W  # noqa: E402


def system():
    return W.convdiff(4, 3, 3, seed=21, permute=True, pe=5.0)


def vector():
    rng = np.random.default_rng(22)
    special = [1234567890123456.5, 0.5, 2.5, -0.0, 5e-324, 2.2250738585072014e-308,
               1.7976931348623157e308, 1 / 3, -1e-300, 1e23]
    return np.concatenate([np.array(special), rng.standard_normal(20) * 10.0 ** rng.integers(
        -30, 30, 20)])


def write_inputs(d):
    s = system()
    with open(os.path.join(d, "A_in.txt"), "w") as f:
        f.write(f"nCells: {s.n} nnz: {s.n + 2 * s.nf} symm: 0\n")
        for i in range(s.n):
            f.write(f"{i} {i} {float(s.diag[i])!r}\n")
        for k in range(s.nf):
            f.write(f"{s.lower_addr[k]} {s.upper_addr[k]} {float(s.upper[k])!r} "
                    f"{float(s.lower[k])!r}\n")
    v = vector()
    with open(os.path.join(d, "v_in.txt"), "w") as f:
        f.write(f"nCells: {v.shape[0]}\n" + "".join(f"{float(x)!r}\n" for x in v))
    with open(os.path.join(d, "interfaces_in.txt"), "w") as f:
        f.write("neighbor processors: 2 faces: total 5\n")
        f.write("processor: 3 size: 2\n0 0.25\n7 -1.5e-3\n")
        f.write("processor: 1 size: 3\n4 2.0\n5 3.141592653589793\n9 -7.0e+12\n")


def main():
    if not ref_available():
        raise SystemExit("build the reference first: make -C oracle ref")
    os.makedirs(OUT, exist_ok=True)
    write_inputs(OUT)
    lib = Oracle("ref").lib
    vp = ctypes.c_void_p
    lib.ref_read_ldu.restype = vp
    lib.ref_read_ldu.argtypes = [ctypes.c_char_p]
    lib.ref_print_ldu.argtypes = [vp, ctypes.c_char_p]
    lib.ref_ldu_destroy.argtypes = [vp]
    lib.ref_read_vector.argtypes = [ctypes.c_char_p, ctypes.c_int, vp]
    lib.ref_print_vector.argtypes = [ctypes.c_char_p, ctypes.c_int, vp]
    lib.ref_read_interfaces.argtypes = [ctypes.c_char_p, vp, vp, vp, vp, vp, vp,
                                        ctypes.c_char_p]
    A = lib.ref_read_ldu(os.path.join(OUT, "A_in.txt").encode())
    lib.ref_print_ldu(A, os.path.join(OUT, "A").encode())
    lib.ref_ldu_destroy(A)
    n = vector().shape[0]
    v = np.zeros(n)
    lib.ref_read_vector(os.path.join(OUT, "v_in.txt").encode(), n, v.ctypes.data)
    lib.ref_print_vector(os.path.join(OUT, "v").encode(), n, v.ctypes.data)
    nn, nf = ctypes.c_int(), ctypes.c_int()
    lib.ref_read_interfaces(os.path.join(OUT, "interfaces_in.txt").encode(),
                            ctypes.addressof(nn), ctypes.addressof(nf), None, None, None, None,
                            os.path.join(OUT, "interfaces").encode())
    print("wrote", sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
