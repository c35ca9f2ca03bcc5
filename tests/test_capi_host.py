"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every symbol include/*.h declares, ingests COO/CSR like the reference, and
reports bad handles as errors instead of crashing."""
import ctypes
import os
import re

import numpy as np
import pytest

from unap_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(",
                             text, flags=re.M):
            if m.group(1) not in ("if", "while", "for", "return", "sizeof"):
                names.append(m.group(1))
    return sorted(set(names))


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    lib = capi.load()
    assert b"sm_103a" in lib.unap_cuda_version()


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(build.build())
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and every declared symbol has a ctypes signature in the Python mirror
    assert not [n for n in names if n not in capi.SIGNATURES]


def test_coo2ldu_known_answer_ex8():
    # test/ex8.cpp: 5x5 unsymmetric COO (0-based there; the C ABI takes
    # 1-based indices, fortranInterface.cpp:90-95)
    row = np.array([0, 0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 4, 4, 4, 4])
    col = np.array([0, 1, 3, 4, 0, 1, 2, 1, 2, 4, 0, 3, 4, 0, 2, 3, 4])
    data = np.array([1.1, 1.2, 1.4, 1.5, 2.1, 2.2, 2.3, 3.2, 3.3, 3.5, 4.1, 4.4, 4.5, 5.1, 5.3,
                     5.4, 5.5])
    # shuffle columns inside each row: reorderCOO must restore column order
    perm = np.array([0, 3, 2, 1, 6, 5, 4, 9, 8, 7, 12, 11, 10, 16, 15, 14, 13])
    h = capi.coo2ldumatrixcreat(data[perm], row[perm] + 1, col[perm] + 1, 5, symm=False)
    m = capi.handle_ldu(h)
    capi.sw_matrix_destroy(h)
    assert list(m["upper_addr"]) == [1, 3, 4, 2, 4, 4]
    assert list(m["lower_addr"]) == [0, 0, 0, 1, 2, 3]
    assert np.array_equal(m["diag"], [1.1, 2.2, 3.3, 4.4, 5.5])
    assert np.array_equal(m["upper"], [1.2, 1.4, 1.5, 2.3, 3.5, 4.5])
    assert np.array_equal(m["lower"], [2.1, 4.1, 5.1, 3.2, 5.3, 5.4])
    assert not m["symm"]


def test_coo2ldu_against_reference(ref):
    # random structurally symmetric COO, row-sorted, columns shuffled per row
    rng = np.random.default_rng(5)
    from unap_gb300 import workloads as W
    s = W.convdiff(4, 3, 3, seed=2, permute=True)
    a = s.dense()
    r, c = np.nonzero(a)
    v = a[r, c]
    h = capi.coo2ldumatrixcreat(v, r + 1, c + 1, s.n, symm=False)
    m = capi.handle_ldu(h)
    capi.sw_matrix_destroy(h)
    vp = ctypes.c_void_p
    r32 = r.astype(np.int32)
    c32 = c.astype(np.int32)
    Aref = ref.lib.ref_coo2ldu(vp(v.ctypes.data), vp(r32.ctypes.data), vp(c32.ctypes.data),
                               s.n, len(v), 0)
    nf = ref.lib.ref_ldu_nfaces(ctypes.c_void_p(Aref))
    l = np.zeros(nf, np.int32)
    u = np.zeros(nf, np.int32)
    lo = np.zeros(nf)
    d = np.zeros(s.n)
    up = np.zeros(nf)
    ref.lib.ref_ldu_get(vp(Aref), vp(l.ctypes.data), vp(u.ctypes.data), vp(lo.ctypes.data),
                        vp(d.ctypes.data), vp(up.ctypes.data))
    ref.lib.ref_ldu_destroy(ctypes.c_void_p(Aref))
    for k, v2 in (("lower_addr", l), ("upper_addr", u), ("lower", lo), ("diag", d),
                  ("upper", up)):
        assert np.array_equal(m[k], v2), k
    del rng


def test_bad_handle_is_an_error_not_a_crash():
    lib = capi.load()
    bogus = np.zeros(8, np.int64)  # valid memory without the handle magic
    rc = lib.unap_cuda_matrix_destroy(bogus.ctypes.data)
    assert rc == -1
    assert b"invalid matrix handle" in lib.unap_cuda_last_error()
    with pytest.raises(capi.UnapCudaError):
        capi.handle_ldu(bogus.ctypes.data)


def test_coo_ingest_rejects_what_the_reference_leaves_undefined():
    """Host form (small matrices stay on the host): rows out of order, a
    repeated entry and a column whose lower entries do not match the row's
    upper ones are errors; the row-sorted input with shuffled columns is
    the system itself."""
    from unap_gb300 import workloads as W
    rng = np.random.default_rng(5)
    s = W.convdiff(6, 5, 4, seed=2, permute=True)
    rows = np.concatenate([np.arange(s.n), s.lower_addr, s.upper_addr])
    cols = np.concatenate([np.arange(s.n), s.upper_addr, s.lower_addr])
    vals = np.concatenate([s.diag, s.upper, s.lower])
    o = np.lexsort((rng.random(rows.shape[0]), rows))
    v, r, c = vals[o], rows[o].astype(np.int32), cols[o].astype(np.int32)
    h = capi.coo2ldumatrixcreat(v, r + 1, c + 1, s.n, symm=False)
    m = capi.handle_ldu(h)
    capi.sw_matrix_destroy(h)
    assert np.array_equal(m["upper_addr"], s.upper_addr) and np.array_equal(m["lower"], s.lower)
    lower = np.nonzero(c < r)[0]
    upper = np.nonzero(c > r)[0]
    k = lower[len(lower) // 2]
    taken = set(c[r == r[k]].tolist())
    c_bad = c.copy()
    c_bad[k] = next(x for x in range(int(r[k])) if x not in taken)
    r_bad = r.copy()
    r_bad[[upper[3], upper[-3]]] = r_bad[[upper[-3], upper[3]]]
    c_dup = c.copy()
    row = np.nonzero(r == r[upper[5]])[0]
    c_dup[row[0]] = c_dup[row[1]]
    for cc, rr, msg in ((c_bad, r, "structurally symmetric"), (c, r_bad, "ascending row order"),
                        (c_dup, r, "repeats an entry")):
        with pytest.raises(capi.UnapCudaError, match=msg):
            capi.coo2ldumatrixcreat(v, rr + 1, cc + 1, s.n, symm=False)


def test_header_is_plain_c_and_links(tmp_path):
    """include/unap_cuda.h compiles as C99 with warnings as errors, and a C
    program calling entry points from both parts links against the library
    (what a Fortran/C caller of the reference relinks to)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lib = build.build()
    src = tmp_path / "caller.c"
    src.write_text(r'''
#include "unap_cuda.h"
#include <stdio.h>
int main(void)
{
    long int A = 0;
    int n = 2, nf = 1, l = 0, u = 1;
    double diag[2] = {2.0, 2.0}, upper = -1.0;
    /* lower == upper: symmetric, the reference's convention */
    ldumatrixcreat_(&A, &n, &nf, &l, &u, &upper, diag, &upper);
    int cells = 0, faces = 0, symm = 0;
    if (unap_cuda_matrix_size(A, &cells, &faces, &symm) != 0) return 1;
    sw_matrix_destroy__(&A);
    printf("%s %d %d %d\n", unap_cuda_version(), cells, faces, symm);
    return cells == 2 && faces == 1 && symm == 1 ? 0 : 2;
}
''')
    exe = tmp_path / "caller"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", os.path.join(ROOT, "include"), str(src), lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # host-only calls: no GPU needed to run it
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, (run.stdout, run.stderr)
    assert "sm_103a" in run.stdout


def _coo_case(rng, n, density):
    """A structurally symmetric COO pattern, grouped by row, each row's
    entries in random column order (the reordering's input)."""
    rows, cols = [], []
    for r in range(n):
        cs = [c for c in range(n) if c == r or rng.random() < density]
        rng.shuffle(cs)
        rows += [r] * len(cs)
        cols += cs
    return (np.array(rows, np.int32), np.array(cols, np.int32),
            rng.standard_normal(len(rows)))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def test_reorder_entry_points_against_reference():
    """reordercoo_/reorderuface__/reorderlface__/reordervalue__ and their
    0-based forms give the reference's matrixConversion results bit for bit
    (where the reference build exists), and a sorted-order check everywhere."""
    from oracle_lib import Oracle, ref_available
    lib = capi.load()
    ref = Oracle("ref").lib if ref_available() else None
    rng = np.random.default_rng(4)
    for n, dens in ((1, 0.0), (7, 0.3), (40, 0.1), (200, 0.02)):
        r0, c0, v0 = _coo_case(rng, n, dens)
        size = len(r0)
        # reordercoo_ (1-based in)
        r, c, v = (r0 + 1).copy(), (c0 + 1).copy(), v0.copy()
        lib.reordercoo_(_dp(v), _ip(r), _ip(c),
                        ctypes.byref(ctypes.c_int(n)), ctypes.byref(ctypes.c_int(size)))
        key = r.astype(np.int64) * n + c
        assert np.all(np.diff(key) > 0)
        order = np.lexsort((c0, r0))
        assert np.array_equal(v, v0[order]) and np.array_equal(r, r0[order])
        if ref is not None:
            rr, cr, vr = r0.copy(), c0.copy(), v0.copy()
            ref.ref_reorder_coo(vr.ctypes.data, rr.ctypes.data, cr.ctypes.data, n, size)
            assert np.array_equal(rr, r) and np.array_equal(cr, c) and np.array_equal(vr, v)
        for by_col, fn in ((0, lib.reorderuface__), (1, lib.reorderlface__)):
            r, c, o = (r0 + 1).copy(), (c0 + 1).copy(), np.zeros(size, np.int32)
            fn(_ip(r), _ip(c), ctypes.byref(ctypes.c_int(n)), ctypes.byref(ctypes.c_int(size)),
               _ip(o))
            assert np.array_equal(np.sort(o), np.arange(size))
            if ref is not None:
                rr, cr, orr = r0.copy(), c0.copy(), np.zeros(size, np.int32)
                ref.ref_reorder_faces(by_col, rr.ctypes.data, cr.ctypes.data, n, size,
                                      orr.ctypes.data)
                assert np.array_equal(rr, r) and np.array_equal(cr, c) and np.array_equal(orr, o)
            vals = v0.copy()
            lib.reordervalue__(_dp(vals), _ip(o), ctypes.byref(ctypes.c_int(size)))
            assert np.array_equal(vals[o], v0)
            if ref is not None:
                vr = v0.copy()
                ref.ref_reorder_value(vr.ctypes.data, o.ctypes.data, size)
                assert np.array_equal(vr, vals)


def test_reorder_rejects_undefined_input():
    """A repeated (row, column) pair or an index out of range: the arrays
    stay as they were and the 0-based call returns UNAP_CUDA_EINVAL."""
    lib = capi.load()
    r = np.array([0, 0, 1], np.int32)
    c = np.array([1, 1, 0], np.int32)
    v = np.array([1.0, 2.0, 3.0])
    before = (r.copy(), c.copy(), v.copy())
    assert lib.unap_cuda_reorder_coo(v.ctypes.data, r.ctypes.data, c.ctypes.data, 2, 3) == -1
    assert all(np.array_equal(a, b) for a, b in zip((r, c, v), before))
    c2 = np.array([1, 5, 0], np.int32)
    o = np.zeros(3, np.int32)
    assert lib.unap_cuda_reorder_lface(r.ctypes.data, c2.ctypes.data, 2, 3, o.ctypes.data) == -1
    assert lib.unap_cuda_reorder_value(v.ctypes.data, np.array([0, 0, 1], np.int32).ctypes.data,
                                       3) == -1
