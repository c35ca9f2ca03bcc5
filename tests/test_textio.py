"""Text dumps in the reference's on-disk formats (host only, no GPU).

Parity is pinned against the reference's own reader and printers
(tools/readData/readFromOpenFOAM/readFromOpenFOAM.cpp,
tools/printData/printUNAP/printUNAP.cpp) built into oracle/_ref: every value
read is bit-identical to the reference reader's, and every file printed is
byte-identical to the reference printer's.  Error returns (where the
reference aborts the process) are checked on our side only.
"""
import ctypes
import os

import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


def _same(a, b):
    return np.array_equal(_bits(a), _bits(b))


def systems():
    return [W.lognormal(7, 6, 5, seed=3, permute=True),
            W.convdiff(6, 5, 4, seed=2, permute=True),
            W.laplace(9, seed=4, permute=False)]


def handle_of(s):
    h = capi.ldumatrixcreat(s)
    return h


def write_ldu_py(path, s, fmt="{:.15e}"):
    """An independent writer of the matrix format (Python's exact decimal
    formatting)."""
    nnz = s.n + s.nf * (1 if s.symm else 2)
    with open(path, "w") as f:
        f.write(f"nCells: {s.n} nnz: {nnz} symm: {1 if s.symm else 0}\n")
        for i in range(s.n):
            f.write(f"{i} {i} {fmt.format(float(s.diag[i]))}\n")
        for k in range(s.nf):
            f.write(f"{s.lower_addr[k]} {s.upper_addr[k]} {fmt.format(float(s.upper[k]))} ")
            if not s.symm:
                f.write(fmt.format(float(s.lower[k])))
            f.write("\n")


class Ref:
    def __init__(self, ref):
        lib = ref.lib
        vp = ctypes.c_void_p
        lib.ref_read_ldu.restype = vp
        lib.ref_read_ldu.argtypes = [ctypes.c_char_p]
        for f in ("ref_ldu_ncells", "ref_ldu_nfaces", "ref_ldu_symm"):
            getattr(lib, f).argtypes = [vp]
        lib.ref_ldu_get.argtypes = [vp] + [vp] * 5
        lib.ref_ldu_destroy.argtypes = [vp]
        lib.ref_print_ldu.argtypes = [vp, ctypes.c_char_p]
        lib.ref_read_vector.argtypes = [ctypes.c_char_p, ctypes.c_int, vp]
        lib.ref_print_vector.argtypes = [ctypes.c_char_p, ctypes.c_int, vp]
        lib.ref_read_interfaces.argtypes = [ctypes.c_char_p, vp, vp, vp, vp, vp, vp,
                                            ctypes.c_char_p]
        self.lib = lib

    def read_ldu(self, path):
        A = self.lib.ref_read_ldu(os.fsencode(path))
        n, nf = self.lib.ref_ldu_ncells(A), self.lib.ref_ldu_nfaces(A)
        out = dict(n=n, nf=nf, symm=bool(self.lib.ref_ldu_symm(A)),
                   lower_addr=np.zeros(nf, np.int32), upper_addr=np.zeros(nf, np.int32),
                   lower=np.zeros(nf), diag=np.zeros(n), upper=np.zeros(nf))
        self.lib.ref_ldu_get(A, out["lower_addr"].ctypes.data, out["upper_addr"].ctypes.data,
                             out["lower"].ctypes.data, out["diag"].ctypes.data,
                             out["upper"].ctypes.data)
        return A, out

    def print_ldu(self, A, name):
        self.lib.ref_print_ldu(A, os.fsencode(name))
        return str(name) + "_0.txt"

    def read_vector(self, path, n):
        v = np.zeros(n)
        self.lib.ref_read_vector(os.fsencode(path), n, v.ctypes.data)
        return v

    def print_vector(self, v, name):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.lib.ref_print_vector(os.fsencode(name), v.shape[0], v.ctypes.data)
        return str(name) + "_0.txt"

    def interfaces(self, path, name=None):
        nn, nf = ctypes.c_int(), ctypes.c_int()
        args = [os.fsencode(path), ctypes.addressof(nn), ctypes.addressof(nf)]
        self.lib.ref_read_interfaces(*args, None, None, None, None, None)
        nb = np.zeros(nn.value, np.int32)
        sz = np.zeros(nn.value, np.int32)
        fc = np.zeros(nf.value, np.int32)
        co = np.zeros(nf.value)
        self.lib.ref_read_interfaces(*args, nb.ctypes.data, sz.ctypes.data, fc.ctypes.data,
                                     co.ctypes.data, None if name is None else os.fsencode(name))
        return dict(neighbour=nb, size=sz, face_cells=fc, coeffs=co)


@pytest.fixture(scope="module")
def R(ref):
    return Ref(ref)


def assert_ldu_equal(m, r):
    assert (m["n"], m["nf"], m["symm"]) == (r["n"], r["nf"], r["symm"])
    for k in ("lower_addr", "upper_addr"):
        assert np.array_equal(m[k], r[k]), k
    for k in ("diag", "upper", "lower"):
        assert _same(m[k], r[k]), k


@pytest.fixture(params=[1, 3, 16])
def io_threads(request, monkeypatch):
    """Splits files into 1, 3 or 16 byte ranges (16 on tiny files puts
    range boundaries inside fields and leaves ranges without a line)."""
    monkeypatch.setenv("UNAP_IO_THREADS", str(request.param))
    return request.param


def test_matrix_read_and_print_match_reference(R, tmp_path, io_threads):
    for s in systems():
        src = tmp_path / f"{s.name}_src.txt"
        write_ldu_py(src, s)
        A, r = R.read_ldu(src)
        h = capi.read_ldu_matrix(src)
        m = capi.handle_ldu(h)
        assert_ldu_equal(m, r)
        # 16 significant digits: half a unit of the 16th plus the read rounding
        assert np.allclose(m["diag"], s.diag, rtol=1e-15, atol=0)
        assert np.allclose(m["upper"], s.upper, rtol=1e-15, atol=0)
        ours = capi.print_ldu_matrix(h, tmp_path / "ours")
        theirs = R.print_ldu(A, tmp_path / "theirs")
        assert open(ours, "rb").read() == open(theirs, "rb").read(), s.name
        # a handle made from arrays prints the same file
        h2 = handle_of(s)
        ours2 = capi.print_ldu_matrix(h2, tmp_path / "ours2")
        assert open(ours2, "rb").read() == open(theirs, "rb").read(), s.name
        capi.sw_matrix_destroy(h)
        capi.sw_matrix_destroy(h2)
        R.lib.ref_ldu_destroy(A)


def awkward_values():
    """Values whose "%.15e" forms need care: exact ties (half-even), signed
    zeros, subnormals, the extremes, infinities and NaNs, and random bit
    patterns over the whole exponent range."""
    rng = np.random.default_rng(17)
    ties = [1234567890123456.5, 0.5, 2.5, 1.0000000000000002, 9.999999999999999e22,
            1e23, 5e-324, 2.2250738585072014e-308, 2.225073858507201e-308,
            1.7976931348623157e308, -0.0, 0.0, 1.0, -1.0, 0.1, 1 / 3,
            np.inf, -np.inf, np.nan, -np.nan]
    bits = rng.integers(0, 2 ** 63 - 1, 3000, dtype=np.int64)
    rnd = bits.view(np.float64)
    rnd = rnd[np.isfinite(rnd)]
    sgn = np.where(rng.random(rnd.shape[0]) < 0.5, -1.0, 1.0)
    return np.concatenate([np.array(ties), rnd * sgn, rng.standard_normal(1000)])


def test_vector_print_and_read_match_reference(R, tmp_path, io_threads):
    v = awkward_values()
    ours = capi.print_vector(v, tmp_path / "v_ours")
    theirs = R.print_vector(v, tmp_path / "v_theirs")
    assert open(ours, "rb").read() == open(theirs, "rb").read()
    back = capi.read_vector(ours, v.shape[0])
    assert _same(back, R.read_vector(ours, v.shape[0]))
    # "%.15e" keeps 16 significant digits: finite values round trip within
    # half a unit in the 16th digit (plus the read rounding), inf and NaN exactly
    # (DBL_MAX prints as 1.797693134862316e+308, which atof reads as inf)
    fin = np.isfinite(v) & (np.abs(v) < 1.797693134862315e308)
    assert np.allclose(back[fin], v[fin], rtol=1e-15, atol=0)
    assert np.isinf(back[np.abs(v) == 1.7976931348623157e308]).all()
    assert np.array_equal(np.isnan(back), np.isnan(v))
    assert np.array_equal(back[np.isinf(v)], v[np.isinf(v)])


def test_awkward_fields_read_like_atof_atoi(R, tmp_path, io_threads):
    """Fields the reference reader accepts through atof/atoi: signs, hex
    floats, overflow and underflow, trailing junk, tabs, CR-LF line ends,
    extra fields, no final newline."""
    reals = ["+1.5", "0x1p3", "1e400", "-1e400", "1e-400", "4.9e-324", "2.4703282292062328e-324",
             "1.5abc", "-0", ".5", "5.", "1e", "1e+", "inf", "-Infinity", "nan", "-nan",
             "abc", "0.1000000000000000055511151231257827", "9007199254740993",
             "1.00000000000000011102230246251565404236316680908203125", "-2.5E-3",
             "123456789012345678901234567890", "1e22", "8.98846567431158e307"]
    n = len(reals)
    lines = ["nCells:\t%d   nnz: %d symm: 0 trailing words" % (n, n + 2 * (n - 1))]
    for i, r in enumerate(reals):
        lines.append(f"{i}\t{i} {r} extra fields here")
    for k in range(n - 1):
        lines.append(f"+{k} {k + 1}junk {reals[k]} {reals[n - 1 - k]}\r")
    path = tmp_path / "awkward.txt"
    path.write_bytes(("\n".join(lines)).encode())  # no final newline
    A, r = R.read_ldu(path)
    h = capi.read_ldu_matrix(path)
    assert_ldu_equal(capi.handle_ldu(h), r)
    # and the printers agree on what was read
    ours = capi.print_ldu_matrix(h, tmp_path / "aw_ours")
    theirs = R.print_ldu(A, tmp_path / "aw_theirs")
    assert open(ours, "rb").read() == open(theirs, "rb").read()
    capi.sw_matrix_destroy(h)
    R.lib.ref_ldu_destroy(A)
    # vectors: first field only, the rest ignored
    vpath = tmp_path / "awkward_v.txt"
    vpath.write_bytes(("nCells: %d\n" % n + "\n".join(f"  {x}\t7 8" for x in reals)
                       + "\n").encode())
    assert _same(capi.read_vector(vpath, n), R.read_vector(vpath, n))


def test_symmetric_file_gives_symmetric_matrix(R, tmp_path):
    s = W.laplace(6, seed=1, permute=True)
    p = tmp_path / "s.txt"
    write_ldu_py(p, s)
    h = capi.read_ldu_matrix(p)
    m = capi.handle_ldu(h)
    assert m["symm"] and _same(m["lower"], m["upper"])
    ours = capi.print_ldu_matrix(h, tmp_path / "o")
    head = open(ours).readline().split()
    assert head == ["nCells:", str(s.n), "nnz:", str(s.n + s.nf), "symm:", "1"]
    # symmetric face lines end in "upper " (one trailing blank), as printed
    # by the reference
    assert open(ours).read().splitlines()[s.n + 1].endswith(" ")
    capi.sw_matrix_destroy(h)


def write_interfaces_py(path, neighbour, size, face_cells, coeffs):
    with open(path, "w") as f:
        f.write(f"neighbor processors: {len(neighbour)} faces: total {int(sum(size))}\n")
        k = 0
        for nb, sz in zip(neighbour, size):
            f.write(f"processor: {nb} size: {sz}\n")
            for _ in range(sz):
                f.write(f"{face_cells[k]} {float(coeffs[k])!r}\n")
                k += 1


def test_interfaces_read_and_print_match_reference(R, tmp_path):
    rng = np.random.default_rng(3)
    neighbour, size = [3, 1, 7], [4, 0, 6]
    fc = rng.integers(0, 50, sum(size)).astype(np.int32)
    co = rng.standard_normal(sum(size))
    p = tmp_path / "interfaces.txt"
    write_interfaces_py(p, neighbour, size, fc, co)
    ours = capi.read_interfaces(p)
    theirs = R.interfaces(p, tmp_path / "if_theirs")
    for k in ("neighbour", "size", "face_cells"):
        assert np.array_equal(ours[k], theirs[k]), k
    assert _same(ours["coeffs"], theirs["coeffs"])
    assert _same(ours["coeffs"], -co)  # stored negated, like the reference's patches
    out = capi.print_interfaces(tmp_path / "if_ours", ours["neighbour"], ours["size"],
                                ours["face_cells"], ours["coeffs"])
    assert open(out, "rb").read() == open(tmp_path / "if_theirs_0.txt", "rb").read()


def test_large_file_same_values_for_any_thread_count(tmp_path, monkeypatch):
    s = W.convdiff(30, 25, 20, seed=9, permute=True)
    p = tmp_path / "big.txt"
    write_ldu_py(p, s)
    got, text = [], []
    for t in ("1", "5", "32"):
        monkeypatch.setenv("UNAP_IO_THREADS", t)
        h = capi.read_ldu_matrix(p)
        got.append(capi.handle_ldu(h))
        out = capi.print_ldu_matrix(h, tmp_path / f"big_{t}")
        capi.sw_matrix_destroy(h)
        text.append(open(out, "rb").read())
    for m, t in zip(got[1:], text[1:]):
        assert_ldu_equal(m, got[0])
        assert t == text[0]
    assert np.array_equal(got[0]["upper_addr"], s.upper_addr)
    assert np.allclose(got[0]["lower"], s.lower, rtol=1e-15, atol=0)


@pytest.mark.parametrize("text,match", [
    ("nCells: 2 nnz: 4 symm: 1\n0 0 1.0\n1 1 2.0\n", "reading 2 lines, while nCells = 2, nFaces = 2"),
    ("nCells: 2 nnz: 3 symm: 1\n0 0 1.0\n1 1\n0 1 0.5\n", "line 3 has fewer than 3 fields"),
    ("nCells: 2 nnz: 4 symm: 0\n0 0 1.0\n1 1 2.0\n0 1 0.5\n", "line 4 has fewer than 4 fields"),
    ("nCells:\n", "reading 0 lines, while nCells = -1"),
    ("", "is empty"),
])
def test_malformed_matrix_files_are_errors(tmp_path, text, match):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(capi.UnapCudaError, match=match):
        capi.read_ldu_matrix(p)


def test_vector_errors(tmp_path):
    p = tmp_path / "v.txt"
    p.write_text("nCells: 3\n1\n2\n3\n")
    with pytest.raises(capi.UnapCudaError, match="fill size = 3, while allocated size = 4"):
        capi.read_vector(p, 4)
    p.write_text("nCells: 3\n1\n2\n")
    with pytest.raises(capi.UnapCudaError, match="reading 2 lines, while nCells = 3"):
        capi.read_vector(p, 3)
    with pytest.raises(capi.UnapCudaError, match="cannot open"):
        capi.read_vector(tmp_path / "missing.txt", 3)
    with pytest.raises(capi.UnapCudaError, match="cannot create"):
        capi.print_vector(np.zeros(2), tmp_path / "no_such_dir" / "v")


@pytest.mark.gpu
def test_text_dump_to_device_solve(cuda, orc, tmp_path):
    """A matrix and right-hand side read from the reference's text dumps
    solve on the device like the same system given as arrays."""
    torch = cuda
    s = W.lognormal(14, 12, 10, seed=31, permute=True)
    write_ldu_py(tmp_path / "A.txt", s, fmt="{!r}")
    with open(tmp_path / "b.txt", "w") as f:
        f.write(f"nCells: {s.n}\n" + "".join(f"{float(v)!r}\n" for v in s.b))
    h = capi.read_ldu_matrix(tmp_path / "A.txt")
    b = capi.read_vector(tmp_path / "b.txt", s.n)
    m = capi.handle_ldu(h)
    # Python's repr round-trips exactly, so the arrays are the system's own
    assert _same(m["upper"], s.upper) and _same(m["diag"], s.diag) and _same(b, s.b)
    # pcgsolversolve_ deletes the handle, like the reference's
    x, n_iter, _ = capi.pcgsolversolve(np.zeros(s.n), h, b, 2, rel_tol=1e-9)
    x_ref, st_ref = orc.pcg(s, 2, s.b, rel_tol=1e-9)
    assert abs(n_iter - st_ref["n_iter"]) <= 1
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "textio")


def test_golden_fixtures_from_the_reference_printer(tmp_path):
    """The reference's printer output committed under tests/golden/textio
    (make_textio_golden.py): reading the same inputs and printing them
    gives those files byte for byte, with no reference build needed."""
    h = capi.read_ldu_matrix(os.path.join(GOLDEN, "A_in.txt"))
    out = capi.print_ldu_matrix(h, tmp_path / "A")
    capi.sw_matrix_destroy(h)
    assert open(out, "rb").read() == open(os.path.join(GOLDEN, "A_0.txt"), "rb").read()
    n = int(open(os.path.join(GOLDEN, "v_in.txt")).readline().split()[1])
    v = capi.read_vector(os.path.join(GOLDEN, "v_in.txt"), n)
    out = capi.print_vector(v, tmp_path / "v")
    assert open(out, "rb").read() == open(os.path.join(GOLDEN, "v_0.txt"), "rb").read()
    i = capi.read_interfaces(os.path.join(GOLDEN, "interfaces_in.txt"))
    out = capi.print_interfaces(tmp_path / "interfaces", i["neighbour"], i["size"],
                                i["face_cells"], i["coeffs"])
    assert open(out, "rb").read() == open(os.path.join(GOLDEN, "interfaces_0.txt"), "rb").read()
    # and the printed matrix reads back to the values printed
    h2 = capi.read_ldu_matrix(os.path.join(GOLDEN, "A_0.txt"))
    m = capi.handle_ldu(h2)
    capi.sw_matrix_destroy(h2)
    assert m["n"] == 36 and not m["symm"]


def test_random_numeric_fields_read_like_the_reference(R, tmp_path):
    """Thousands of numeric fields in random spellings (fixed, scientific
    and shortest forms, signs, leading zeros, upper-case exponents, many or
    few digits, subnormal and huge magnitudes) read bit for bit like the
    reference reader."""
    rng = np.random.default_rng(99)
    out = []
    for _ in range(4000):
        m = rng.standard_normal() * 10.0 ** rng.integers(-320, 309)
        kind = rng.integers(0, 7)
        if kind == 0:
            t = repr(float(m))
        elif kind == 1:
            t = f"{m:.{rng.integers(0, 25)}e}"
        elif kind == 2:
            t = f"{m:.{rng.integers(1, 20)}g}"
        elif kind == 3:
            t = f"{m:.{rng.integers(0, 12)}E}"
        elif kind == 4:
            t = f"{rng.integers(-10**12, 10**12)}"
        elif kind == 5:
            t = "+" + f"{abs(m):.17e}"
        else:
            digits = "".join(str(d) for d in rng.integers(0, 10, rng.integers(1, 40)))
            t = f"{'-' if rng.random() < 0.5 else ''}00{digits[:5]}.{digits[5:]}e{rng.integers(-330, 330)}"
        out.append(t)
    p = tmp_path / "fuzz.txt"
    p.write_text(f"nCells: {len(out)}\n" + "\n".join(out) + "\n")
    assert _same(capi.read_vector(p, len(out)), R.read_vector(p, len(out)))
