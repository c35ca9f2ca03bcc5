"""The reference's C++ class API (include/unap/): programs written against
UNAP compile and link against the headers and libunap_cuda.so.

* The reference's own example programs that use only the solve path
  (test/ex1-ex5, ex8: lduMatrix, PCG, PBiCGStab, the LDU preconditioners,
  the smoothers, lduAgglomeration, MGSolver, coo2ldu) compile UNCHANGED, with
  no warning under -Wall -Wextra, where the reference tree is present.
* This repository's C++ test programs (tests/cxx/) compile warning-free.
Running them needs the GPU (tests/test_gpu_cxx_api.py); these checks do not.
"""
import os

import pytest

from cxx_util import CXX_DIR, compile_program, compiler, reference_tree

pytestmark = pytest.mark.skipif(compiler() is None, reason="no C++ compiler")

REFERENCE_EXAMPLES = ["ex1", "ex2", "ex3", "ex4", "ex5", "ex8"]


@pytest.mark.parametrize("name", REFERENCE_EXAMPLES)
def test_reference_example_compiles_unchanged(name, tmp_path):
    tree = reference_tree()
    if tree is None:
        pytest.skip("reference tree not present on this host")
    src = os.path.join(tree, "test", f"{name}.cpp")
    rc, err = compile_program(src, str(tmp_path / name), extra=["-Wall", "-Wextra"])
    assert rc == 0, err[-3000:]
    # the reference's own sources trip no warning of the API headers
    assert "include/unap" not in err, err[-3000:]


@pytest.mark.parametrize("name", ["known_answers", "api_driver"])
def test_own_programs_compile(name, tmp_path):
    rc, err = compile_program(os.path.join(CXX_DIR, f"{name}.cpp"), str(tmp_path / name),
                              extra=["-Wall", "-Wextra", "-Werror"])
    assert rc == 0, err[-3000:]


def test_label_int64_build(tmp_path):
    """With 64-bit labels (-DLABEL_INT64, the reference's SConstruct setting)
    the API still compiles: labels are converted at the C ABI."""
    rc, err = compile_program(os.path.join(CXX_DIR, "api_driver.cpp"), str(tmp_path / "drv64"),
                              extra=["-DLABEL_INT64", "-Wall"])
    assert rc == 0, err[-3000:]
