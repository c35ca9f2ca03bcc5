"""Compiling C++ programs against the UNAP C++ API (include/unap/) and
libunap_cuda.so, for the C++ API tests."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include", "unap")
CXX_DIR = os.path.join(ROOT, "tests", "cxx")


def compiler():
    return shutil.which("g++") or shutil.which("c++")


def lib_dir():
    from unap_gb300 import capi
    capi.load()
    return os.path.dirname(capi.lib_path())


def compile_program(src, out, extra=()):
    """g++ -std=c++11 with warnings as errors for our own programs; returns
    (returncode, stderr)."""
    ld = lib_dir()
    cmd = [compiler(), "-std=c++11", "-O1", "-I", INCLUDE, *extra, src, "-o", out,
           "-L", ld, "-lunap_cuda", f"-Wl,-rpath,{ld}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, r.stderr


def reference_tree():
    """The reference source tree recorded by the oracle's reference build,
    or the UNAP_REFERENCE_ROOT environment variable; None when absent."""
    cands = [os.environ.get("UNAP_REFERENCE_ROOT")]
    rec = os.path.join(ROOT, "oracle", "_ref", "reference_root.txt")
    if os.path.exists(rec):
        with open(rec) as f:
            cands.append(f.read().strip())
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "test")):
            return c
    return None
