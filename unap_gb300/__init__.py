"""unap_gb300 -- GB300-native (sm_103a) implementation of UNAP's solve path.

The product is the shared library ``libunap_cuda.so`` (C ABI in
``include/unap_cuda.h``, CUDA kernels and C++ host code in ``csrc/``).  This
package holds the build recipe (``build``), the ctypes mirror of the C ABI
(``capi``) and the seeded synthetic workloads (``workloads``).
"""
from . import build  # noqa: F401

__all__ = ["build", "capi", "workloads"]


def __getattr__(name):
    if name in ("capi", "workloads"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
