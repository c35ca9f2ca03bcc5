"""unap_cuda_spmv_noalloc: the SpMV entry point that allocates nothing.

It serves callers that cannot allocate device memory at call time (a code
that reserved its whole device-memory budget before its time loop, or a host
thread that must not take the CUDA allocator's locks).  Its scratch is a
fixed 2 x 1,048,576-double array inside the library, shared by every call.
The tests call it through the C ABI and compare it with unap_cuda_spmv
(the same kernels in the same order, so the results must be bit-identical)
on two calls in a row, on a second matrix after the first, and check that a
matrix above the limit is rejected with a message.

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from unap_gb300 import capi
from unap_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _spmv_both(torch, A, x):
    lib = capi.load()
    y_ref = torch.zeros_like(x)
    y = torch.full_like(x, np.nan)
    A.spmv(x, y_ref)
    capi.check(lib.unap_cuda_spmv_noalloc(A.handle, ctypes.c_void_p(x.data_ptr()),
                                          ctypes.c_void_p(y.data_ptr())))
    torch.cuda.synchronize()
    return y.cpu().numpy(), y_ref.cpu().numpy()


def test_spmv_noalloc_matches_spmv_twice(cuda):
    torch = cuda
    s = W.lognormal(20, 18, 16, seed=3, permute=True)
    A = capi.DeviceMatrix(s)
    rng = np.random.default_rng(5)
    for _ in range(2):  # the scratch keeps the previous call's contents
        x = torch.tensor(rng.standard_normal(s.n), device="cuda")
        y, y_ref = _spmv_both(torch, A, x)
        assert np.array_equal(y, y_ref)
    A.close()


def test_spmv_noalloc_second_matrix_after_first(cuda):
    torch = cuda
    rng = np.random.default_rng(6)
    for s in (W.laplace(30, 28, 26, seed=1, permute=True), W.convdiff(9, seed=2, permute=True)):
        A = capi.DeviceMatrix(s)
        x = torch.tensor(rng.standard_normal(s.n), device="cuda")
        y, y_ref = _spmv_both(torch, A, x)
        assert np.array_equal(y, y_ref), s.name
        A.close()


def test_spmv_noalloc_rejects_too_large(cuda):
    torch = cuda
    s = W.laplace(104, 104, 100, seed=4, permute=False)  # 1,081,600 cells > 1,048,576
    A = capi.DeviceMatrix(s)
    x = torch.ones(s.n, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    lib = capi.load()
    rc = lib.unap_cuda_spmv_noalloc(A.handle, ctypes.c_void_p(x.data_ptr()),
                                    ctypes.c_void_p(y.data_ptr()))
    assert rc == -1
    assert "static scratch limit" in lib.unap_cuda_last_error().decode()
    A.close()
