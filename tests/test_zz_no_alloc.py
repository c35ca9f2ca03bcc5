"""unap_cuda_spmv_noalloc: the SpMV entry point that allocates nothing.

It serves callers that cannot allocate device memory at call time (a code
that reserved its whole device-memory budget before its time loop, or a host
thread that must not take the CUDA allocator's locks).  Its scratch is a
fixed 2 x 1,048,576-double array inside the library, shared by every call.
The tests call it through the C ABI and compare it with unap_cuda_spmv
(the same kernels in the same order, so the results must be bit-identical)
on two calls in a row and on a second matrix after the first; made first on
a fresh matrix, it leaves the free device memory unchanged and equals the
oracle's SpMV; a matrix above the limit is rejected with a message.

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


def test_spmv_noalloc_first_on_fresh_handle_allocates_nothing(cuda, orc):
    """The no-alloc call made first on a freshly built matrix (no call has
    allocated the handle's scratch yet): the free device memory is the same
    before and after a warm second call, the result equals the oracle's SpMV
    bit for bit, and only then does unap_cuda_spmv (which allocates) give
    the same bits."""
    torch = cuda
    lib = capi.load()
    s = W.lognormal(18, 16, 14, seed=7, permute=True)
    A = capi.DeviceMatrix(s)
    rng = np.random.default_rng(8)
    xs = [rng.standard_normal(s.n) for _ in range(2)]
    xd = [torch.tensor(v, device="cuda") for v in xs]
    ys = [torch.full_like(xd[0], np.nan) for _ in range(2)]
    torch.cuda.synchronize()

    def call(x, y):
        capi.check(lib.unap_cuda_spmv_noalloc(A.handle, ctypes.c_void_p(x.data_ptr()),
                                              ctypes.c_void_p(y.data_ptr())))

    call(xd[0], ys[0])  # first call: looks up the scratch array's address
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    call(xd[1], ys[1])
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    for x, y in zip(xs, ys):
        assert np.array_equal(y.cpu().numpy(), orc.spmv(s, x))
    y_ref = torch.zeros_like(xd[1])
    A.spmv(xd[1], y_ref)
    assert np.array_equal(ys[1].cpu().numpy(), y_ref.cpu().numpy())
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
