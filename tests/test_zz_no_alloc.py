"""The allocation-free test-RMSE entry point (cdmf_cuda_rmse_coo_noalloc).

It serves callers that cannot let the library call cudaMalloc, such as a
process that hands out all of its device memory from its own pool, or a
runtime whose device memory budget is fixed at start-up.  The caller hands in
device arrays it already owns.  The kernel's scratch sits in a fixed device
array inside the library.
This file checks, through the C ABI, that the result matches the allocating
entry point (cdmf_cuda_rmse_coo) on two calls in a row and on calls of
different sizes: the shared scratch must not carry one call's values into the
next.  The file is named to run last.
"""
import ctypes

import numpy as np
import pytest

from cdmf_gb300 import _lib

pytestmark = pytest.mark.gpu
RMSE_ATOL = 1e-5


def _case(seed, m, n, k, nt):
    rng = np.random.default_rng(seed)
    W = rng.standard_normal((k, m)).astype(np.float32)
    H = rng.standard_normal((k, n)).astype(np.float32)
    rows = rng.integers(0, m, nt).astype(np.uint32)
    cols = rng.integers(0, n, nt).astype(np.uint32)
    vals = rng.uniform(1, 5, nt).astype(np.float64)
    vals[::997] = np.nan                       # NaN terms are skipped but counted
    return W, H, rows, cols, vals


def _allocating(W, H, rows, cols, vals):
    k, m = W.shape
    n = H.shape[1]
    r = ctypes.c_double()
    nans = ctypes.c_int64()
    U = ctypes.c_uint32
    st = _lib.load().cdmf_cuda_rmse_coo(k, m, n, _lib.ptr(W, ctypes.c_float), _lib.ptr(H, ctypes.c_float),
                                        rows.size, _lib.ptr(rows, U), _lib.ptr(cols, U),
                                        _lib.ptr(vals, ctypes.c_double), 0, ctypes.byref(r), ctypes.byref(nans))
    assert st == 0, st
    return r.value, nans.value


def _noalloc(dev, stream):
    W, H, rows, cols, vals = dev
    k, m = W.shape
    n = H.shape[1]
    r = ctypes.c_double()
    nans = ctypes.c_int64()
    st = _lib.load().cdmf_cuda_rmse_coo_noalloc(k, m, n, W.data_ptr(), H.data_ptr(), rows.numel(), rows.data_ptr(),
                                                cols.data_ptr(), vals.data_ptr(), stream, ctypes.byref(r),
                                                ctypes.byref(nans))
    assert st == 0, st
    return r.value, nans.value


def _to_device(torch, arrays):
    out = []
    for a in arrays:
        t = torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()
        out.append(t)
    torch.cuda.synchronize()
    return out


def test_noalloc_matches_allocating_entry_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    stream = torch.cuda.current_stream().cuda_stream
    for seed, (m, n, k, nt) in enumerate([(3000, 700, 8, 5000), (40000, 9000, 16, 400000), (500, 80, 3, 1000)]):
        host = _case(seed, m, n, k, nt)
        ref, ref_nans = _allocating(*host)
        dev = _to_device(torch, host)
        for call in range(2):
            got, nans = _noalloc(dev, stream)
            assert abs(got - ref) <= RMSE_ATOL, (seed, call, got, ref)
            assert nans == ref_nans, (seed, call, nans, ref_nans)


def test_noalloc_rejects_oversized_and_bad_arguments():
    lib = _lib.load()
    r = ctypes.c_double()
    big = _lib.load().cdmf_cuda_rmse_coo_noalloc
    # beyond the stated maximum: rejected before any device work
    assert big(4, 10, 10, 1, 1, (1 << 31), 1, 1, 1, None, ctypes.byref(r), None) == -8
    assert lib.cdmf_cuda_rmse_coo_noalloc(0, 10, 10, 1, 1, 5, 1, 1, 1, None, ctypes.byref(r), None) == -1
    assert lib.cdmf_cuda_rmse_coo_noalloc(4, 10, 10, 1, 1, 0, 1, 1, 1, None, ctypes.byref(r), None) == -5
