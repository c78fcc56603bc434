"""Dual SpMV front end (cdmf_spmv_*), the replacement for the reference's
CSR5 handle (src/anonymouslib_opencl.h:11-26): y_t = A x and y_b = row sums
of x^2 over each row's pattern (csr5_spmv.cl:135-147), checked against FP64
numpy on a matrix whose rows fall in every work class (split, CTA, warp,
8-lane group, thread, empty)."""
import ctypes

import numpy as np
import pytest

from cdmf_gb300 import _lib, formats

pytestmark = pytest.mark.gpu
SUM_RTOL = 1e-5   # FP32 tree sums: bound relative to the sum of |terms|


def _matrix(seed=0):
    rng = np.random.default_rng(seed)
    n = 120000
    lens = np.concatenate([[90000, 0, 17000], rng.integers(4097, 9000, 6), rng.integers(257, 4096, 40),
                           rng.integers(13, 256, 400), rng.integers(1, 12, 3000), np.zeros(50, np.int64)])
    rng.shuffle(lens)
    rows = np.repeat(np.arange(lens.size), lens)
    cols = np.concatenate([rng.choice(n, size=L, replace=False) if L <= n else rng.integers(0, n, L) for L in lens])
    vals = rng.standard_normal(rows.size)
    m = lens.size
    csr_ptr, csr_idx, csr_val, *_ = formats.compress(m, n, rows, cols, vals)
    x = rng.standard_normal(n).astype(np.float32)
    return m, n, csr_ptr, csr_idx, csr_val, x


class Handle:
    def __init__(self, m, n):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        assert self.lib.cdmf_spmv_create(m, n, 0, ctypes.byref(h)) == 0
        self.h = h

    def close(self):
        self.lib.cdmf_spmv_destroy(self.h)


def _dev(torch, a):
    return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()


def test_dual_spmv_matches_fp64_and_repeats_bit_for_bit():
    torch = pytest.importorskip("torch")
    m, n, ptr, idx, val, x = _matrix()
    dp, di, dv, dx = (_dev(torch, a) for a in (ptr, idx, val, x))
    yt = torch.empty(m, dtype=torch.float32, device="cuda")
    yb = torch.empty(m, dtype=torch.float32, device="cuda")
    H = Handle(m, n)
    lib = H.lib
    try:
        assert lib.cdmf_spmv_input_csr(H.h, idx.size, dp.data_ptr(), di.data_ptr(), dv.data_ptr()) == 0
        assert lib.cdmf_spmv_set_x(H.h, dx.data_ptr()) == 0
        # CSR form: no SpMV, as the reference's handle refuses it
        assert lib.cdmf_spmv_run(H.h, 1.0, yt.data_ptr(), yb.data_ptr(), None) == -7
        assert lib.cdmf_spmv_as_csr5(H.h) == 0
        ms = ctypes.c_double()
        assert lib.cdmf_spmv_run(H.h, 1.0, yt.data_ptr(), yb.data_ptr(), ctypes.byref(ms)) == 0
        t1, b1 = yt.cpu().numpy().copy(), yb.cpu().numpy().copy()
        assert lib.cdmf_spmv_run(H.h, 1.0, yt.data_ptr(), yb.data_ptr(), None) == 0
        assert np.array_equal(t1.view(np.uint32), yt.cpu().numpy().view(np.uint32))
        assert np.array_equal(b1.view(np.uint32), yb.cpu().numpy().view(np.uint32))
        assert lib.cdmf_spmv_as_csr(H.h) == 0
        assert lib.cdmf_spmv_run(H.h, 1.0, yt.data_ptr(), yb.data_ptr(), None) == -7
    finally:
        H.close()
    rows = np.repeat(np.arange(m), np.diff(ptr.astype(np.int64)))
    xv = x.astype(np.float64)[idx]
    terms = val.astype(np.float64) * xv
    ref_t = np.bincount(rows, terms, minlength=m)
    ref_b = np.bincount(rows, xv * xv, minlength=m)
    scale_t = np.bincount(rows, np.abs(terms), minlength=m)
    assert np.all(np.abs(t1 - ref_t) <= SUM_RTOL * scale_t + 1e-30)
    assert np.all(np.abs(b1 - ref_b) <= SUM_RTOL * ref_b + 1e-30)
    assert np.all(t1[np.diff(ptr) == 0] == 0) and np.all(b1[np.diff(ptr) == 0] == 0)


def test_malformed_input_refused():
    torch = pytest.importorskip("torch")
    m, n = 4, 5
    lib = _lib.load()
    H = Handle(m, n)
    try:
        bad_ptr = _dev(torch, np.array([0, 2, 1, 3, 3], np.uint32))     # not monotone
        idx = _dev(torch, np.array([0, 1, 2], np.uint32))
        val = _dev(torch, np.ones(3, np.float32))
        assert lib.cdmf_spmv_input_csr(H.h, 3, bad_ptr.data_ptr(), idx.data_ptr(), val.data_ptr()) == -1
        ptr = _dev(torch, np.array([0, 2, 2, 3, 3], np.uint32))
        oob = _dev(torch, np.array([0, 5, 2], np.uint32))                # column 5 of 5
        assert lib.cdmf_spmv_input_csr(H.h, 3, ptr.data_ptr(), oob.data_ptr(), val.data_ptr()) == 0
        assert lib.cdmf_spmv_as_csr5(H.h) == -1
    finally:
        H.close()
