"""Host-side data path: converter, on-disk format, generator, transposition."""
import ctypes
import os

import numpy as np
import pytest

from conftest import load_golden
from cdmf_gb300 import _lib, formats, synth


@pytest.mark.parametrize("name", ["simple", "tricky_simple", "mini"])
def test_converter_matches_scipy_structures(name):
    # golden structures were written by scipy's tocsr/tocsc (the reference's converter)
    R, _ = load_golden(name)
    mine = formats.from_coo(R.m, R.n, *R.coo(), R.te_row, R.te_col, R.te_val)
    for f in ("csr_ptr", "csr_idx", "csc_ptr", "csc_idx"):
        assert np.array_equal(getattr(mine, f), getattr(R, f)), f
    for f in ("csr_val", "csc_val"):
        assert np.array_equal(getattr(mine, f).view(np.uint32), getattr(R, f).view(np.uint32)), f


def test_duplicates_summed_and_explicit_zeros_kept():
    R = formats.from_coo(3, 3, [0, 0, 2, 1], [1, 1, 0, 2], [1.0, 2.0, 0.0, 4.0], [], [], [])
    assert R.nnz == 3
    assert R.csr_ptr.tolist() == [0, 1, 2, 3] and R.csr_val.tolist() == [3.0, 4.0, 0.0]
    assert R.csc_ptr.tolist() == [0, 1, 2, 3] and R.csc_idx.tolist() == [2, 0, 1]


def test_dir_roundtrip(tmp_path):
    R, _ = load_golden("mini")
    formats.write_dir(str(tmp_path), R)
    S = formats.read_dir(str(tmp_path))
    for f in ("csr_ptr", "csr_idx", "csr_val", "csc_ptr", "csc_idx", "csc_val", "te_row", "te_col", "te_val"):
        assert np.array_equal(getattr(S, f), getattr(R, f)), f
    meta = open(os.path.join(str(tmp_path), "meta")).read().split()
    assert meta[:3] == [str(R.m), str(R.n), str(R.nnz)]


def test_read_dir_truncated(tmp_path):
    R, _ = load_golden("simple")
    formats.write_dir(str(tmp_path), R)
    p = os.path.join(str(tmp_path), "R_train_csc.data.bin")
    open(p, "wb").write(open(p, "rb").read()[:-4])
    with pytest.raises(IOError):
        formats.read_dir(str(tmp_path))


def test_csr_to_csc_and_perm():
    R, _ = load_golden("mini")
    lib = _lib.load()
    cp = np.empty(R.n + 1, np.uint32)
    ci = np.empty(R.nnz, np.uint32)
    cv = np.empty(R.nnz, np.float32)
    perm = np.empty(R.nnz, np.uint32)
    U, F = ctypes.c_uint32, ctypes.c_float
    st = lib.cdmf_csr_to_csc(R.m, R.n, R.nnz, _lib.ptr(R.csr_ptr, U), _lib.ptr(R.csr_idx, U), _lib.ptr(R.csr_val, F),
                             _lib.ptr(cp, U), _lib.ptr(ci, U), _lib.ptr(cv, F), _lib.ptr(perm, U))
    assert st == 0
    assert np.array_equal(cp, R.csc_ptr) and np.array_equal(ci, R.csc_idx) and np.array_equal(cv, R.csc_val)
    assert np.array_equal(R.csr_val[perm], R.csc_val)
    assert np.array_equal(np.sort(perm), np.arange(R.nnz, dtype=np.uint32))


def test_synth_thread_invariance():
    a = synth.generate(threads=1, m=5000, n=800, nnz_total=80000, row_max=400, col_cap=2500, seed=11)
    b = synth.generate(threads=4, m=5000, n=800, nnz_total=80000, row_max=400, col_cap=2500, seed=11)
    for f in ("csr_ptr", "csr_idx", "csr_val", "csc_ptr", "csc_idx", "te_row", "te_col", "te_val"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_synth_cpu_scale_shape():
    R, run = synth.config("cpu_scale")
    assert (R.m, R.n, R.nnz + R.nnz_test, R.nnz_test) == (20000, 4000, 1_000_000, 10000)
    assert set(np.unique(R.csr_val).tolist()) <= {1.0, 2.0, 3.0, 4.0, 5.0}
    rows, cols, _ = R.coo()
    key = rows.astype(np.int64) * R.n + cols
    assert np.all(np.diff(key) > 0)                    # distinct, row-major sorted
    tkey = R.te_row.astype(np.int64) * R.n + R.te_col
    assert np.intersect1d(key, tkey).size == 0         # test disjoint from train
    assert run == dict(k=16, lambda_=0.05, maxiter=5, maxinneriter=1)


def test_initial_col_matches_reference():
    # simple.npz's W0 is the reference's own initial_col(10, 6) output
    _, z = load_golden("simple")
    X = synth.reference_initial_col(10, 6)
    assert np.array_equal(X.view(np.uint32), z["W0"].view(np.uint32))


def test_text_pair_and_test_file(tmp_path):
    """The reference fixtures' 1-based text format: a train/test pair read
    with from_text gives the structures from_coo gives for the 0-based
    entries, and the test.txt that write_dir emits for -p 1 reads back to
    the same test set."""
    R, _ = load_golden("mini")
    rows, cols, vals = R.coo()
    train = tmp_path / "mini.dat"
    test = tmp_path / "mini.test"
    train.write_text("".join(f"{i + 1} {j + 1} {float(v)!r}\n" for i, j, v in zip(rows, cols, vals)))
    test.write_text("".join(f"{i + 1}\t{j + 1}\t{float(v)!r}\n" for i, j, v in zip(R.te_row, R.te_col, R.te_val)))
    S = formats.from_text(str(train), str(test), R.m, R.n)
    for f in ("csr_ptr", "csr_idx", "csc_ptr", "csc_idx", "te_row", "te_col"):
        assert np.array_equal(getattr(S, f), getattr(R, f)), f
    for f in ("csr_val", "csc_val", "te_val"):
        assert np.array_equal(getattr(S, f).view(np.uint32), getattr(R, f).view(np.uint32)), f
    d = tmp_path / "dir"
    formats.write_dir(str(d), R)
    tr, tc, tv = formats.read_text_ratings(str(d / "test.txt"))
    assert np.array_equal(tr, R.te_row) and np.array_equal(tc, R.te_col)
    assert np.array_equal(tv.astype(np.float32).view(np.uint32), R.te_val.view(np.uint32))
    empty = tmp_path / "empty.txt"
    empty.write_text("")
    assert all(a.size == 0 for a in formats.read_text_ratings(str(empty)))
