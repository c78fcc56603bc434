"""cdmf's on-disk rating format and its in-memory matrix.

Directory layout, as the reference's converters write it
(data/a/a_compress.py:79-246) and its loader reads it (src/tools.cpp:271-347):
  meta_modified_all   "m n\\nnnz\\n" + 9 train file names + "nnz_test\\n" + 3 test file names
  meta                "m n\\nnnz train.txt\\nnnz_test test.txt\\n"  (src/tools.cpp:489-541)
  R_train_coo.{data,row,col}.bin, R_train_csr.{indptr,indices,data}.bin,
  R_train_csc.{indptr,indices,data}.bin, R_test_coo.{data,row,col}.bin
  test.txt            1-based "u i r" lines
Indices are int32 (read as 32-bit unsigned), values float32.
"""
import os
import warnings
from dataclasses import dataclass

import numpy as np

TRAIN_FILES = [
    "R_train_coo.data.bin", "R_train_coo.row.bin", "R_train_coo.col.bin",
    "R_train_csr.indptr.bin", "R_train_csr.indices.bin", "R_train_csr.data.bin",
    "R_train_csc.indptr.bin", "R_train_csc.indices.bin", "R_train_csc.data.bin",
]
TEST_FILES = ["R_test_coo.data.bin", "R_test_coo.row.bin", "R_test_coo.col.bin"]


@dataclass
class RatingMatrix:
    """Training matrix in CSR and CSC plus the test COO (SparseMatrix + TestData,
    src/pmf_util.h:13-161)."""
    m: int
    n: int
    csr_ptr: np.ndarray
    csr_idx: np.ndarray
    csr_val: np.ndarray
    csc_ptr: np.ndarray
    csc_idx: np.ndarray
    csc_val: np.ndarray
    te_row: np.ndarray
    te_col: np.ndarray
    te_val: np.ndarray

    @property
    def nnz(self):
        return int(self.csr_idx.size)

    @property
    def nnz_test(self):
        return int(self.te_row.size)

    @property
    def max_row_nnz(self):
        return int(np.diff(self.csr_ptr.astype(np.int64)).max()) if self.m else 0

    @property
    def max_col_nnz(self):
        return int(np.diff(self.csc_ptr.astype(np.int64)).max()) if self.n else 0

    def coo(self):
        """Row-major COO of the training matrix."""
        rows = np.repeat(np.arange(self.m, dtype=np.uint32), np.diff(self.csr_ptr.astype(np.int64)))
        return rows, self.csr_idx, self.csr_val


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def compress(m, n, rows, cols, vals):
    """COO -> canonical CSR and CSC: duplicates summed, indices ascending inside
    each line (what scipy's tocsr/tocsc give, data/a/a_compress.py:147-148)."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    if rows.size and (rows.min() < 0 or rows.max() >= m or cols.min() < 0 or cols.max() >= n):
        raise ValueError("COO index out of range")
    key = rows * n + cols
    order = np.argsort(key, kind="stable")
    key, vals = key[order], vals[order]
    uniq, start = np.unique(key, return_index=True)
    summed = np.add.reduceat(vals, start) if vals.size else vals
    r, c = uniq // n, uniq % n
    csr_ptr = np.zeros(m + 1, dtype=np.int64)
    np.add.at(csr_ptr, r + 1, 1)
    csr_ptr = np.cumsum(csr_ptr)
    corder = np.argsort(c, kind="stable")
    csc_ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(csc_ptr, c + 1, 1)
    csc_ptr = np.cumsum(csc_ptr)
    return (_u32(csr_ptr), _u32(c), _f32(summed), _u32(csc_ptr), _u32(r[corder]), _f32(summed[corder]))


def compress_gpu(m, n, rows, cols, vals, device=0):
    """compress() on the GPU through cdmf_cuda_compress: same arrays, bit for
    bit (duplicates summed in FP64 in input order, stored as float)."""
    import ctypes
    from . import _lib
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    cols = np.ascontiguousarray(cols, dtype=np.uint32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    nnz = rows.size
    if cols.size != nnz or vals.size != nnz:
        raise ValueError("rows, cols and vals differ in length")
    csr_ptr = np.empty(m + 1, np.uint32)
    csc_ptr = np.empty(n + 1, np.uint32)
    csr_idx, csc_idx = np.empty(nnz, np.uint32), np.empty(nnz, np.uint32)
    csr_val, csc_val = np.empty(nnz, np.float32), np.empty(nnz, np.float32)
    out = ctypes.c_int64()
    U32, F32, F64 = ctypes.c_uint32, ctypes.c_float, ctypes.c_double
    p = _lib.ptr
    _lib.check(_lib.load().cdmf_cuda_compress(m, n, nnz, p(rows, U32), p(cols, U32), p(vals, F64), device,
                                              p(csr_ptr, U32), p(csr_idx, U32), p(csr_val, F32), p(csc_ptr, U32),
                                              p(csc_idx, U32), p(csc_val, F32), ctypes.byref(out)),
               "cdmf_cuda_compress")
    u = out.value
    return csr_ptr, csr_idx[:u].copy(), csr_val[:u].copy(), csc_ptr, csc_idx[:u].copy(), csc_val[:u].copy()


def from_coo(m, n, rows, cols, vals, te_rows, te_cols, te_vals):
    csr_ptr, csr_idx, csr_val, csc_ptr, csc_idx, csc_val = compress(m, n, rows, cols, vals)
    return RatingMatrix(m, n, csr_ptr, csr_idx, csr_val, csc_ptr, csc_idx, csc_val,
                        _u32(te_rows), _u32(te_cols), _f32(te_vals))


def read_text_ratings(path):
    """1-based "u<ws>i<ws>r" lines -> 0-based int arrays and float values."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)   # an empty file is an empty set here
        data = np.loadtxt(path, dtype=np.float64, ndmin=2)
    if data.size == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0, np.float64)
    return data[:, 0].astype(np.int64) - 1, data[:, 1].astype(np.int64) - 1, data[:, 2]


def from_text(train_path, test_path, m=None, n=None):
    """The reference fixtures' text pair (e.g. data/simple/simple.dat + .test)."""
    r, c, v = read_text_ratings(train_path)
    tr, tc, tv = read_text_ratings(test_path)
    m = int(r.max() + 1) if m is None else m
    n = int(c.max() + 1) if n is None else n
    return from_coo(m, n, r, c, v, tr, tc, tv)


def write_dir(path, R):
    """Writes R in cdmf's directory format."""
    os.makedirs(path, exist_ok=True)
    rows, cols, vals = R.coo()
    arrays = [
        _f32(vals), rows.astype(np.int32), cols.astype(np.int32),
        R.csr_ptr.astype(np.int32), R.csr_idx.astype(np.int32), _f32(R.csr_val),
        R.csc_ptr.astype(np.int32), R.csc_idx.astype(np.int32), _f32(R.csc_val),
    ]
    for name, arr in zip(TRAIN_FILES, arrays):
        arr.tofile(os.path.join(path, name))
    for name, arr in zip(TEST_FILES, [_f32(R.te_val), R.te_row.astype(np.int32), R.te_col.astype(np.int32)]):
        arr.tofile(os.path.join(path, name))
    with open(os.path.join(path, "meta_modified_all"), "w") as f:
        f.write(f"{R.m} {R.n}\n{R.nnz}\n")
        f.write("".join(x + "\n" for x in TRAIN_FILES))
        f.write(f"{R.nnz_test}\n")
        f.write("".join(x + "\n" for x in TEST_FILES))
    with open(os.path.join(path, "meta"), "w") as f:
        f.write(f"{R.m} {R.n}\n{R.nnz} train.txt\n{R.nnz_test} test.txt\n")
    with open(os.path.join(path, "test.txt"), "w") as f:
        for i, j, v in zip(R.te_row.tolist(), R.te_col.tolist(), R.te_val.tolist()):
            f.write(f"{i + 1} {j + 1} {v!r}\n")


def read_dir(path):
    """Reads a cdmf directory the way load() does (src/tools.cpp:271-347)."""
    with open(os.path.join(path, "meta_modified_all")) as f:
        tok = f.read().split()
    m, n, nnz = int(tok[0]), int(tok[1]), int(tok[2])
    train = tok[3:12]
    nnz_test = int(tok[12])
    test = tok[13:16]

    def rd(name, dtype, count):
        a = np.fromfile(os.path.join(path, name), dtype=dtype, count=count)
        if a.size != count:
            raise IOError(f"{name}: expected {count} items, read {a.size}")
        return a

    return RatingMatrix(
        m, n,
        _u32(rd(train[3], np.uint32, m + 1)), _u32(rd(train[4], np.uint32, nnz)), _f32(rd(train[5], np.float32, nnz)),
        _u32(rd(train[6], np.uint32, n + 1)), _u32(rd(train[7], np.uint32, nnz)), _f32(rd(train[8], np.float32, nnz)),
        _u32(rd(test[1], np.uint32, nnz_test)), _u32(rd(test[2], np.uint32, nnz_test)),
        _f32(rd(test[0], np.float32, nnz_test)),
    )
