"""GPU COO -> CSR/CSC build (cdmf_cuda_compress) against the host restatement
of scipy's tocsr/tocsc (formats.compress, itself checked against the
reference fixtures' arrays): every array bit for bit."""
import numpy as np
import pytest

from conftest import load_golden
from cdmf_gb300 import _lib, formats, synth

pytestmark = pytest.mark.gpu


def _same(got, ref):
    names = ("csr_ptr", "csr_idx", "csr_val", "csc_ptr", "csc_idx", "csc_val")
    for name, g, r in zip(names, got, ref):
        assert g.dtype == r.dtype and g.shape == r.shape, name
        assert np.array_equal(g.view(np.uint32), r.view(np.uint32)), name


def test_random_coo_with_duplicates_bit_exact():
    rng = np.random.default_rng(7)
    m, n, nnz = 5000, 700, 200_000
    rows = rng.integers(0, m, nnz)
    cols = rng.integers(0, n, nnz)
    # a tenth of the entries repeated up to three times, in scattered order
    rep = rng.integers(0, nnz, nnz // 10)
    rows = np.concatenate([rows, rows[rep], rows[rep[::3]]])
    cols = np.concatenate([cols, cols[rep], cols[rep[::3]]])
    vals = rng.uniform(0.5, 5.0, rows.size)           # non-integer: the summation order shows
    perm = rng.permutation(rows.size)
    rows, cols, vals = rows[perm], cols[perm], vals[perm]
    _same(formats.compress_gpu(m, n, rows, cols, vals), formats.compress(m, n, rows, cols, vals))


@pytest.mark.parametrize("name", ["simple", "tricky_simple", "mini"])
def test_reference_fixture_arrays_from_shuffled_coo(name):
    """The reference's own CSR/CSC files (data/simple, data/tricky_simple) and
    the seeded mini case, rebuilt from their COO in random order."""
    R, _ = load_golden(name)
    rows, cols, vals = R.coo()
    perm = np.random.default_rng(1).permutation(rows.size)
    got = formats.compress_gpu(R.m, R.n, rows[perm], cols[perm], vals[perm].astype(np.float64))
    _same(got, (R.csr_ptr, R.csr_idx, R.csr_val, R.csc_ptr, R.csc_idx, R.csc_val))


def test_edge_cases():
    e = np.zeros(0, np.int64)
    got = formats.compress_gpu(3, 4, e, e, np.zeros(0))
    assert np.array_equal(got[0], np.zeros(4, np.uint32)) and np.array_equal(got[3], np.zeros(5, np.uint32))
    assert all(a.size == 0 for a in (got[1], got[2], got[4], got[5]))
    # empty first/last rows and columns, one row, one column
    for m, n, rows, cols in [(6, 5, [2, 2, 3], [1, 3, 1]), (1, 9, [0, 0, 0], [8, 0, 4]), (7, 1, [6, 0, 3], [0, 0, 0])]:
        rows, cols = np.array(rows), np.array(cols)
        vals = np.arange(1.0, rows.size + 1)
        _same(formats.compress_gpu(m, n, rows, cols, vals), formats.compress(m, n, rows, cols, vals))
    # an index out of range is rejected before anything is written
    with pytest.raises(_lib.CdmfError) as ei:
        formats.compress_gpu(4, 4, np.array([0, 4]), np.array([1, 1]), np.array([1.0, 2.0]))
    assert ei.value.status == -1


def test_movielens_shaped_matrix_round_trip():
    """20M nonzeros: the generator's CSR/CSC, rebuilt from its COO in random
    order."""
    R, _ = synth.config("ml20m_shape")
    rows, cols, vals = R.coo()
    perm = np.random.default_rng(3).permutation(rows.size)
    got = formats.compress_gpu(R.m, R.n, rows[perm], cols[perm], vals[perm].astype(np.float64))
    _same(got, (R.csr_ptr, R.csr_idx, R.csr_val, R.csc_ptr, R.csc_idx, R.csc_val))
