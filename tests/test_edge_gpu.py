"""Degenerate shapes through the engine, against the oracle: a single
nonzero, one row, one column, mostly empty lines, no nonzeros at all, k = 1,
and every residual mode on them (the reference handles empty lines at
src/cdmf_ref.cpp:9 by returning 0)."""
import numpy as np
import pytest

from cdmf_gb300 import engine, formats, synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _matrix(m, n, cells, test_cells=((0, 0),), seed=0):
    rng = np.random.default_rng(seed)
    rows = np.array([c[0] for c in cells], np.int64)
    cols = np.array([c[1] for c in cells], np.int64)
    vals = rng.integers(1, 6, len(cells)).astype(np.float32)
    tr = np.array([c[0] for c in test_cells], np.uint32)
    tc = np.array([c[1] for c in test_cells], np.uint32)
    tv = rng.integers(1, 6, len(test_cells)).astype(np.float32)
    return formats.from_coo(m, n, rows, cols, vals, tr, tc, tv)


def _cases():
    rng = np.random.default_rng(5)
    sparse = sorted({(int(rng.integers(0, 60)), int(rng.integers(0, 45))) for _ in range(7)})
    row = [(0, j) for j in range(0, 300, 3)]
    col = [(i, 0) for i in range(0, 500, 2)]
    return {
        "single": (1, 1, [(0, 0)]),
        "one_row": (1, 300, row),
        "one_col": (500, 1, col),
        "mostly_empty": (60, 45, sparse),
    }


@pytest.mark.parametrize("name", ["single", "one_row", "one_col", "mostly_empty"])
@pytest.mark.parametrize("k", [1, 3])
def test_degenerate_shapes_sequential_bit_exact(name, k):
    m, n, cells = _cases()[name]
    R = _matrix(m, n, cells)
    W0 = synth.initial_w(k, m, seed=1)
    ref = oracle.ccdpp(R, W0, k, 0.05, 3, 2, threads=1, history=True)
    with engine.Engine(R, k, 0.05, 3, 2, reduce="sequential") as e:
        e.set_factors(W0)
        rm = e.run(3)
        W, H = e.factors()
    assert np.array_equal(bits(W), bits(ref["W"])) and np.array_equal(bits(H), bits(ref["H"]))
    assert np.max(np.abs(rm - ref["rmse"])) <= 1e-12


@pytest.mark.parametrize("name", ["single", "one_row", "one_col", "mostly_empty"])
@pytest.mark.parametrize("residual,version", [("f32", 1), ("bf16", 1), ("f16", 1), ("f32", 3)])
def test_degenerate_shapes_all_modes(name, residual, version):
    m, n, cells = _cases()[name]
    R = _matrix(m, n, cells)
    k = 2
    W0 = synth.initial_w(k, m, seed=2)
    r64 = oracle.ccdpp(R, W0.astype(np.float64), k, 0.05, 3, 1, dtype=np.float64)
    with engine.Engine(R, k, 0.05, 3, 1, residual=residual, version=version) as e:
        e.set_factors(W0)
        rm = e.run(3)
        W, H = e.factors()
    tol = 1e-3 if residual != "f32" else 1e-5
    assert np.all(np.isfinite(W)) and np.all(np.isfinite(H))
    assert abs(rm[-1] - r64["rmse"][-1]) <= tol * max(1.0, r64["rmse"][-1]), (rm, r64["rmse"])


def test_no_nonzeros():
    """An empty training matrix: every line is empty, so W and H become 0
    (src/cdmf_ref.cpp:9) and the RMSE is that of predicting 0."""
    R = _matrix(7, 5, [], test_cells=((1, 2), (6, 4)))
    W0 = synth.initial_w(3, 7, seed=0)
    for residual in ("f32", "bf16"):
        with engine.Engine(R, 3, 0.05, 2, 1, residual=residual) as e:
            e.set_factors(W0)
            rm = e.run(2)
            W, H = e.factors()
        assert not W.any() and not H.any()
        expect = float(np.sqrt(np.mean(R.te_val.astype(np.float64) ** 2)))
        assert abs(rm[-1] - expect) <= 1e-12
