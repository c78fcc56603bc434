"""The synthetic stand-ins for the reference's Jester, MovieLens-20M and
Netflix runs (their shapes, value distributions, k, lambda and outer x
inner; the Netflix shape at k = 64, the benchmark's configuration, and at
k = 32) through the engine, against the oracle's test-RMSE trajectories in
tests/golden/workloads.json (FP32 = the reference's arithmetic, pinned bit for
bit to the reference's own engine; FP64 = the same algorithm in double),
after every outer iteration:
  - FP32 residual, tree order, versions 1 and 3: within the reference's own
    FP32 error of the FP64 oracle, max(1e-5, 2 |rmse32 - rmse64|);
  - FP16 and BF16 residuals: within 1e-3 of the FP64 oracle;
  - FP16 and BF16: on the trajectory of the CPU model of the 16-bit mode
    (oracle/mixed_model.c, the engine's refresh schedule) to within twice the
    reference's FP32 error + 2e-5;
  - reference order (Jester-shaped): the FP32 oracle's RMSE to 1e-12;
  - the benchmark's options (CUDA graphs, autotuned bins) on the Netflix
    shapes: the same bounds.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from cdmf_gb300 import engine, synth

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(GOLDEN, "workloads.json")))
FP32_FLOOR = 1e-5
MIXED_ATOL = 1e-3
SEQ_ATOL = 1e-12
MODEL_ATOL = 2e-5
EARLY_REFRESH = 32   # the engine's refresh period (features) in the first outer iteration


def bit_sum(a):
    return int(np.ascontiguousarray(a).view(np.uint32).astype(np.int64).sum())


def inputs_checksums(R, W0):
    return dict(m=int(R.m), n=int(R.n), nnz=int(R.nnz), nnz_test=int(R.te_val.size),
                csr_idx_sum=bit_sum(R.csr_idx), csr_val_sum=bit_sum(R.csr_val), te_row_sum=bit_sum(R.te_row),
                te_val_sum=bit_sum(R.te_val), w0_sum=bit_sum(W0))


# Fixture name -> (generator preset, run-parameter overrides).
VARIANTS = {"netflix_shape_k32": ("netflix_shape", {"k": 32})}
_MATRICES = {}


def _matrix(preset):
    """One generated matrix per preset at a time (the Netflix shape holds
    about 2 GB of host memory)."""
    if preset not in _MATRICES:
        _MATRICES.clear()
        _MATRICES[preset] = synth.config(preset)
    R, run = _MATRICES[preset]
    return R, dict(run)


@pytest.fixture(scope="module", params=["jester_shape", "ml20m_shape", "netflix_shape", "netflix_shape_k32"])
def workload(request):
    name = request.param
    g = GOLD[name]
    preset, over = VARIANTS.get(name, (name, {}))
    R, run = _matrix(preset)
    run.update(over)
    assert (run["k"], run["maxiter"], run["maxinneriter"]) == (g["k"], g["maxiter"], g["maxinner"])
    assert g.get("reference_pinned"), "the FP32 trajectory is pinned to the reference's own engine"
    W0 = synth.initial_w(g["k"], R.m, seed=0)
    assert inputs_checksums(R, W0) == g["inputs"], "the generator no longer makes the matrix of the trajectories"
    return name, R, W0, g


def _run(R, W0, g, **kw):
    with engine.Engine(R, g["k"], g["lam"], g["maxiter"], g["maxinner"], **kw) as e:
        e.set_factors(W0)
        rm = e.run(g["maxiter"])
        st = e.stats()
    assert st["nonfinite"] == 0
    return np.asarray(rm, np.float64)


@pytest.mark.parametrize("version", [1, 3])
def test_fp32_within_reference_error(workload, version):
    name, R, W0, g = workload
    r32, r64 = np.asarray(g["rmse_f32"]), np.asarray(g["rmse_f64"])
    rm = _run(R, W0, g, residual="f32", version=version)
    bound = np.maximum(FP32_FLOOR, 2 * np.abs(r32 - r64))
    assert np.all(np.abs(rm - r64) <= bound), (name, (rm - r64).tolist(), bound.tolist())


@pytest.mark.parametrize("residual", ["f16", "bf16"])
def test_mixed_within_1e3_of_fp64(workload, residual):
    name, R, W0, g = workload
    r64 = np.asarray(g["rmse_f64"])
    rm = _run(R, W0, g, residual=residual)
    assert np.all(np.abs(rm - r64) <= MIXED_ATOL), (name, residual, (rm - r64).tolist())
    # the engine follows the CPU model of its 16-bit mode (oracle/mixed_model.c)
    # to within twice the reference's own FP32 error: the model sums each
    # line sequentially, as the reference does, the engine in trees
    assert g.get("model_early_refresh") == EARLY_REFRESH, "model trajectory of another refresh schedule"
    model, r32 = np.asarray(g["model_" + residual]), np.asarray(g["rmse_f32"])
    tol = 2 * np.abs(r32 - r64) + MODEL_ATOL
    assert np.all(np.abs(rm - model) <= tol), (name, residual, (rm - model).tolist(), tol.tolist())


def test_reference_order_matches_fp32_oracle(workload):
    name, R, W0, g = workload
    if name != "jester_shape":
        pytest.skip("one thread per line is slow on the 67k-nonzero columns; the Jester shape covers it")
    rm = _run(R, W0, g, residual="f32", reduce="sequential")
    assert np.max(np.abs(rm - np.asarray(g["rmse_f32"]))) <= SEQ_ATOL, (rm - np.asarray(g["rmse_f32"])).tolist()


@pytest.mark.parametrize("residual", ["f32", "bf16"])
def test_benchmark_options(workload, residual):
    """The benchmark's own engine options -- outer iterations replayed as CUDA
    graphs, bin limits picked by the autotuner -- on the Netflix-shaped
    workloads it measures, held to the same trajectories."""
    name, R, W0, g = workload
    if not name.startswith("netflix_shape"):
        pytest.skip("the benchmark runs the Netflix-shaped workload")
    rm = _run(R, W0, g, residual=residual, use_graph=True, autotune=True)
    r32, r64 = np.asarray(g["rmse_f32"]), np.asarray(g["rmse_f64"])
    if residual == "f32":
        bound = np.maximum(FP32_FLOOR, 2 * np.abs(r32 - r64))
        assert np.all(np.abs(rm - r64) <= bound), (name, (rm - r64).tolist(), bound.tolist())
        return
    assert np.all(np.abs(rm - r64) <= MIXED_ATOL), (name, residual, (rm - r64).tolist())
    model = np.asarray(g["model_" + residual])
    tol = 2 * np.abs(r32 - r64) + MODEL_ATOL
    assert np.all(np.abs(rm - model) <= tol), (name, residual, (rm - model).tolist(), tol.tolist())
