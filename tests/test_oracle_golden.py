"""The CPU oracle against golden vectors produced by the reference's own
engine (tests/golden/make_golden.py runs src/cdmf_ref.cpp unmodified)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from cdmf_gb300 import formats
from oracle import oracle

META = json.load(open(os.path.join(GOLDEN, "golden.json")))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32 if a.dtype == np.float32 else np.uint64)


@pytest.mark.parametrize("name", ["simple", "tricky_simple", "mini"])
def test_oracle_bit_exact_vs_reference(name):
    R, z = load_golden(name)
    md = META[name]
    out = oracle.ccdpp(R, z["W0"], md["k"], md["lam"], md["maxiter"], md["maxinner"], threads=2, history=True,
                       residuals=True)
    assert np.array_equal(bits(out["W_hist"]), bits(z["W_hist"]))
    assert np.array_equal(bits(out["H_hist"]), bits(z["H_hist"]))
    assert np.array_equal(bits(out["res_csc"]), bits(z["res_csc"]))
    assert np.array_equal(bits(out["res_csr"]), bits(z["res_csr"]))
    assert np.array_equal(out["rmse"], z["rmse"])


def test_simple_known_values():
    # data/simple with the reference's ctest flags: the values the reference prints
    md = META["simple"]
    assert abs(md["rmse"][-1] - 0.097691) < 5e-7
    _, z = load_golden("simple")
    assert abs(float(z["W_hist"][-1][0][0]) - 1.35162961) < 1e-7
    assert abs(META["tricky_simple"]["rmse"][-1] - 1.225676) < 5e-7


def test_oracle_cpu_scale_digest():
    from golden.make_golden import matrix_digest  # noqa: F401  (same digest definition)
    from cdmf_gb300 import synth
    md = META["cpu_scale"]
    R, run = synth.config("cpu_scale")
    if matrix_digest(R) != md["matrix_sha256"]:
        pytest.skip("generator output differs on this host's libm; digests do not apply")
    W0 = synth.initial_w(md["k"], R.m, seed=0)
    out = oracle.ccdpp(R, W0, md["k"], md["lam"], md["maxiter"], md["maxinner"], threads=4, history=True)
    assert [hashlib.sha256(w.tobytes()).hexdigest() for w in out["W_hist"]] == md["W_sha256"]
    assert [hashlib.sha256(h.tobytes()).hexdigest() for h in out["H_hist"]] == md["H_sha256"]
    assert np.array_equal(out["rmse"], np.array(md["rmse"]))


def test_oracle_thread_invariance():
    R, z = load_golden("mini")
    md = META["mini"]
    a = oracle.ccdpp(R, z["W0"], md["k"], md["lam"], 2, md["maxinner"], threads=1)
    b = oracle.ccdpp(R, z["W0"], md["k"], md["lam"], 2, md["maxinner"], threads=4)
    assert np.array_equal(bits(a["W"]), bits(b["W"])) and np.array_equal(bits(a["H"]), bits(b["H"]))


def test_outer_iteration_composes():
    # running outer iterations one at a time from the state equals one run
    R, z = load_golden("mini")
    md = META["mini"]
    k = md["k"]
    W = z["W0"].copy()
    H = np.zeros((k, R.n), np.float32)
    rc, rr = R.csc_val.copy(), R.csr_val.copy()
    for j in range(1, md["maxiter"] + 1):
        oracle.outer_iteration(R, W, H, rc, rr, k, md["lam"], md["maxinner"], j, threads=2)
        assert np.array_equal(bits(W), bits(z["W_hist"][j - 1]))
        assert np.array_equal(bits(H), bits(z["H_hist"][j - 1]))
    assert np.array_equal(bits(rc), bits(z["res_csc"]))


def test_fp64_oracle_tracks_fp32():
    R, z = load_golden("mini")
    md = META["mini"]
    a = oracle.ccdpp(R, z["W0"], md["k"], md["lam"], md["maxiter"], md["maxinner"], dtype=np.float32)
    b = oracle.ccdpp(R, z["W0"].astype(np.float64), md["k"], md["lam"], md["maxiter"], md["maxinner"],
                     dtype=np.float64)
    assert np.max(np.abs(a["rmse"] - b["rmse"])) < 1e-4
    assert np.max(np.abs(a["W"] - b["W"])) < 1e-3 * np.max(np.abs(b["W"]))


def test_oracle_objective_hand_case():
    """2 x 2 ratings [[1, 0], [2, 3]] (3 nonzeros), k = 1: the FP64 objective
    by hand: residual squares plus lambda times count-weighted factor norms."""
    e = np.zeros(0, np.uint32)
    R = formats.from_coo(2, 2, np.array([0, 1, 1]), np.array([0, 0, 1]), np.array([1.0, 2.0, 3.0], np.float32),
                         e, e, np.zeros(0, np.float32))
    W = np.array([[0.5, 2.0]], np.float32)
    H = np.array([[1.0, -1.0]], np.float32)
    res = np.array([0.25, -0.5, 1.0], np.float32)
    sq, reg, tot = oracle.objective(R, W, H, res, 0.5)
    assert sq == pytest.approx(0.0625 + 0.25 + 1.0, abs=1e-15)
    # rows: nnz 1 and 2; columns: nnz 2 and 1
    assert reg == pytest.approx(0.5 * (1 * 0.25 + 2 * 4.0 + 2 * 1.0 + 1 * 1.0), abs=1e-15)
    assert tot == pytest.approx(sq + reg, abs=1e-15)


def test_workload_fixture_jester_shape():
    """tests/golden/workloads.json (make_workloads.py) for the Jester-shaped
    workload: the generator still makes the recorded inputs, and the oracle
    reproduces the recorded FP32 trajectory exactly (the GPU workload tests
    compare against these trajectories)."""
    from golden.make_workloads import checksums
    from cdmf_gb300 import synth
    gold = json.load(open(os.path.join(GOLDEN, "workloads.json")))
    # make_workloads.py --pin ran the reference's own engine on these
    assert all(gold[w].get("reference_pinned") for w in ("jester_shape", "ml20m_shape", "netflix_shape"))
    g = gold["jester_shape"]
    R, run = synth.config("jester_shape")
    W0 = synth.initial_w(g["k"], R.m, seed=0)
    assert checksums(R, W0) == g["inputs"]
    out = oracle.ccdpp(R, W0, g["k"], g["lam"], g["maxiter"], g["maxinner"], threads=4)
    assert out["rmse"].tolist() == g["rmse_f32"]


@pytest.mark.parametrize("name", ["simple", "tricky_simple", "mini"])
def test_mixed_model_with_fp32_storage_is_the_reference(name):
    """oracle/mixed_model.c with FP32 storage (fused subtract and add-back,
    one residual array) reproduces the reference's own outputs bit for bit."""
    R, z = load_golden(name)
    md = META[name]
    out = oracle.mixed_model(R, z["W0"], md["k"], md["lam"], md["maxiter"], md["maxinner"], storage="f32",
                             threads=2)
    assert np.array_equal(bits(out["W"]), bits(z["W_hist"][-1]))
    assert np.array_equal(bits(out["H"]), bits(z["H_hist"][-1]))
    assert np.array_equal(out["rmse"], z["rmse"])


def test_mixed_model_first_iteration_drift_jester_shape():
    """The 16-bit model on the Jester-shaped workload: every outer iteration
    within 1e-3 of the FP64 oracle; the first outer iteration, which runs
    before the first refresh, drifts more in BF16 than in FP16, and less when
    refreshes are added inside it."""
    from cdmf_gb300 import synth
    g = json.load(open(os.path.join(GOLDEN, "workloads.json")))["jester_shape"]
    R, _ = synth.config("jester_shape")
    W0 = synth.initial_w(g["k"], R.m, seed=0)
    r64 = np.array(g["rmse_f64"])
    err = {}
    for storage, every in (("bf16", 0), ("bf16", 4), ("f16", 0)):
        out = oracle.mixed_model(R, W0, g["k"], g["lam"], g["maxiter"], g["maxinner"], storage=storage,
                                 refresh_every=every)
        d = np.abs(out["rmse"] - r64)
        assert np.all(d <= 1e-3), (storage, every, d.tolist())
        err[(storage, every)] = d[0]
        if every == 0:   # the trajectories the GPU workload test compares against
            assert out["rmse"].tolist() == g["model_" + storage]
    assert err[("f16", 0)] < err[("bf16", 0)] and err[("bf16", 4)] < err[("bf16", 0)], err
