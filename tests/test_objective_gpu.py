"""FP64 objective monitor (cdmf_cuda_objective) against the oracle's FP64
restatement, and CCD++'s descent property at a realistic size.

The objective is sum r_ij^2 + lambda (sum_i nnz_i |w_i|^2 + sum_j nnz_j |h_j|^2):
the loss UpdateRating accumulates (src/cdmf_ref.cpp:20-43) plus the
regulariser whose coordinate minimiser is RankOneUpdate (src/cdmf_ref.cpp:7-17).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from cdmf_gb300 import engine, synth
from oracle import oracle

pytestmark = pytest.mark.gpu

META = json.load(open(os.path.join(GOLDEN, "golden.json")))
SUM_RTOL = 1e-12      # FP64 sums of the same float32 values in another order
DESCENT_RTOL = 1e-6   # FP32 rounding of the factor updates between two monitors


def _close(a, b, rtol):
    return abs(a - b) <= rtol * max(1.0, abs(b))


def test_objective_matches_oracle_on_reference_state():
    """Reference order gives the reference's state bit for bit; the objective
    of that state must equal the oracle's FP64 objective of the golden state."""
    R, z = load_golden("mini")
    md = META["mini"]
    with engine.Engine(R, md["k"], md["lam"], md["maxiter"], md["maxinner"], reduce="sequential") as e:
        e.set_factors(z["W0"])
        before = e.objective()
        ref0 = oracle.objective(R, z["W0"], np.zeros((md["k"], R.n), np.float32), R.csc_val, md["lam"])
        for a, b in zip(before, ref0):
            assert _close(a, b, SUM_RTOL), (before, ref0)
        e.run(md["maxiter"])
        got = e.objective()
    ref = oracle.objective(R, z["W_hist"][-1], z["H_hist"][-1], z["res_csc"], md["lam"])
    for a, b in zip(got, ref):
        assert _close(a, b, SUM_RTOL), (got, ref)
    assert got[2] < before[2]


@pytest.mark.parametrize("residual,layout", [("f32", "lines"), ("bf16", "lines"), ("f16", "lines"),
                                             ("f32", "blocked")])
def test_objective_matches_own_state(residual, layout):
    """Any residual mode or layout: the monitor equals the FP64 objective of
    the state the engine hands back."""
    R, run = synth.config("cpu_scale")
    W0 = synth.initial_w(run["k"], R.m, seed=0)
    with engine.Engine(R, run["k"], run["lambda_"], 3, 1, residual=residual, layout=layout) as e:
        e.set_factors(W0)
        e.run(2)
        got = e.objective()
        st = e.state()
    ref = oracle.objective(R, st["W"], st["H"], st["res_csc"], run["lambda_"])
    for a, b in zip(got, ref):
        assert _close(a, b, 1e-9), (got, ref)


def test_objective_descends_each_outer_netflix_like_rows():
    """Every rank-one update minimises the objective exactly in one block of
    coordinates, so it never rises between outer iterations (up to FP32
    rounding of the updates)."""
    R, run = synth.config("cpu_scale")
    W0 = synth.initial_w(16, R.m, seed=1)
    with engine.Engine(R, 16, run["lambda_"], 8, 1) as e:
        e.set_factors(W0)
        prev = e.objective()[2]
        for _ in range(6):
            e.run(1)
            cur = e.objective()[2]
            assert cur <= prev * (1 + DESCENT_RTOL), (cur, prev)
            prev = cur
