"""CUDA engine vs the oracle and the reference's golden vectors.

Two reduction modes:
  sequential -- every line is summed by one thread in index order, the
                reference's order: results must be BIT-EXACT after every outer
                iteration (W, H, both residual copies) and the RMSE equal;
  tree       -- the production mode (warp / CTA / split-line trees).  A
                reordered FP32 sum cannot reproduce the reference's rounding,
                and CCD++ amplifies rounding through the residual chain (the
                first feature agrees to ~1e-7; later features inherit the
                previous features' rounding), so the bar is the reference's
                OWN FP32 error, measured against the FP64 oracle on the same
                inputs.  After every outer iteration:
                  fro(gpu - ref32) <= 2 * fro(ref32 - ref64) + 1e-6
                  fro(gpu - ref64) <= 1.5 * fro(ref32 - ref64) + 1e-7
                  elementwise rel(gpu, ref32) <= 2 * rel(ref32, ref64) + 1e-4
                  |rmse_gpu - rmse_ref32| <= max(1e-5, 2 * |rmse_ref32 - rmse_ref64|)
                fro(x - r) = ||x - r||_F / ||r||_F; rel(x, r) = max |x - r| /
                max(|r|, 0.1 * rms of r's feature vector).
"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from cdmf_gb300 import _lib, engine, synth
from oracle import oracle

pytestmark = pytest.mark.gpu
META = json.load(open(os.path.join(GOLDEN, "golden.json")))
RTOL = 1e-5
RMSE_ATOL = 1e-5


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def rel_err(x, ref):
    x = np.asarray(x, np.float64).reshape(ref.shape[0], -1)
    ref = np.asarray(ref, np.float64).reshape(ref.shape[0], -1)
    rms = np.sqrt(np.mean(ref * ref, axis=1, keepdims=True))
    scale = np.maximum(np.abs(ref), 0.1 * rms)
    return float((np.abs(x - ref) / np.where(scale > 0, scale, 1.0)).max())


def fro(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    nr = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (nr if nr > 0 else 1.0))


def within_budget(x, ref32, ref64):
    """x (GPU, tree order) against the reference's own FP32 error budget."""
    b_fro = fro(ref32, ref64)
    b_rel = rel_err(ref32, ref64)
    got = dict(fro32=fro(x, ref32), fro64=fro(x, ref64), rel32=rel_err(x, ref32), budget_fro=b_fro, budget_rel=b_rel)
    ok = (got["fro32"] <= 2 * b_fro + 1e-6 and got["fro64"] <= 1.5 * b_fro + 1e-7
          and got["rel32"] <= 2 * b_rel + 1e-4)
    return ok, got


@pytest.mark.parametrize("name", ["simple", "tricky_simple", "mini"])
def test_sequential_bit_exact_each_outer(name):
    R, z = load_golden(name)
    md = META[name]
    with engine.Engine(R, md["k"], md["lam"], md["maxiter"], md["maxinner"], reduce="sequential") as e:
        e.set_factors(z["W0"])
        for j in range(md["maxiter"]):
            rm = e.run(1)
            W, H = e.factors()
            assert np.array_equal(bits(W), bits(z["W_hist"][j])), f"W after outer {j + 1}"
            assert np.array_equal(bits(H), bits(z["H_hist"][j])), f"H after outer {j + 1}"
            assert abs(rm[0] - z["rmse"][j]) <= 1e-12
        st = e.state()
    assert np.array_equal(bits(st["res_csc"]), bits(z["res_csc"]))
    assert np.array_equal(bits(st["res_csr"]), bits(z["res_csr"]))


def rmse_ok(got, r32, r64):
    return abs(got - r32) <= max(RMSE_ATOL, 2 * abs(r32 - r64))


@pytest.mark.parametrize("version", [1, 3])
@pytest.mark.parametrize("name", ["simple", "tricky_simple", "mini"])
def test_tree_within_fp32_budget_each_outer(name, version):
    R, z = load_golden(name)
    md = META[name]
    r64 = oracle.ccdpp(R, z["W0"].astype(np.float64), md["k"], md["lam"], md["maxiter"], md["maxinner"],
                       dtype=np.float64, history=True)
    with engine.Engine(R, md["k"], md["lam"], md["maxiter"], md["maxinner"], version=version) as e:
        e.set_factors(z["W0"])
        for j in range(md["maxiter"]):
            rm = e.run(1)
            W, H = e.factors()
            okw, gw = within_budget(W, z["W_hist"][j], r64["W_hist"][j])
            okh, gh = within_budget(H, z["H_hist"][j], r64["H_hist"][j])
            assert okw and okh, (j, gw, gh)
            assert rmse_ok(rm[0], z["rmse"][j], r64["rmse"][j]), (rm[0], z["rmse"][j], r64["rmse"][j])


def test_one_shot_train_matches_handle_api():
    R, z = load_golden("mini")
    md = META["mini"]
    W, H, rm = engine.train(R, z["W0"], md["k"], md["lam"], md["maxiter"], md["maxinner"], reduce="sequential")
    assert np.array_equal(bits(W), bits(z["W_hist"][-1])) and np.array_equal(bits(H), bits(z["H_hist"][-1]))
    assert np.max(np.abs(rm - z["rmse"])) <= 1e-12


@pytest.fixture(scope="module")
def cpu_scale():
    R, run = synth.config("cpu_scale")
    W0 = synth.initial_w(run["k"], R.m, seed=0)
    ref = oracle.ccdpp(R, W0, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"], threads=8,
                       history=True, residuals=True)
    ref["f64"] = oracle.ccdpp(R, W0.astype(np.float64), run["k"], run["lambda_"], run["maxiter"],
                              run["maxinneriter"], threads=8, dtype=np.float64, history=True)
    return R, run, W0, ref


def test_cpu_scale_sequential_bit_exact(cpu_scale):
    R, run, W0, ref = cpu_scale
    with engine.Engine(R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"], reduce="sequential") as e:
        e.set_factors(W0)
        for j in range(run["maxiter"]):
            rm = e.run(1)
            W, H = e.factors()
            assert np.array_equal(bits(W), bits(ref["W_hist"][j])) and np.array_equal(bits(H), bits(ref["H_hist"][j]))
            assert abs(rm[0] - ref["rmse"][j]) <= 1e-12
        st = e.state()
    assert np.array_equal(bits(st["res_csc"]), bits(ref["res_csc"]))
    assert np.array_equal(bits(st["res_csr"]), bits(ref["res_csr"]))


@pytest.mark.parametrize("version", [1, 3])
def test_cpu_scale_tree_one_step_parity(cpu_scale, version):
    """From the oracle's state after outer j, one GPU outer iteration lands
    within the FP32 budget of the oracle's outer j+1 (errors do not compound)."""
    R, run, W0, ref = cpu_scale
    k, lam, T = run["k"], run["lambda_"], run["maxinneriter"]
    W = W0.copy()
    H = np.zeros((k, R.n), np.float32)
    rc, rr = R.csc_val.copy(), R.csr_val.copy()
    with engine.Engine(R, k, lam, run["maxiter"], T, version=version) as e:
        for j in range(1, run["maxiter"] + 1):
            e.set_state(W, H, rc, rr, j)
            rm = e.run(1)
            Wg, Hg = e.factors()
            W64, H64 = W.astype(np.float64), H.astype(np.float64)
            rc64, rr64 = rc.astype(np.float64), rr.astype(np.float64)
            oracle.outer_iteration(R, W64, H64, rc64, rr64, k, lam, T, j, threads=8)
            oracle.outer_iteration(R, W, H, rc, rr, k, lam, T, j, threads=8)
            okw, gw = within_budget(Wg, W, W64)
            okh, gh = within_budget(Hg, H, H64)
            assert okw and okh, (j, gw, gh)
            assert rmse_ok(rm[0], oracle.rmse(R, W, H, k), oracle.rmse(R, W64, H64, k))


@pytest.mark.parametrize("version", [1, 3])
def test_cpu_scale_tree_free_running(cpu_scale, version):
    R, run, W0, ref = cpu_scale
    with engine.Engine(R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"], version=version) as e:
        e.set_factors(W0)
        rm = e.run(run["maxiter"])
        W, H = e.factors()
    assert all(rmse_ok(a, b, c) for a, b, c in zip(rm, ref["rmse"], ref["f64"]["rmse"])), (rm, ref["rmse"])
    okw, gw = within_budget(W, ref["W"], ref["f64"]["W"])
    okh, gh = within_budget(H, ref["H"], ref["f64"]["H"])
    assert okw and okh, (gw, gh)


@pytest.mark.parametrize("k,T", [(1, 3), (3, 1), (2, 2)])
def test_small_rank_and_inner_counts_bit_exact(k, T):
    R, z = load_golden("mini")
    W0 = synth.initial_w(k, R.m, seed=5)
    ref = oracle.ccdpp(R, W0, k, 0.1, 3, T, history=True, residuals=True)
    with engine.Engine(R, k, 0.1, 3, T, reduce="sequential") as e:
        e.set_factors(W0)
        rm = e.run(3)
        st = e.state()
    assert np.array_equal(bits(st["W"]), bits(ref["W"])) and np.array_equal(bits(st["H"]), bits(ref["H"]))
    assert np.array_equal(bits(st["res_csc"]), bits(ref["res_csc"]))
    assert np.array_equal(bits(st["res_csr"]), bits(ref["res_csr"]))
    assert np.max(np.abs(rm - ref["rmse"])) <= 1e-12


def test_state_roundtrip_continues_identically():
    R, z = load_golden("mini")
    md = META["mini"]
    with engine.Engine(R, md["k"], md["lam"], md["maxiter"], md["maxinner"], reduce="sequential") as e:
        e.set_factors(z["W0"])
        e.run(2)
        st = e.state()            # flushes the pending subtract
        e.set_state(st["W"], st["H"], st["res_csc"], st["res_csr"], st["next_oiter"])
        e.run(2)
        W, H = e.factors()
    assert np.array_equal(bits(W), bits(z["W_hist"][3])) and np.array_equal(bits(H), bits(z["H_hist"][3]))


@pytest.mark.parametrize("version", [1, 3])
def test_split_lines_within_fp32_budget(version):
    # a matrix with very long columns exercises the split-line bin (lines
    # above cta_max = 16384 here, set explicitly)
    R = synth.generate(m=60000, n=40, nnz_total=900000, test_fraction=0.01, row_alpha=0.5, row_min=1, row_max=40,
                       col_alpha=0.3, col_cap=60000, rank=4, seed=21)
    W0 = synth.initial_w(4, R.m, seed=1)
    ref = oracle.ccdpp(R, W0, 4, 0.05, 2, 2, threads=8, history=True)
    r64 = oracle.ccdpp(R, W0.astype(np.float64), 4, 0.05, 2, 2, threads=8, dtype=np.float64, history=True)
    with engine.Engine(R, 4, 0.05, 2, 2, version=version) as e:
        e.set_bincfg(cta_max=16384)
        c, _ = e.bins("csc")
        assert c[4] > 0, c
        e.set_factors(W0)
        for j in range(2):
            rm = e.run(1)
            W, H = e.factors()
            okw, gw = within_budget(W, ref["W_hist"][j], r64["W_hist"][j])
            okh, gh = within_budget(H, ref["H_hist"][j], r64["H_hist"][j])
            assert okw and okh, (j, gw, gh)
            assert rmse_ok(rm[0], ref["rmse"][j], r64["rmse"][j]), (rm[0], ref["rmse"][j], r64["rmse"][j])
    with engine.Engine(R, 4, 0.05, 2, 2, reduce="sequential") as e:
        e.set_factors(W0)
        e.run(2)
        W, H = e.factors()
    assert np.array_equal(bits(W), bits(ref["W"])) and np.array_equal(bits(H), bits(ref["H"]))


@pytest.mark.parametrize("version", [1, 3])
@pytest.mark.parametrize("residual", ["bf16", "f16"])
def test_mixed_residual_rmse_vs_fp64_oracle(cpu_scale, residual, version):
    """16-bit residual storage with FP32 factors and accumulation and a
    per-outer-iteration FP32 refresh: test RMSE within 1e-3 of the FP64
    oracle after every outer iteration."""
    R, run, W0, ref = cpu_scale
    r64 = oracle.ccdpp(R, W0.astype(np.float64), run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"],
                       threads=8, dtype=np.float64)
    with engine.Engine(R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"], residual=residual,
                       version=version) as e:
        e.set_factors(W0)
        rm = e.run(run["maxiter"])
        st = e.stats()
        state = e.state()
    assert np.max(np.abs(rm - r64["rmse"])) <= 1e-3, (rm, r64["rmse"])
    assert st["refresh_launches"] == run["maxiter"] - 1 and st["nonfinite"] == 0
    assert 0.0 < st["drift_rms"] < 5e-2, st["drift_rms"]
    # both residual copies hold the same values (CSC order vs CSR order)
    from cdmf_gb300 import _lib
    import ctypes
    perm = np.empty(R.nnz, np.uint32)
    cp, ci = np.empty(R.n + 1, np.uint32), np.empty(R.nnz, np.uint32)
    U = ctypes.c_uint32
    _lib.load().cdmf_csr_to_csc(R.m, R.n, R.nnz, _lib.ptr(R.csr_ptr, U), _lib.ptr(R.csr_idx, U), None,
                                _lib.ptr(cp, U), _lib.ptr(ci, U), None, _lib.ptr(perm, U))
    assert np.array_equal(bits(state["res_csc"]), bits(state["res_csr"][perm]))


def test_mixed_refresh_restores_exact_residual(cpu_scale):
    """Right after a refresh the stored residual is R - W^T H rounded once to
    BF16 (checked against a float64 recomputation on the host)."""
    R, run, W0, ref = cpu_scale
    with engine.Engine(R, run["k"], run["lambda_"], 3, 1, residual="bf16") as e:
        e.set_factors(W0)
        e.run(2)
        e.set_profiling(False)
        st = e.state()
    W, H = st["W"].astype(np.float64), st["H"].astype(np.float64)
    rows, cols, vals = R.coo()
    exact = vals.astype(np.float64) - np.einsum("ti,ti->i", W[:, rows], H[:, cols])
    got = st["res_csr"].astype(np.float64)
    # after 2 outer iterations the residual went through one refresh and k
    # further BF16 updates: it stays within a few BF16 ulps of the exact one
    err = np.abs(got - exact)
    assert np.sqrt(np.mean(err ** 2)) < 2e-2 and np.max(err) < 0.25


@pytest.mark.parametrize("residual,graph", [("f32", False), ("bf16", True)])
def test_train_queued_matches_run(cpu_scale, residual, graph):
    """cdmf_cuda_train queues each outer iteration before it reads the
    previous one's RMSE: factors and RMSE are those of an engine run one
    outer iteration at a time, bit for bit, and the callback sees every
    iteration in order, with its RMSE and growing times."""
    R, run, W0, ref = cpu_scale
    n, k = run["maxiter"], run["k"]
    with engine.Engine(R, k, run["lambda_"], n, run["maxinneriter"], residual=residual, use_graph=graph) as e:
        e.set_factors(W0)
        rm1 = np.concatenate([e.run(1) for _ in range(n)])
        W1, H1 = e.factors()
    o = engine.make_opts(k, run["lambda_"], n, run["maxinneriter"], residual=residual, use_graph=graph)
    p = engine._problem(R)
    W2 = np.ascontiguousarray(W0, np.float32).copy()
    H2 = np.zeros((k, R.n), np.float32)
    rm2 = np.zeros(n)
    seen = []
    cb = _lib.OUTER_CB(lambda it, rmse, ms, user: seen.append((it, rmse, ms)))
    st = _lib.load().cdmf_cuda_train(ctypes.byref(p), ctypes.byref(o), _lib.ptr(W2, ctypes.c_float),
                                     _lib.ptr(H2, ctypes.c_float), _lib.ptr(rm2, ctypes.c_double), cb, None)
    assert st == 0
    assert np.array_equal(bits(W1), bits(W2)) and np.array_equal(bits(H1), bits(H2))
    assert np.array_equal(rm1, rm2)
    assert [s[0] for s in seen] == list(range(1, n + 1))
    assert np.array_equal(np.array([s[1] for s in seen]), rm2)
    ms = [s[2] for s in seen]
    assert ms[0] > 0 and all(a <= b for a, b in zip(ms, ms[1:]))


@pytest.mark.parametrize("graph", [False, True])
def test_train_stops_on_non_finite_refresh(cpu_scale, graph):
    """A rating beyond FP16's range (65,504) leaves a non-finite FP16
    residual: the refresh at the start of outer iteration 2 counts it, and
    cdmf_cuda_train stops with CDMF_ERR_NUMERIC after the callback of outer
    iteration 1, leaving the caller's factors untouched."""
    from cdmf_gb300 import formats
    R, run, W0, ref = cpu_scale
    rows, cols, vals = R.coo()
    vals = vals.copy()
    vals[0] = 1e6
    Rb = formats.from_coo(R.m, R.n, rows, cols, vals, R.te_row, R.te_col, R.te_val)
    k = run["k"]
    o = engine.make_opts(k, run["lambda_"], 4, 1, residual="f16", use_graph=graph)
    p = engine._problem(Rb)
    W = np.ascontiguousarray(W0, np.float32).copy()
    H = np.zeros((k, Rb.n), np.float32)
    seen = []
    cb = _lib.OUTER_CB(lambda it, rmse, ms, user: seen.append(it))
    st = _lib.load().cdmf_cuda_train(ctypes.byref(p), ctypes.byref(o), _lib.ptr(W, ctypes.c_float),
                                     _lib.ptr(H, ctypes.c_float), None, cb, None)
    assert st == -6, st   # CDMF_ERR_NUMERIC
    assert seen == [1]
    assert np.array_equal(bits(W), bits(np.ascontiguousarray(W0, np.float32)))


@pytest.mark.parametrize("version", [1, 3])
@pytest.mark.parametrize("residual", ["f32", "bf16"])
def test_graph_replay_identical(cpu_scale, residual, version):
    """Outer iterations replayed from CUDA graphs give bit-identical factors
    and RMSE to the eagerly launched schedule."""
    R, run, W0, ref = cpu_scale
    out = []
    for graph in (False, True):
        with engine.Engine(R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"], residual=residual,
                           use_graph=graph, version=version) as e:
            e.set_factors(W0)
            rm = e.run(run["maxiter"])
            W, H = e.factors()
            out.append((W, H, rm, e.stats()))
    (W0_, H0_, r0, s0), (W1, H1, r1, s1) = out
    assert np.array_equal(bits(W0_), bits(W1)) and np.array_equal(bits(H0_), bits(H1))
    assert np.array_equal(r0, r1)
    assert s0["launches"] == s1["launches"]


@pytest.mark.parametrize("k,T", [(1, 3), (3, 1)])
def test_tile_version_small_rank_within_budget(k, T):
    R, z = load_golden("mini")
    W0 = synth.initial_w(k, R.m, seed=5)
    ref = oracle.ccdpp(R, W0, k, 0.1, 3, T, history=True)
    r64 = oracle.ccdpp(R, W0.astype(np.float64), k, 0.1, 3, T, dtype=np.float64, history=True)
    with engine.Engine(R, k, 0.1, 3, T, version=3) as e:
        e.set_factors(W0)
        for j in range(3):
            rm = e.run(1)
            W, H = e.factors()
            okw, gw = within_budget(W, ref["W_hist"][j], r64["W_hist"][j])
            okh, gh = within_budget(H, ref["H_hist"][j], r64["H_hist"][j])
            assert okw and okh, (j, gw, gh)
            assert rmse_ok(rm[0], ref["rmse"][j], r64["rmse"][j])


def test_tile_version_deterministic():
    R, z = load_golden("mini")
    md = META["mini"]
    outs = []
    for _ in range(2):
        with engine.Engine(R, md["k"], md["lam"], md["maxiter"], md["maxinner"], version=3) as e:
            e.set_factors(z["W0"])
            e.run(md["maxiter"])
            outs.append(e.state())
    for f in ("W", "H", "res_csc", "res_csr"):
        assert np.array_equal(bits(outs[0][f]), bits(outs[1][f])), f


def test_autotune_and_bincfg(cpu_scale):
    """The autotuner picks valid thresholds, leaves a fresh state, and any
    bin plan keeps the results within the FP32 budget."""
    R, run, W0, ref = cpu_scale
    with engine.Engine(R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"]) as e:
        cfg, ms = e.autotune()
        assert ms > 0 and cfg["thread_max"] <= cfg["warp_max"] <= cfg["cta_max"]
        assert e.bincfg() == cfg
        for plan in (cfg, dict(group_max=0, warp_max=1024, cta_max=8192, chunk=4096)):
            e.set_bincfg(**plan)
            e.set_factors(W0)
            rm = e.run(run["maxiter"])
            W, H = e.factors()
            okw, gw = within_budget(W, ref["W"], ref["f64"]["W"])
            okh, gh = within_budget(H, ref["H"], ref["f64"]["H"])
            assert okw and okh, (plan, gw, gh)
            assert all(rmse_ok(a, b, c) for a, b, c in zip(rm, ref["rmse"], ref["f64"]["rmse"]))
    with pytest.raises(Exception):
        with engine.Engine(R, run["k"], run["lambda_"], 1, 1) as e:
            e.set_bincfg(warp_max=100, cta_max=50)


@pytest.mark.parametrize("opts", [dict(layout="blocked"), dict(version=3), dict(reduce="sequential")])
def test_autotune_leaves_unbinned_sweeps_alone(cpu_scale, opts):
    """Handles whose sweeps do not run on the length bins (blocked layout,
    tile kernel, reference order) get no search: the plan stays as created
    and no time is reported."""
    R, run, W0, ref = cpu_scale
    with engine.Engine(R, run["k"], run["lambda_"], 1, 1, **opts) as e:
        before = e.bincfg()
        cfg, ms = e.autotune()
        assert ms == 0 and cfg == before == e.bincfg()


def test_autotune_pick_reused_by_next_handle(cpu_scale):
    """A handle created with autotune on for a shape already tuned in this
    process is planned with the kept pick from the start: same bins, and
    results bit-identical to the handle before it."""
    R, run, W0, ref = cpu_scale
    outs = []
    for _ in range(2):
        with engine.Engine(R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"], autotune=True,
                           use_graph=True) as e:
            cfg = e.bincfg()
            e.set_factors(W0)
            rm = e.run(run["maxiter"])
            W, H = e.factors()
            outs.append((cfg, W, H, rm))
    (c0, W0_, H0_, r0), (c1, W1, H1, r1) = outs
    assert c0 == c1
    assert np.array_equal(bits(W0_), bits(W1)) and np.array_equal(bits(H0_), bits(H1)) and np.array_equal(r0, r1)


def test_bincfg_change_after_graph_runs(cpu_scale):
    """A new bin plan after outer iterations were captured as CUDA graphs
    drops those graphs: the next runs take the new plan, bit for bit as an
    engine created with it."""
    R, run, W0, ref = cpu_scale
    plan = dict(group_max=0, warp_max=1024, cta_max=8192, chunk=4096)
    args = (R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"])
    with engine.Engine(*args, use_graph=True) as e:
        e.set_factors(W0)
        e.run(2)
        e.set_bincfg(**plan)
        e.set_factors(W0)
        rm1 = e.run(2)
        W1, H1 = e.factors()
    with engine.Engine(*args, use_graph=True) as f:
        f.set_bincfg(**plan)
        f.set_factors(W0)
        rm2 = f.run(2)
        W2, H2 = f.factors()
    assert np.array_equal(rm1, rm2)
    assert np.array_equal(bits(W1), bits(W2)) and np.array_equal(bits(H1), bits(H2))


# ---- cross-index-blocked layout ---------------------------------------------

@pytest.mark.parametrize("name", ["mini", "simple", "tricky_simple"])
def test_blocked_within_fp32_budget_each_outer(name):
    R, z = load_golden(name)
    md = META[name]
    r64 = oracle.ccdpp(R, z["W0"].astype(np.float64), md["k"], md["lam"], md["maxiter"], md["maxinner"],
                       dtype=np.float64, history=True)
    with engine.Engine(R, md["k"], md["lam"], md["maxiter"], md["maxinner"], layout="blocked") as e:
        e.set_factors(z["W0"])
        for j in range(md["maxiter"]):
            rm = e.run(1)
            W, H = e.factors()
            okw, gw = within_budget(W, z["W_hist"][j], r64["W_hist"][j])
            okh, gh = within_budget(H, z["H_hist"][j], r64["H_hist"][j])
            assert okw and okh, (j, gw, gh)
            assert rmse_ok(rm[0], z["rmse"][j], r64["rmse"][j])


def test_blocked_cpu_scale_one_step_and_free(cpu_scale):
    R, run, W0, ref = cpu_scale
    k, lam, T = run["k"], run["lambda_"], run["maxinneriter"]
    with engine.Engine(R, k, lam, run["maxiter"], T, layout="blocked") as e:
        e.set_factors(W0)
        rm = e.run(run["maxiter"])
        W, H = e.factors()
        okw, gw = within_budget(W, ref["W"], ref["f64"]["W"])
        okh, gh = within_budget(H, ref["H"], ref["f64"]["H"])
        assert okw and okh, (gw, gh)
        assert all(rmse_ok(a, b, c) for a, b, c in zip(rm, ref["rmse"], ref["f64"]["rmse"]))
        # one step from the oracle's state after outer 2
        Wst, Hst = ref["W_hist"][1].copy(), ref["H_hist"][1].copy()
        r2 = oracle.ccdpp(R, W0, k, lam, 2, T, threads=8, residuals=True)
        e.set_state(Wst, Hst, r2["res_csc"], r2["res_csr"], 3)
        rm = e.run(1)
        Wg, Hg = e.factors()
        W64, H64 = Wst.astype(np.float64), Hst.astype(np.float64)
        rc64, rr64 = r2["res_csc"].astype(np.float64), r2["res_csr"].astype(np.float64)
        oracle.outer_iteration(R, W64, H64, rc64, rr64, k, lam, T, 3, threads=8)
        okw, gw = within_budget(Wg, ref["W_hist"][2], W64)
        okh, gh = within_budget(Hg, ref["H_hist"][2], H64)
        assert okw and okh, (gw, gh)


@pytest.mark.parametrize("residual", ["bf16", "f16"])
def test_blocked_mixed_residual(cpu_scale, residual):
    R, run, W0, ref = cpu_scale
    r64 = ref["f64"]
    with engine.Engine(R, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"], residual=residual,
                       layout="blocked", use_graph=True) as e:
        e.set_factors(W0)
        rm = e.run(run["maxiter"])
        st = e.stats()
        state = e.state()
    assert np.max(np.abs(rm - r64["rmse"])) <= 1e-3, (rm, r64["rmse"])
    assert st["nonfinite"] == 0 and 0.0 < st["drift_rms"] < 5e-2
    rows, cols, vals = R.coo()
    exact = vals.astype(np.float64) - np.einsum("ti,ti->i", state["W"][:, rows].astype(np.float64),
                                                state["H"][:, cols].astype(np.float64))
    assert np.sqrt(np.mean((state["res_csr"] - exact) ** 2)) < 5e-2


def test_blocked_deterministic_and_state_roundtrip(cpu_scale):
    R, run, W0, ref = cpu_scale
    outs = []
    for split in (False, True):
        with engine.Engine(R, run["k"], run["lambda_"], 4, 1, layout="blocked") as e:
            e.set_factors(W0)
            if split:
                e.run(2)
                st = e.state()
                e.set_state(st["W"], st["H"], st["res_csc"], st["res_csr"], st["next_oiter"])
                e.run(2)
            else:
                e.run(4)
            outs.append(e.state())
    for f in ("W", "H", "res_csc", "res_csr"):
        assert np.array_equal(bits(outs[0][f]), bits(outs[1][f])), f


@pytest.mark.parametrize("residual", ["f32", "bf16"])
def test_device_relabel_matches_host_relabel(cpu_scale, residual):
    """The degree relabelling built on the GPU at create gives the same engine
    as the host build: identical factors, residual state and RMSE, bit for bit."""
    R, run, W0, ref = cpu_scale
    out = []
    for where in (True, "host"):
        with engine.Engine(R, run["k"], run["lambda_"], 3, 1, residual=residual, relabel=where) as e:
            e.set_factors(W0)
            rm = e.run(2)
            st = e.state()
            out.append((rm, st))
    (rm1, s1), (rm2, s2) = out
    assert np.array_equal(rm1, rm2)
    for key in ("W", "H", "res_csc", "res_csr"):
        assert np.array_equal(bits(s1[key]), bits(s2[key])), key


@pytest.mark.parametrize("residual", ["f32"])
def test_shared_memory_cross_table_matches_global(cpu_scale, residual, monkeypatch):
    """Narrow matrices stage the CSR sweep's cross table in shared memory; the
    result must equal the L1/L2 gather path bit for bit (CDMF_NO_SMEMQ turns
    the staging off at create)."""
    R, run, W0, ref = cpu_scale
    out = []
    for off in (False, True):
        if off:
            monkeypatch.setenv("CDMF_NO_SMEMQ", "1")
        with engine.Engine(R, run["k"], run["lambda_"], 3, 1, residual=residual) as e:
            e.set_factors(W0)
            rm = e.run(3)
            out.append((rm, e.state()))
    (rm1, s1), (rm2, s2) = out
    assert np.array_equal(rm1, rm2)
    for key in ("W", "H", "res_csc", "res_csr"):
        assert np.array_equal(bits(s1[key]), bits(s2[key])), key


@pytest.mark.parametrize("residual", ["f32", "bf16"])
def test_sixteen_bit_column_indices_match(cpu_scale, residual, monkeypatch):
    """Matrices with at most 65,536 columns stream 16-bit column indices in
    the CSR sweeps; the result must equal the 32-bit path bit for bit
    (CDMF_NO_IDX16 turns the narrow copy off at create)."""
    R, run, W0, ref = cpu_scale
    assert R.n <= 65536
    out = []
    for off in (False, True):
        if off:
            monkeypatch.setenv("CDMF_NO_IDX16", "1")
        with engine.Engine(R, run["k"], run["lambda_"], 3, 1, residual=residual) as e:
            e.set_factors(W0)
            rm = e.run(3)
            out.append((rm, e.state()))
    (rm1, s1), (rm2, s2) = out
    assert np.array_equal(rm1, rm2)
    for key in ("W", "H", "res_csc", "res_csr"):
        assert np.array_equal(bits(s1[key]), bits(s2[key])), key


@pytest.fixture(scope="module")
def large_tall():
    """17.5M nonzeros over 300,000 rows: above the 16M-nonzero threshold of the
    pipelined CSC sweep, with rows in five segments of 65,536."""
    return synth.generate(m=300_000, n=4_000, nnz_total=17_500_000, test_fraction=0.01, row_alpha=0.9,
                          row_max=2_000, col_alpha=0.9, col_cap=60_000, rank=6, seed=5)


@pytest.mark.parametrize("residual", ["f32", "bf16"])
def test_sixteen_bit_row_offsets_match(large_tall, residual, monkeypatch):
    """From 16M nonzeros, FP32 runs on matrices with at most 8 * 65,536 rows
    stream the CSC row indices of the first CSC sweep as 16-bit offsets inside
    65,536-row segments (each column's segment ends in a small table); the
    result must equal the 32-bit path bit for bit (CDMF_NO_IDX16 turns both
    narrow copies off at create).  BF16 runs keep 32-bit row indices: the
    comparison then covers the 16-bit column indices alone."""
    R = large_tall
    assert R.nnz >= 16 << 20 and 65536 < R.m <= 8 << 16
    k = 8
    W0 = synth.initial_w(k, R.m, seed=0)
    out = []
    for off in (False, True):
        if off:
            monkeypatch.setenv("CDMF_NO_IDX16", "1")
        with engine.Engine(R, k, 0.05, 2, 1, residual=residual) as e:
            e.set_factors(W0)
            rm = e.run(2)
            out.append((rm, e.state()))
    (rm1, s1), (rm2, s2) = out
    assert np.array_equal(rm1, rm2)
    for key in ("W", "H", "res_csc", "res_csr"):
        assert np.array_equal(bits(s1[key]), bits(s2[key])), key
