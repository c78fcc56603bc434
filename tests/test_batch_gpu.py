"""Batched factorisations (cdmf_cuda_batch_*): grouped persistent sweeps give
bit-identical results to running each problem through its own handle."""
import numpy as np
import pytest

from cdmf_gb300 import engine, synth

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def small_batch(count=6, seed=4):
    probs, runs = [], []
    rng = np.random.default_rng(seed)
    for q in range(count):
        m = int(rng.integers(800, 6000))
        n = int(rng.integers(300, 1500))
        nnz = int(min(0.2 * m * n, rng.integers(20000, 120000)))
        R = synth.generate(m=m, n=n, nnz_total=nnz, test_fraction=0.02, row_alpha=0.9, row_max=max(1, n // 2),
                           col_alpha=0.9, col_cap=max(1, m // 2), rank=6, seed=100 + q)
        probs.append(R)
        runs.append(dict(k=int(rng.choice([2, 4, 8])), lambda_=float(rng.choice([0.01, 0.05, 0.1, 0.5]))))
    return probs, runs


@pytest.mark.parametrize("residual", ["f32", "bf16"])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_individual_runs(residual, graph):
    probs, runs = small_batch()
    W0s = [synth.initial_w(r["k"], R.m, seed=q) for q, (R, r) in enumerate(zip(probs, runs))]
    with engine.Batch(probs, runs, maxiter=3, maxinneriter=1, residual=residual, use_graph=graph) as b:
        b.set_factors(W0s)
        rm = b.run(3)
        Ws, Hs = b.factors()
        st = b.stats()
    assert st["updates"] == 3 * sum(r["k"] for r in runs)
    for q, (R, r) in enumerate(zip(probs, runs)):
        with engine.Engine(R, r["k"], r["lambda_"], 3, 1, residual=residual, version=1) as e:
            e.set_factors(W0s[q])
            rq = e.run(3)
            W, H = e.factors()
        assert np.array_equal(bits(W), bits(Ws[q])) and np.array_equal(bits(H), bits(Hs[q])), q
        assert np.array_equal(rq, rm[q]), (q, rq, rm[q])


def test_batch_replay_and_sequential_agree():
    probs, runs = small_batch(count=5, seed=9)
    W0s = [synth.initial_w(r["k"], R.m, seed=q) for q, (R, r) in enumerate(zip(probs, runs))]
    with engine.Batch(probs, runs, maxiter=4, maxinneriter=2, use_graph=True) as b:
        outs = []
        for _ in range(2):                       # second run replays the captured graph
            b.set_factors(W0s)
            outs.append((b.run(4), b.factors()))
        b.set_factors(W0s)
        rs, ms = b.run_sequential(4)
        Ws, Hs = b.factors()
    (r0, (W0, H0)), (r1, (W1, H1)) = outs
    assert np.array_equal(r0, r1) and np.array_equal(r0, rs)
    for q in range(len(probs)):
        assert np.array_equal(bits(W0[q]), bits(W1[q])) and np.array_equal(bits(W0[q]), bits(Ws[q]))
        assert np.array_equal(bits(H0[q]), bits(H1[q])) and np.array_equal(bits(H0[q]), bits(Hs[q]))
    assert ms > 0
