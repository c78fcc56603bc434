"""The benchmark's full workload (480,189 x 17,770, 99M training nonzeros,
k = 64, T = 1) through the engine, checked by size-independent properties:
the FP64 objective never rises between outer iterations, the two residual
copies hold the same values (same sum of squares), and the 16-bit residual
mode stays within 1e-3 RMSE of the FP32 mode.  The oracle is too slow at this
size; the small cases pin the arithmetic itself."""
import numpy as np
import pytest

from cdmf_gb300 import engine, synth

pytestmark = pytest.mark.gpu
DESCENT_RTOL = 1e-6
MIXED_RMSE_ATOL = 1e-3


@pytest.fixture(scope="module")
def netflix():
    R, run = synth.config("netflix_shape")
    W0 = synth.initial_w(run["k"], R.m, seed=0)
    return R, run, W0


def _run(R, run, W0, residual, outer=3):
    objs, rms = [], []
    with engine.Engine(R, run["k"], run["lambda_"], outer, run["maxinneriter"], residual=residual,
                       use_graph=True) as e:
        e.set_factors(W0)
        objs.append(e.objective())
        for _ in range(outer):
            rms.append(float(e.run(1)[0]))
            objs.append(e.objective())
        st = e.state()
    return objs, rms, st


def test_full_size_descent_copies_and_mixed_precision(netflix):
    R, run, W0 = netflix
    out = {res: _run(R, run, W0, res) for res in ("f32", "bf16")}
    for res, (objs, rms, st) in out.items():
        tot = [o[2] for o in objs]
        for a, b in zip(tot, tot[1:]):
            assert b <= a * (1 + DESCENT_RTOL), (res, tot)
        # both copies: the same values in two orders
        sq_csc = float(np.dot(st["res_csc"].astype(np.float64), st["res_csc"].astype(np.float64)))
        sq_csr = float(np.dot(st["res_csr"].astype(np.float64), st["res_csr"].astype(np.float64)))
        assert abs(sq_csc - sq_csr) <= 1e-9 * sq_csr, (res, sq_csc, sq_csr)
        # the monitor reads the same residual
        assert abs(objs[-1][0] - sq_csr) <= 1e-9 * sq_csr, (res, objs[-1][0], sq_csr)
        assert all(np.isfinite(rms))
    r32, r16 = out["f32"][1], out["bf16"][1]
    assert max(abs(a - b) for a, b in zip(r32, r16)) <= MIXED_RMSE_ATOL, (r32, r16)
