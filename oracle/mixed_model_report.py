"""Error of the engine's 16-bit residual mode, modelled on the CPU
(oracle/mixed_model.c), against the FP64 oracle trajectory of a
benchmark-shaped workload (tests/golden/workloads.json).  Test and analysis
infrastructure only.

Usage: python oracle/mixed_model_report.py WORKLOAD STORAGE:REFRESH_EVERY[:all] ...
e.g.   python oracle/mixed_model_report.py ml20m_shape bf16:0 bf16:32 f16:0 f32:0
(":all" keeps the extra refreshes in every outer iteration, not only the first)
prints, per variant, |RMSE - FP64 RMSE| in the first outer iteration and the
largest over the later ones (and the distance to the FP32 oracle, which is 0
for f32 storage: the model is then the reference's arithmetic), then
RMSE - FP64 RMSE after every outer iteration.

WORKLOAD batch64 runs the 64 uneven problems of the batched benchmark
(synth.batch_specs, W0 seeded by problem), the FP64 oracle computed on the
spot, and prints per variant the problems furthest from FP64.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from cdmf_gb300 import synth  # noqa: E402
from oracle import oracle  # noqa: E402


def main(name, variants):
    g = json.load(open(os.path.join(os.path.dirname(HERE), "tests", "golden", "workloads.json")))[name]
    R, _ = synth.config(name)
    W0 = synth.initial_w(g["k"], R.m, seed=0)
    r32, r64 = np.array(g["rmse_f32"]), np.array(g["rmse_f64"])
    for v in variants:
        storage, every, *scope = v.split(":")
        t0 = time.time()
        out = oracle.mixed_model(R, W0, g["k"], g["lam"], g["maxiter"], g["maxinner"], storage=storage,
                                 refresh_every=int(every), refresh_all=scope == ["all"])
        d = out["rmse"] - r64
        later = np.abs(d[1:]).max() if d.size > 1 else 0.0
        print(f"{name} {storage} refresh_every={every}: iteration 1 {d[0]:+.2e}, later max {later:.2e}, "
              f"max vs FP32 oracle {np.abs(out['rmse'] - r32).max():.2e} ({time.time() - t0:.0f} s)", flush=True)
        print("  per outer iteration: " + " ".join(f"{x:+.1e}" for x in d), flush=True)


def main_batch(variants, count=64):
    specs = synth.batch_specs(count, seed=0)
    probs = []
    for q, sp in enumerate(specs):
        R = synth.generate(**sp["matrix"])
        run = sp["run"]
        W0 = synth.initial_w(run["k"], R.m, seed=q)
        r64 = oracle.ccdpp(R, W0.astype(np.float64), run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"],
                           dtype=np.float64)["rmse"]
        probs.append((R, run, W0, r64))
    for v in variants:
        storage, every, *scope = v.split(":")
        worst = []
        for q, (R, run, W0, r64) in enumerate(probs):
            out = oracle.mixed_model(R, W0, run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"],
                                     storage=storage, refresh_every=int(every), refresh_all=scope == ["all"])
            d = np.abs(out["rmse"] - r64)
            worst.append((float(d.max()), int(d.argmax()) + 1, q, run["k"], run["lambda_"], int(R.nnz)))
        worst.sort(reverse=True)
        over = sum(1 for w in worst if w[0] > 1e-3)
        print(f"batch64 {storage} refresh_every={every}: {over} of {len(worst)} problems beyond 1e-3 of FP64; "
              f"largest {worst[0][0]:.2e}", flush=True)
        for w in worst[:5]:
            print(f"  {w[0]:.2e} at outer iteration {w[1]}: problem {w[2]}, k={w[3]}, lambda={w[4]}, nnz={w[5]}")


if __name__ == "__main__":
    if sys.argv[1] == "batch64":
        main_batch(sys.argv[2:])
    else:
        main(sys.argv[1], sys.argv[2:])
