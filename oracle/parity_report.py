"""Distance of the engine's production summation order from the reference's
arithmetic, per benchmark-shaped workload -- test and analysis infrastructure.

For each workload (cdmf_gb300.synth presets, W0 = synth.initial_w(k, m,
seed=0), H = 0, the workload's k, lambda and outer x inner) it runs the
oracle in FP32 (the reference's arithmetic, src/cdmf_ref.cpp:47-140) and in
FP64 on the host cores, and the GB300 engine with an FP32 residual in both
reduction orders, and prints after the last outer iteration:
  - the relative Frobenius distance of W and of H: tree order vs the FP32
    oracle, the FP32 oracle vs the FP64 oracle, tree order vs FP64;
  - the largest elementwise relative difference, tree order vs FP32 oracle
    (over entries of magnitude above 1e-6);
  - the same for the reference order (reduce=sequential), which is 0 where
    the engine is bit-exact;
  - |RMSE - RMSE32|.
Needs a CUDA device.  The Netflix-shaped workloads take minutes of host time.

Usage: python oracle/parity_report.py [workload ...]
       workloads: cpu_scale jester_shape ml20m_shape netflix_shape netflix_shape_k32
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from cdmf_gb300 import engine, synth  # noqa: E402
from oracle import oracle  # noqa: E402

VARIANTS = {"netflix_shape_k32": ("netflix_shape", {"k": 32})}
SEQUENTIAL_MAX_NNZ = 25_000_000   # one thread per line: slow on the largest matrices


def fro(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def elem(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    big = np.abs(b) > 1e-6
    return float((np.abs(a - b)[big] / np.abs(b)[big]).max()) if np.any(big) else 0.0


def report(name):
    preset, over = VARIANTS.get(name, (name, {}))
    R, run = synth.config(preset)
    run.update(over)
    k, lam, it, T = run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"]
    W0 = synth.initial_w(k, R.m, seed=0)
    t0 = time.time()
    r32 = oracle.ccdpp(R, W0, k, lam, it, T)
    r64 = oracle.ccdpp(R, W0.astype(np.float64), k, lam, it, T, dtype=np.float64)
    host_s = time.time() - t0
    rows = []
    orders = ["tree"] + (["sequential"] if R.nnz <= SEQUENTIAL_MAX_NNZ else [])
    for reduce in orders:
        with engine.Engine(R, k, lam, it, T, residual="f32", reduce=reduce) as e:
            e.set_factors(W0)
            rm = e.run(it)
            W, H = e.factors()
        rows.append((reduce, fro(W, r32["W"]), fro(H, r32["H"]), elem(W, r32["W"]), fro(W, r64["W"]),
                     fro(H, r64["H"]), abs(float(rm[-1]) - float(r32["rmse"][-1]))))
    print(f"{name}: {R.m} x {R.n}, {R.nnz} nonzeros, k={k}, lambda={lam}, {it} x {T} "
          f"(oracle {host_s:.0f} s on the host)")
    print(f"  FP32 oracle vs FP64 oracle: W {fro(r32['W'], r64['W']):.2e}  H {fro(r32['H'], r64['H']):.2e}  "
          f"W elementwise {elem(r32['W'], r64['W']):.2e}")
    for reduce, fw, fh, ew, fw64, fh64, drm in rows:
        print(f"  {reduce:10s} vs FP32 oracle: W {fw:.2e}  H {fh:.2e}  W elementwise {ew:.2e}  |dRMSE| {drm:.1e};"
              f"  vs FP64: W {fw64:.2e}  H {fh64:.2e}", flush=True)


if __name__ == "__main__":
    for name in sys.argv[1:] or ("cpu_scale", "jester_shape", "ml20m_shape", "netflix_shape", "netflix_shape_k32"):
        report(name)
