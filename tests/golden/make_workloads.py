"""Generates tests/golden/workloads.json: the oracle's test-RMSE trajectories
(FP32 = the reference's arithmetic, FP64 = the same algorithm in double) on
the synthetic stand-ins for the reference's benchmark data sets, with
checksums of the generated matrix and initial factors so a test knows the
matrix it regenerates is the one the trajectories belong to.

Workloads (cdmf_gb300.synth presets, W0 = synth.initial_w(k, m, seed=0), H = 0):
  jester_shape   73,421 x 100, 4.2M nonzeros, k=10, lambda=0.5, 15 x 2
  ml20m_shape    138,493 x 26,744, 19.6M nonzeros, k=128, lambda=0.1, 10 x 3
  netflix_shape  480,189 x 17,770, 99.1M nonzeros, k=64, lambda=0.05, 20 x 1
  netflix_shape_k32  the same matrix at k=32
The oracle restatement is pinned bit for bit to the reference's own engine
by make_golden.py on small cases and by `--pin` below on these workloads;
the trajectories are too slow to recompute inside a GPU test (netflix_shape
takes minutes of CPU per precision).

Where the reference's sources are (oracle/_ref built by oracle/build_ref.sh),
`--pin` runs the reference's own engine on a workload already in the file and
checks the oracle against it bit for bit (final W and H, last RMSE) before
marking the entry "reference_pinned".

`--model` adds the trajectories of the CPU model of the engine's 16-bit
residual mode (oracle/mixed_model.c) for BF16 and FP16 storage, on the
engine's refresh schedule (every outer iteration after the first, and every
EARLY_REFRESH features while no refresh has run).

`--batch` writes tests/golden/batch64.json: for each of the 64 uneven
problems of the batched workload (synth.batch_specs, W0 seeded by problem
index), the input checksums and the test-RMSE trajectories of the FP32 and
FP64 oracles and of the 16-bit model in BF16 and FP16.

Usage: python tests/golden/make_workloads.py [workload ...]          (merges into the file)
       python tests/golden/make_workloads.py --pin [workload ...]    (pins existing entries)
       python tests/golden/make_workloads.py --model [workload ...]  (adds the 16-bit model)
       python tests/golden/make_workloads.py --batch                 (the 64-problem batch)
"""
import json
import os
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from cdmf_gb300 import formats, synth  # noqa: E402
from oracle import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "workloads.json")
BATCH_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "batch64.json")
DEFAULT = ("jester_shape", "ml20m_shape", "netflix_shape", "netflix_shape_k32")
# Fixture name -> (generator preset, run-parameter overrides).
VARIANTS = {"netflix_shape_k32": ("netflix_shape", {"k": 32})}
# The engine's 16-bit modes refresh the residual every EARLY_REFRESH features
# until the first per-outer-iteration refresh has run.
EARLY_REFRESH = 32


def load(name):
    """(matrix, run parameters) of a fixture name."""
    preset, over = VARIANTS.get(name, (name, {}))
    R, run = synth.config(preset)
    run.update(over)
    return R, run


def bit_sum(a):
    """Sum of the 32-bit patterns: exact and independent of summation order."""
    return int(np.ascontiguousarray(a).view(np.uint32).astype(np.int64).sum())


def checksums(R, W0):
    """Sizes and bit-pattern sums that identify the generated inputs."""
    return dict(m=int(R.m), n=int(R.n), nnz=int(R.nnz), nnz_test=int(R.te_val.size),
                csr_idx_sum=bit_sum(R.csr_idx), csr_val_sum=bit_sum(R.csr_val), te_row_sum=bit_sum(R.te_row),
                te_val_sum=bit_sum(R.te_val), w0_sum=bit_sum(W0))


def make(name):
    R, run = load(name)
    k, lam, T, it = run["k"], run["lambda_"], run["maxinneriter"], run["maxiter"]
    W0 = synth.initial_w(k, R.m, seed=0)
    out = dict(k=k, lam=lam, maxiter=it, maxinner=T, inputs=checksums(R, W0))
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        t0 = time.time()
        r = oracle.ccdpp(R, W0.astype(dt), k, lam, it, T, dtype=dt)
        out["rmse_" + tag] = [float(x) for x in r["rmse"]]
        print(f"{name} {tag}: {time.time() - t0:.1f} s, final RMSE {r['rmse'][-1]:.9f}", flush=True)
    return out


def pin(name, entry):
    """The reference's cdmf_ref on the workload against the oracle, bit for bit."""
    if not oracle.reference_available():
        raise SystemExit("oracle/_ref is not built (oracle/build_ref.sh needs the reference sources)")
    R, run = load(name)
    k, lam, T, it = entry["k"], entry["lam"], entry["maxinner"], entry["maxiter"]
    W0 = synth.initial_w(k, R.m, seed=0)
    if checksums(R, W0) != entry["inputs"]:
        raise SystemExit(f"{name}: the generator no longer makes the recorded inputs")
    t0 = time.time()
    with tempfile.TemporaryDirectory(dir=os.path.dirname(OUT)) as tmp:
        formats.write_dir(tmp, R)
        ref = oracle.reference_run(tmp, W0, k, lam, it, T, threads=os.cpu_count() or 1)
    o = oracle.ccdpp(R, W0, k, lam, it, T)
    same = (np.array_equal(o["W"].view(np.uint32), ref["W"].view(np.uint32))
            and np.array_equal(o["H"].view(np.uint32), ref["H"].view(np.uint32))
            and ref["rmse"] == o["rmse"][-1] == entry["rmse_f32"][-1])
    if not same:
        raise SystemExit(f"{name}: the oracle differs from the reference; nothing written")
    print(f"{name}: oracle == reference bit for bit ({time.time() - t0:.0f} s)", flush=True)
    entry["reference_pinned"] = True


def main(names):
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for name in names:
        data[name] = make(name)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


def model(name, entry):
    """The 16-bit model's trajectories (oracle/mixed_model.c, the engine's
    refresh schedule) for BF16 and FP16 storage."""
    R, _ = load(name)
    W0 = synth.initial_w(entry["k"], R.m, seed=0)
    if checksums(R, W0) != entry["inputs"]:
        raise SystemExit(f"{name}: the generator no longer makes the recorded inputs")
    for storage in ("bf16", "f16"):
        t0 = time.time()
        out = oracle.mixed_model(R, W0, entry["k"], entry["lam"], entry["maxiter"], entry["maxinner"],
                                 storage=storage, refresh_every=EARLY_REFRESH)
        entry["model_" + storage] = [float(x) for x in out["rmse"]]
        print(f"{name} model {storage}: {time.time() - t0:.0f} s", flush=True)
    entry["model_early_refresh"] = EARLY_REFRESH


def main_model(names):
    data = json.load(open(OUT))
    for name in names:
        model(name, data[name])
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


def main_pin(names):
    data = json.load(open(OUT))
    for name in names:
        pin(name, data[name])
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


def main_batch(count=64):
    """The 64-problem batch: FP32 / FP64 oracle and 16-bit model trajectories."""
    specs = synth.batch_specs(count, seed=0)
    out = {"count": count, "seed": 0, "model_early_refresh": EARLY_REFRESH, "problems": []}
    t0 = time.time()
    for q, sp in enumerate(specs):
        R = synth.generate(**sp["matrix"])
        run = sp["run"]
        k, lam, it, T = run["k"], run["lambda_"], run["maxiter"], run["maxinneriter"]
        W0 = synth.initial_w(k, R.m, seed=q)
        e = dict(k=k, lam=lam, maxiter=it, maxinner=T, inputs=checksums(R, W0))
        for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
            e["rmse_" + tag] = [float(x) for x in oracle.ccdpp(R, W0.astype(dt), k, lam, it, T, dtype=dt)["rmse"]]
        for storage in ("bf16", "f16"):
            r = oracle.mixed_model(R, W0, k, lam, it, T, storage=storage, refresh_every=EARLY_REFRESH)["rmse"]
            e["model_" + storage] = [float(x) for x in r]
        out["problems"].append(e)
        print(f"batch64 problem {q}: {time.time() - t0:.0f} s", flush=True)
    with open(BATCH_OUT, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    if sys.argv[1:2] == ["--pin"]:
        main_pin(sys.argv[2:] or ("jester_shape", "ml20m_shape"))
    elif sys.argv[1:2] == ["--batch"]:
        main_batch()
    elif sys.argv[1:2] == ["--model"]:
        main_model(sys.argv[2:] or ("jester_shape", "ml20m_shape"))
    else:
        main(sys.argv[1:] or DEFAULT)
