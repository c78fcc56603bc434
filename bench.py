"""Benchmark: CCD++ rank-one updates/s on the 480,189 x 17,770 / 99.07M-train-nnz
synthetic (Netflix-shaped), k=64, lambda=0.05, 1 inner iteration.

One step = one outer iteration = 64 rank-one updates (each: add-back, one CSC
and one CSR sweep, subtract) + the fused test RMSE, with the matrix resident
in HBM.  The residual copies (1.6 GB at FP32) are far larger than L2, so no
L2 flush is needed between steps.

Printed as one JSON line (rank 0):
  value  -- updates/s, device-resident, CUDA events on the engine stream
  e2e    -- updates/s through cdmf_cuda_train (the reference's engine call)
            from page-locked host buffers: upload of R, 20 outer iterations
            with a per-iteration RMSE read-back, download of W and H
            (median of 3 calls; the SM clocks over the calls and the
            engine's phase times of each call beside it)
  roofline -- the sweep kernel: compulsory bytes per launch / mean launch time
  cpu_baseline -- the oracle CPU port of the reference engine on the host cores
  k32    -- the same matrix at rank 32, the workload's other rank (updates/s,
            BF16 and the FP32 comparison)
  batch64 -- the 64 uneven problems in one batched run against the same
            problems run one after another (--no-batch leaves it out)

--impl reference: the reference's CPU engine (oracle port; the reference
sources are not on the GPU host) on the same workload and config, all host
threads: W outer iterations untimed, then K timed ones, each k rank-one
updates and the test RMSE, as the GPU arm's steps.  It loads the oracle
libraries only (the matrix comes from the generator built into
oracle/libsynth.so).

Multi-GPU: `torchrun --nproc-per-node N bench.py --gpus N` runs one
independent replica per GPU (weak scaling, no collective in the data path);
rank 0 prints updates/s summed over ranks, timed as the max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "CCD++ rank-one updates/s & HBM GB/s at matched test RMSE, mixed vs FP32"
UNIT = "rank-one updates/s"
WORKLOAD = "netflix_shape"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, ws, rank):
        self.ws, self.rank = ws, rank
        self.pg = None
        if ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=rank, world_size=ws)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # raw samples: CDMF_CLOCKS_DIR when set (to keep them), else the temp directory
        folder = os.environ.get("CDMF_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(folder, f"cdmf_clocks_{os.getpid()}_{device}.csv")

    def __enter__(self):
        self.f = None
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            # nvidia-smi's start-up (NVML initialisation) makes driver calls of
            # its own; let it finish before the timed work starts
            time.sleep(1.0)
        except Exception:
            self.proc = None
            if self.f:
                self.f.close()
                os.remove(self.path)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per sweep launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "sweep_kernel_netflix_bf16.md")
    if not os.path.exists(path):
        return None
    out = {}
    for line in open(path):
        for key in ("workload", "residual", "traffic_bytes_per_launch"):
            if line.startswith(key + ":"):
                out[key] = line.split(":", 1)[1].strip()
    if "traffic_bytes_per_launch" not in out:
        return None
    return {"workload": out.get("workload"), "residual": out.get("residual"),
            "dram_bytes_per_launch": int(out["traffic_bytes_per_launch"])}


def cpu_outer_iterations(R, run, W0, threads, n_warm, n_timed=None, budget_s=None):
    """The oracle port of the reference's engine (src/cdmf_ref.cpp:69-137) on
    the host cores, with OpenMP over `threads`: whole outer iterations (k
    rank-one updates, then the test RMSE of src/tools.cpp:543-582) from W0,
    H = 0.  n_warm iterations untimed, then n_timed timed ones (or, with
    budget_s, timed ones until that many seconds are spent, at least one).
    Returns (seconds per timed iteration, test RMSE after each)."""
    from oracle import oracle
    k, lam, T = run["k"], run["lambda_"], run["maxinneriter"]
    W = np.ascontiguousarray(W0, np.float32).copy()
    H = np.zeros((k, R.n), np.float32)
    rc, rr = R.csc_val.copy(), R.csr_val.copy()
    oiter = 1
    for _ in range(n_warm):
        oracle.outer_iteration(R, W, H, rc, rr, k, lam, T, oiter, threads=threads)
        oracle.rmse(R, W, H, k)
        oiter += 1
    secs, rms = [], []
    while (n_timed is not None and len(secs) < n_timed) or (
            n_timed is None and (not secs or sum(secs) < budget_s)):
        t0 = time.perf_counter()
        oracle.outer_iteration(R, W, H, rc, rr, k, lam, T, oiter, threads=threads)
        rms.append(oracle.rmse(R, W, H, k))
        secs.append(time.perf_counter() - t0)
        oiter += 1
    return secs, rms


def workload_config(R, run, ws):
    """The `config` of both arms: the same workload, step and L2 policy."""
    return {"workload": f"{WORKLOAD} {R.m}x{R.n} train_nnz={R.nnz} test_nnz={R.nnz_test} k={run['k']} "
                        f"lambda={run['lambda_']} T={run['maxinneriter']}",
            "step": "one outer iteration (k rank-one updates + test RMSE)",
            "l2": "no flush: the residual copies streamed every feature exceed L2",
            "parallelism": f"replicas x{ws}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="cuda", choices=["cuda", "reference"])
    ap.add_argument("--residual", default="bf16", choices=["f32", "bf16", "f16"],
                    help="residual storage of the headline run (mixed precision: bf16)")
    ap.add_argument("--compare", default="f32", choices=["f32", "bf16", "f16", "none"],
                    help="residual storage of the comparison run reported beside the headline")
    ap.add_argument("--k", type=int, default=64)
    ap.add_argument("--version", type=int, default=1, choices=[1, 2, 3],
                    help="1/2: row-length-binned sweeps, 3: nonzero-balanced tiles")
    ap.add_argument("--graph", type=int, default=1, help="replay outer iterations from CUDA graphs")
    ap.add_argument("--relabel", type=int, default=1, help="renumber rows and columns by degree inside the engine")
    ap.add_argument("--autotune", type=int, default=1,
                    help="pick the bin thresholds by timing at create (the single-problem runs)")
    ap.add_argument("--batch-autotune", type=int, default=0,
                    help="the same for every problem of the 64-problem batch (off: limits tuned for a problem "
                         "alone slow the batched run)")
    ap.add_argument("--layout", default="lines", choices=["lines", "blocked"],
                    help="residual copy layout: lines (binned sweeps) or blocked (shared-memory gather tables)")
    ap.add_argument("--e2e-outer", type=int, default=20)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="device-resident timing only (no e2e, no CPU leg)")
    ap.add_argument("--workload", default=WORKLOAD, choices=[WORKLOAD, "batch64"],
                    help="batch64: 64 uneven problems in one batched run vs per-problem runs")
    ap.add_argument("--batch-residual", default="f16", choices=["f32", "bf16", "f16"],
                    help="residual storage of the 64-problem batch (FP16: within 1e-3 of FP64 on all 64)")
    ap.add_argument("--no-batch", action="store_true", help="leave the 64-problem batch out of the headline run")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    args.warmup = max(3, args.warmup)

    from cdmf_gb300 import synth
    threads = os.cpu_count() or 1
    if args.workload == "batch64" and args.impl == "cuda":
        if rank != 0:   # one batch on one GPU; other ranks have nothing to add
            return
        return bench_batch(args, threads)

    if args.impl == "reference":
        if rank != 0:
            return
        # the oracle libraries only: the generator built into oracle/libsynth.so
        # makes the same matrix as the engine library's copy
        from oracle import oracle
        R, run = synth.config(WORKLOAD, threads=threads, lib=oracle.synth_lib())
        run["k"] = args.k
        W0 = synth.initial_w(run["k"], R.m, seed=0)
        secs, rms = cpu_outer_iterations(R, run, W0, threads, n_warm=args.warmup, n_timed=args.steps)
        value = run["k"] * len(secs) / sum(secs)
        line = {
            "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded, Netflix-shaped; the data set itself is not available)",
            "config": workload_config(R, run, ws),
            "test_rmse": rms[-1],
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"outer iterations {args.warmup + 1}-{args.warmup + args.steps} "
                                       f"({run['k']} rank-one updates and the test RMSE each) on the full "
                                       f"matrix, {sum(secs):.1f} s, oracle port of src/cdmf_ref.cpp, "
                                       f"OpenMP over {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return

    from cdmf_gb300 import engine, _lib
    dist = Dist(ws, rank)
    device = local
    R, run = synth.config(WORKLOAD, threads=threads)
    run["k"] = args.k
    k, lam, T = run["k"], run["lambda_"], run["maxinneriter"]
    W0 = synth.initial_w(k, R.m, seed=rank)

    def measure(residual, k=k, W0=W0):
        """Device-resident timing of args.steps outer iterations + a roofline pass."""
        t_create = time.perf_counter()
        e = engine.Engine(R, k, lam, maxiter=max(args.steps, args.e2e_outer), maxinneriter=T, residual=residual,
                          device=device, version=args.version, use_graph=bool(args.graph),
                          relabel=bool(args.relabel), layout=args.layout, autotune=bool(args.autotune))
        t_create = time.perf_counter() - t_create
        bincfg = e.bincfg()
        e.set_factors(W0)
        e.run(args.warmup)
        dist.barrier()
        with ClockSampler(device) as clk:
            rm = e.run(args.steps)
            st = e.stats()
        t_ms = dist.max(st["train_ms"])
        dist.barrier()
        # roofline pass: per-launch events around the sweeps
        e.set_profiling(True)
        e.run(2)
        sp = e.stats()
        e.set_profiling(False)
        e.close()
        n_sweeps = sp["sweep_csc_launches"] + sp["sweep_csr_launches"]
        sweep_ms = sp["sweep_csc_ms"] + sp["sweep_csr_ms"]
        bytes_launch = sp["bytes_per_update"] / (2 * T)
        mean_launch_s = sweep_ms / 1e3 / n_sweeps
        return dict(value=ws * st["updates"] / (t_ms / 1e3), t_ms=t_ms, launches=st["launches"],
                    achieved=bytes_launch / mean_launch_s / 1e9, bytes_launch=bytes_launch,
                    mean_launch_s=mean_launch_s, test_rmse=float(rm[-1]) if rm is not None else None,
                    clocks=clk.summary(), refresh_ms_per_outer=sp["refresh_ms"] / 2, rmse_ms_per_outer=sp["rmse_ms"] / 2,
                    create_s=t_create, bincfg=bincfg)

    head = measure(args.residual)
    comp = measure(args.compare) if args.compare != "none" else None
    # the same matrix at the workload's other rank, k = 32 (both residuals)
    k32 = None
    if not args.quick and args.k == 64:
        W32 = synth.initial_w(32, R.m, seed=rank)
        k32 = {"residual": measure(args.residual, 32, W32)}
        if args.compare != "none":
            k32["compare"] = measure(args.compare, 32, W32)
    value, t_ms, launches = head["value"], head["t_ms"], head["launches"]
    achieved, bytes_launch, mean_launch_s = head["achieved"], head["bytes_launch"], head["mean_launch_s"]
    test_rmse = head["test_rmse"]
    peak, peak_kind = measured_peak()
    tr = profiled_traffic()
    traffic = None
    if (tr and tr.get("workload") == WORKLOAD and tr.get("residual") == args.residual and args.version in (1, 2)
            and args.layout == "lines" and args.k == 64):
        traffic = tr.get("dram_bytes_per_launch")

    if args.quick:
        args.no_cpu = True
    e2e = None
    if not args.quick:
        e2e = run_e2e(R, W0, k, lam, T, args, dist, ws, device)
    fmt = None
    if not args.quick and rank == 0:
        fmt = measure_formats(R, peak)
    batch = None
    if not args.quick and not args.no_batch and rank == 0:
        batch = measure_batch(args, threads, args.batch_residual)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        secs, _ = cpu_outer_iterations(R, run, W0, threads, n_warm=1, budget_s=args.cpu_budget)
        cpu = {"value": k * len(secs) / sum(secs), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"outer iterations 2-{len(secs) + 1} ({k} rank-one updates and the test RMSE each) "
                         f"on the full matrix, {sum(secs):.1f} s, oracle port of src/cdmf_ref.cpp, OpenMP "
                         f"over {threads} threads"}
    dist.close()
    if rank != 0:
        return
    clocks = head["clocks"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.residual == "f32" else f"{args.residual} residual, f32 factors and accumulation",
        "data": "synthetic (seeded, Netflix-shaped; the data set itself is not available)",
        "config": workload_config(R, run, ws),
        "engine": {"residual": args.residual, "version": args.version, "cuda_graph": bool(args.graph),
                   "relabel": bool(args.relabel), "layout": args.layout, "autotune": bool(args.autotune)},
        "outer_per_s": 1e3 * args.steps / t_ms,
        "hbm_gbs_sweeps": achieved,
        "test_rmse": test_rmse,
        "gpu_launches": launches,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind,
                     "kernel": ("blocked_sweep_kernel + blocked_combine_kernel" if args.layout == "blocked" else
                                "tile_sweep_kernel" if args.version == 3 else "sweep_kernel")
                               + " (CSC h-sweep + CSR w-sweep)",
                     "bytes_per_launch": bytes_launch, "mean_launch_ms": mean_launch_s * 1e3},
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if comp is not None:
        line["comparison"] = {"residual": args.compare, "value": comp["value"], "unit": UNIT,
                              "ms_per_step": comp["t_ms"] / args.steps, "test_rmse": comp["test_rmse"],
                              "roofline_frac": comp["achieved"] / peak, "hbm_gbs_sweeps": comp["achieved"]}
        line["mixed_vs_fp32"] = value / comp["value"] if args.compare == "f32" else None
    line["refresh_ms_per_outer"] = head["refresh_ms_per_outer"]
    line["create_s"] = head["create_s"]
    line["bincfg"] = head["bincfg"]
    if fmt is not None:
        line["formats"] = fmt
    line["rmse_ms_per_outer"] = head["rmse_ms_per_outer"]
    if k32 is not None:
        a = k32["residual"]
        line["k32"] = {"value": a["value"], "unit": UNIT, "residual": args.residual,
                       "ms_per_step": a["t_ms"] / args.steps, "test_rmse": a["test_rmse"],
                       "roofline_frac": a["achieved"] / peak, "hbm_gbs_sweeps": a["achieved"]}
        if "compare" in k32:
            c = k32["compare"]
            line["k32"]["comparison"] = {"residual": args.compare, "value": c["value"],
                                         "ms_per_step": c["t_ms"] / args.steps, "test_rmse": c["test_rmse"],
                                         "roofline_frac": c["achieved"] / peak}
            line["k32"]["mixed_vs_fp32"] = a["value"] / c["value"] if args.compare == "f32" else None
    if batch is not None:
        line["batch64"] = batch
    print(json.dumps(line), flush=True)


def measure_batch(args, threads, residual):
    """64 independent problems (sizes, k and lambda drawn per problem, 10 x 1):
    one batched run (each problem's launches on its own stream, the whole run
    one CUDA graph) against the same problems run one after another through
    their own handles.  Returns the batch's measurement as a dict."""
    from cdmf_gb300 import engine, synth
    specs = synth.batch_specs(64, seed=0)
    probs = [synth.generate(threads=threads, **sp["matrix"]) for sp in specs]
    runs = [sp["run"] for sp in specs]
    W0s = [synth.initial_w(r["k"], R.m, seed=q) for q, (R, r) in enumerate(zip(probs, runs))]
    n_outer = 10
    t_create = time.perf_counter()
    with engine.Batch(probs, runs, maxiter=n_outer, maxinneriter=1, residual=residual,
                      use_graph=bool(args.graph), autotune=bool(args.batch_autotune)) as b:
        t_create = time.perf_counter() - t_create
        for _ in range(args.warmup):
            b.set_factors(W0s)
            b.run(n_outer)
        t_batch, t_seq = [], []
        rs = None
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                b.set_factors(W0s)
                rm = b.run(n_outer)
                st = b.stats()
                t_batch.append(st["train_ms"])
                if args.quick:   # batched runs only (profiling)
                    continue
                b.set_factors(W0s)
                rs, ms = b.run_sequential(n_outer)
                t_seq.append(ms)
    updates = sum(r["k"] for r in runs) * n_outer
    tb = statistics.median(t_batch)
    tsq = statistics.median(t_seq) if t_seq else None
    return {
        "metric": "batched CCD++ rank-one updates/s (64 uneven problems)", "value": updates / (tb / 1e3),
        "unit": "rank-one updates/s", "ms_per_run": tb, "runs_timed": args.steps,
        "residual": residual,
        "data": "synthetic (seeded): m logU[1k,200k], n logU[500,20k], nnz logU[50k,5M] <= 30% fill",
        "config": {"workload": "batch64", "problems": 64, "total_train_nnz": int(sum(R.nnz for R in probs)),
                   "outer": n_outer, "inner": 1, "step": "one batched run of 10 outer iterations",
                   "autotune": bool(args.batch_autotune)},
        "create_s": t_create,
        "sequential_ms": tsq, "speedup_vs_sequential": tsq / tb if tsq else None,
        "rmse_equal_to_sequential": bool(np.array_equal(rm, rs)) if rs is not None else None,
        "gpu_launches": st["launches"], "clocks": clk.summary(),
    }


def bench_batch(args, threads):
    """--workload batch64: the batch measurement as its own JSON line."""
    b = measure_batch(args, threads, args.batch_residual)
    line = {"metric": b["metric"], "value": b["value"], "unit": b["unit"], "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": b["ms_per_run"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": f"{b['residual']} residual, f32 factors and accumulation"}
    line.update({k: v for k, v in b.items() if k not in line})
    print(json.dumps(line), flush=True)


def measure_formats(R, peak):
    """The format-build and dual-SpMV entry points on the same matrix:
    cdmf_cuda_compress from the shuffled host COO (upload, sorts, download
    included) and one cdmf_spmv_run over the CSR (kernel time; compulsory
    bytes = index, value and row pointers, x once, 8 B written per row)."""
    import ctypes
    import torch
    from cdmf_gb300 import formats, _lib
    rows, cols, vals = R.coo()
    perm = np.random.default_rng(0).permutation(rows.size)
    rows, cols, vals = rows[perm], cols[perm], vals[perm].astype(np.float64)
    formats.compress_gpu(R.m, R.n, rows[:1000], cols[:1000], vals[:1000])   # warm-up
    t0 = time.perf_counter()
    got = formats.compress_gpu(R.m, R.n, rows, cols, vals)
    compress_s = time.perf_counter() - t0
    same = all(np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in
               zip(got, (R.csr_ptr, R.csr_idx, R.csr_val, R.csc_ptr, R.csc_idx, R.csc_val)))
    lib = _lib.load()
    dev = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()
    dp, di, dv = dev(R.csr_ptr), dev(R.csr_idx), dev(R.csr_val)
    dx = torch.rand(R.n, dtype=torch.float32, device="cuda")
    yt = torch.empty(R.m, dtype=torch.float32, device="cuda")
    yb = torch.empty(R.m, dtype=torch.float32, device="cuda")
    h = ctypes.c_void_p()
    _lib.check(lib.cdmf_spmv_create(R.m, R.n, 0, ctypes.byref(h)), "cdmf_spmv_create")
    try:
        _lib.check(lib.cdmf_spmv_input_csr(h, R.nnz, dp.data_ptr(), di.data_ptr(), dv.data_ptr()), "input_csr")
        _lib.check(lib.cdmf_spmv_as_csr5(h), "as_csr5")
        _lib.check(lib.cdmf_spmv_set_x(h, dx.data_ptr()), "set_x")
        ms = ctypes.c_double()
        times = []
        for _ in range(6):
            _lib.check(lib.cdmf_spmv_run(h, 1.0, yt.data_ptr(), yb.data_ptr(), ctypes.byref(ms)), "spmv")
            times.append(ms.value)
    finally:
        lib.cdmf_spmv_destroy(h)
    spmv_ms = statistics.median(times[1:])
    spmv_bytes = 8.0 * R.nnz + 4.0 * (R.m + 1) + 4.0 * R.n + 8.0 * R.m   # compulsory: x read once
    return {"compress_s": compress_s, "compress_nnz": int(rows.size), "compress_matches_host_build": bool(same),
            "spmv_ms": spmv_ms, "spmv_gbs": spmv_bytes / spmv_ms / 1e6,
            "spmv_frac": spmv_bytes / spmv_ms / 1e6 / peak}


def with_phase_times(fn):
    """Runs fn() with the engine's stderr (the phase times that verbose
    options print) captured; returns (fn's result, {phase: ms})."""
    import re
    sys.stderr.flush()
    saved = os.dup(2)
    with tempfile.TemporaryFile() as tf:
        os.dup2(tf.fileno(), 2)
        try:
            out = fn()
        finally:
            os.dup2(saved, 2)
            os.close(saved)
        tf.seek(0)
        text = tf.read().decode(errors="replace")
    phases = {}
    for kind, what, ms in re.findall(r"\[cdmf\] (train|create): (.+?)\s+([0-9.]+) ms", text):
        phases[(what.strip() if kind == "train" else "create/" + what.strip())] = float(ms)
    return out, phases


def run_e2e(R, W0, k, lam, T, args, dist, ws, device):
    """updates/s through cdmf_cuda_train from page-locked host buffers."""
    from cdmf_gb300 import engine, _lib
    from cdmf_gb300.formats import RatingMatrix
    arrays = {}
    owners = []
    for name in ("csr_ptr", "csr_idx", "csr_val", "csc_ptr", "csc_idx", "csc_val", "te_row", "te_col", "te_val"):
        src = getattr(R, name)
        a, o = _lib.pinned_empty(src.shape, src.dtype)
        a[...] = src
        arrays[name] = a
        owners.append(o)
    Rp = RatingMatrix(R.m, R.n, **arrays)
    Wp, ow = _lib.pinned_empty(W0.shape, np.float32)
    owners.append(ow)
    Hp, oh = _lib.pinned_empty((k, R.n), np.float32)
    owners.append(oh)
    # the engine copies the caller's CSC arrays only when it does not build
    # the renumbered copies itself on the device (relabel off, or blocked)
    copied = [f for f in arrays if not (f.startswith("csc_") and args.relabel and args.layout == "lines")]
    h2d = sum(getattr(Rp, f).nbytes for f in copied) + W0.nbytes
    d2h = W0.nbytes + 4 * k * R.n + 8 * args.e2e_outer
    Wp[...] = W0
    kw = dict(residual=args.residual, device=device, version=args.version, use_graph=bool(args.graph),
              relabel=bool(args.relabel), layout=args.layout, autotune=bool(args.autotune))
    # warms the context; with the autotuner on, also its per-shape cache, so
    # the timed calls reuse the limits it picked
    engine.train(Rp, Wp, k, lam, 1, T, H=Hp, inplace=True, **kw)
    # three timed calls, each from the same W0; the median call is reported
    # (verbose: the engine prints its phase times, recorded per call; one
    # clock sampler runs through the three calls)
    times, phases = [], []
    with ClockSampler(device) as clk:
        for _ in range(3):
            Wp[...] = W0
            dist.barrier()
            t0 = time.perf_counter()
            (_, _, e2e_rm), ph = with_phase_times(
                lambda: engine.train(Rp, Wp, k, lam, args.e2e_outer, T, H=Hp, inplace=True, verbose=1, **kw))
            times.append(dist.max(time.perf_counter() - t0))
            phases.append(ph)
    clocks = clk.summary()
    e2e_s = statistics.median(times)
    e2e_value = ws * k * args.e2e_outer / e2e_s
    return {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "step": f"one cdmf_cuda_train call: upload, {args.e2e_outer} outer iterations, download "
                    f"(median of {len(times)} calls" + ("; bin limits from the autotuner's per-shape cache, "
                                                         "filled by an untimed first call)" if args.autotune
                                                         else ")"),
            "seconds": e2e_s, "seconds_all": times, "clocks": clocks, "phases_ms_per_call": phases,
            "test_rmse": float(e2e_rm[-1])}


if __name__ == "__main__":
    main()
