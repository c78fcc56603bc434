"""Generates the golden vectors under tests/golden/ by running the REFERENCE's
own CPU engine (src/cdmf_ref.cpp + src/tools.cpp, compiled unmodified into
oracle/_ref by oracle/build_ref.sh) -- run here, where the reference sources
are; the GPU host only reads the committed .npz files.

Cases:
  simple, tricky_simple: the reference's own fixtures (data/simple,
      data/tricky_simple), converted with scipy exactly as their
      *_compress.py scripts do (coo -> tocsr/tocsc), with the reference's
      ctest parameters (CMakeLists.txt:63-67: -k 10 -t 5 -T 3 -l 0.05) and
      the reference's initial_col factors;
  mini: a seeded synthetic matrix (1,500 x 400, Zipf degrees, an empty row
      and column planted), k=8, lambda=0.05, 4 x 2, injected W ~ U(0, 1/sqrt(k)).
  cpu_scale: the 20,000 x 4,000 / 1M-nnz workload, k=16, lambda=0.05, 5 x 1;
      stored as RMSE values and SHA-256 digests of the final W and H
      (with the digest of the generated matrix, to know when they apply).
For every case the output after j outer iterations is the reference run with
maxiter = j (the reference restarts deterministically from the injected W).
The script also checks the oracle restatement (oracle/ccdpp_oracle.c)
against the reference bit for bit and refuses to write on a mismatch.

Usage: python tests/golden/make_golden.py [reference_root]
"""
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from cdmf_gb300 import formats, synth  # noqa: E402
from oracle import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def scipy_convert(ref_root, name, m, n):
    """data/<name>/<name>_compress.py:79-155 with scipy (the reference's converter)."""
    from scipy import sparse
    d = os.path.join(ref_root, "data", name)
    tr = np.loadtxt(os.path.join(d, name + ".dat"), delimiter="\t",
                    dtype=[("f0", np.int32), ("f1", np.int32), ("f2", np.float64)], unpack=True)
    te = np.loadtxt(os.path.join(d, name + ".test"), delimiter="\t",
                    dtype=[("f0", np.int32), ("f1", np.int32), ("f2", np.float64)], unpack=True)
    te_coo = sparse.coo_matrix((te[2], (te[0] - 1, te[1] - 1)))
    tr_coo = sparse.coo_matrix((tr[2], (tr[0] - 1, tr[1] - 1)))
    csr, csc = tr_coo.tocsr(), tr_coo.tocsc()
    u32 = lambda a: np.ascontiguousarray(a, dtype=np.uint32)  # noqa: E731
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    return formats.RatingMatrix(m, n, u32(csr.indptr), u32(csr.indices), f32(csr.data), u32(csc.indptr),
                                u32(csc.indices), f32(csc.data), u32(te_coo.row), u32(te_coo.col), f32(te_coo.data))


def run_reference(R, W0, k, lam, maxiter, maxinner):
    """Reference outputs after 1..maxiter outer iterations."""
    Wh, Hh, rm = [], [], []
    with tempfile.TemporaryDirectory() as tmp:
        formats.write_dir(tmp, R)
        for j in range(1, maxiter + 1):
            out = oracle.reference_run(tmp, W0, k, lam, j, maxinner, threads=4, residuals=(j == maxiter))
            Wh.append(out["W"])
            Hh.append(out["H"])
            rm.append(out["rmse"])
    return np.stack(Wh), np.stack(Hh), np.array(rm), out["res_csc"], out["res_csr"]


def check_oracle(R, W0, k, lam, maxiter, maxinner, Wh, Hh, rm, rc, rr, label):
    got = oracle.ccdpp(R, W0, k, lam, maxiter, maxinner, threads=4, history=True, residuals=True)
    ok = (np.array_equal(got["W_hist"].view(np.uint32), Wh.view(np.uint32))
          and np.array_equal(got["H_hist"].view(np.uint32), Hh.view(np.uint32))
          and np.array_equal(got["res_csc"].view(np.uint32), rc.view(np.uint32))
          and np.array_equal(got["res_csr"].view(np.uint32), rr.view(np.uint32))
          and np.array_equal(got["rmse"], rm))
    if not ok:
        raise SystemExit(f"oracle restatement differs from the reference on {label}")
    print(f"{label}: oracle == reference bit for bit ({maxiter} outer iterations)")


def matrix_arrays(R):
    return dict(m=R.m, n=R.n, csr_ptr=R.csr_ptr, csr_idx=R.csr_idx, csr_val=R.csr_val, csc_ptr=R.csc_ptr,
                csc_idx=R.csc_idx, csc_val=R.csc_val, te_row=R.te_row, te_col=R.te_col, te_val=R.te_val)


def matrix_digest(R):
    h = hashlib.sha256()
    for a in (R.csr_ptr, R.csr_idx, R.csr_val, R.csc_ptr, R.csc_idx, R.csc_val, R.te_row, R.te_col, R.te_val):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def mini_matrix():
    R = synth.generate(m=1500, n=400, nnz_total=30000, test_fraction=0.02, row_alpha=0.9, row_min=1, row_max=200,
                       col_alpha=0.9, col_cap=750, rank=6, factor_std=0.6, offset=3.0, noise_std=0.5, quantum=1.0,
                       vmin=1.0, vmax=5.0, seed=7)
    # plant an empty row (7) and an empty column (5): drop their training entries
    rows, cols, vals = R.coo()
    keep = (rows != 7) & (cols != 5)
    return formats.from_coo(R.m, R.n, rows[keep], cols[keep], vals[keep], R.te_row, R.te_col, R.te_val)


def main():
    ref_root = (sys.argv[1] if len(sys.argv) > 1 else
                os.environ.get("CDMF_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference")))
    oracle.build()
    if not oracle.reference_available():
        raise SystemExit("oracle/_ref/libcdmf_ref.so missing: the reference sources are needed")
    meta = {}
    for name, (m, n) in (("simple", (6, 5)), ("tricky_simple", (5, 5))):
        R = scipy_convert(ref_root, name, m, n)
        # our own converter must give the same integer structures
        mine = formats.from_coo(m, n, *R.coo(), R.te_row, R.te_col, R.te_val)
        for f in ("csr_ptr", "csr_idx", "csc_ptr", "csc_idx"):
            assert np.array_equal(getattr(mine, f), getattr(R, f)), (name, f)
        k, lam, T, t = 10, 0.05, 3, 5
        W0 = oracle.reference_initial_col(k, m)
        assert np.array_equal(W0.view(np.uint32), synth.reference_initial_col(k, m).view(np.uint32))
        Wh, Hh, rm, rc, rr = run_reference(R, W0, k, lam, t, T)
        check_oracle(R, W0, k, lam, t, T, Wh, Hh, rm, rc, rr, name)
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), W0=W0, W_hist=Wh, H_hist=Hh, rmse=rm, res_csc=rc,
                            res_csr=rr, **matrix_arrays(R))
        meta[name] = dict(k=k, lam=lam, maxinner=T, maxiter=t, rmse=rm.tolist(), source=f"data/{name}")
    R = mini_matrix()
    k, lam, T, t = 8, 0.05, 2, 4
    W0 = synth.initial_w(k, R.m, seed=0)
    Wh, Hh, rm, rc, rr = run_reference(R, W0, k, lam, t, T)
    check_oracle(R, W0, k, lam, t, T, Wh, Hh, rm, rc, rr, "mini")
    np.savez_compressed(os.path.join(OUT, "mini.npz"), W0=W0, W_hist=Wh, H_hist=Hh, rmse=rm, res_csc=rc, res_csr=rr,
                        **matrix_arrays(R))
    meta["mini"] = dict(k=k, lam=lam, maxinner=T, maxiter=t, rmse=rm.tolist(), source="synthetic seed 7")
    R, run = synth.config("cpu_scale")
    k, lam, T, t = run["k"], run["lambda_"], run["maxinneriter"], run["maxiter"]
    W0 = synth.initial_w(k, R.m, seed=0)
    Wh, Hh, rm, rc, rr = run_reference(R, W0, k, lam, t, T)
    check_oracle(R, W0, k, lam, t, T, Wh, Hh, rm, rc, rr, "cpu_scale")
    meta["cpu_scale"] = dict(k=k, lam=lam, maxinner=T, maxiter=t, rmse=rm.tolist(), matrix_sha256=matrix_digest(R),
                             W0="initial_w(k, m, seed=0)",
                             W_sha256=[hashlib.sha256(w.tobytes()).hexdigest() for w in Wh],
                             H_sha256=[hashlib.sha256(h.tobytes()).hexdigest() for h in Hh])
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
