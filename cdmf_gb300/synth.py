"""Seeded synthetic rating matrices for the five workloads of this engine.

The reference measured on Netflix, MovieLens-20M and Jester
(SomeResults/*-GPU0{2,3}); those data sets are not available, so seeded
synthetic matrices with their shapes, sizes and value distributions stand in
for them.  Generation runs in libcdmf_cuda.so (include/cdmf_synth.h), or in
any other library built from the same generator source.
"""
import ctypes
import math

import numpy as np

from . import _lib
from .formats import RatingMatrix


def spec(**kw):
    s = _lib.SynthSpec()
    defaults = dict(nnz_test=-1, test_fraction=0.01, row_mode=0, row_alpha=1.0, row_min=1, row_max=0,
                    col_mode=0, col_alpha=1.0, col_cap=0, col_beta_a=2.0, col_beta_b=1.5, col_min_one=1,
                    rank=10, factor_std=0.6, planted_std=0.0, offset=3.0, noise_std=0.5, quantum=1.0,
                    vmin=1.0, vmax=5.0, seed=0)
    defaults.update(kw)
    if defaults["row_max"] <= 0:
        defaults["row_max"] = defaults["n"]
    for k, v in defaults.items():
        setattr(s, k, v)
    return s


# Workload presets.  Each entry: matrix spec + CCD++ run parameters.
CONFIGS = {
    # 20,000 x 4,000, 1.0M distinct nonzeros, Zipf 0.8 rows and columns, >= 1
    # per row and column, integer 1-5 from a planted rank-10 model (U, V ~
    # N(0, 0.6)) + 3.0 + N(0, 0.5), 1 % held out.  k=16, lambda=0.05, 5 x 1.
    "cpu_scale": dict(
        matrix=dict(m=20000, n=4000, nnz_total=1_000_000, test_fraction=0.01, row_alpha=0.8, row_min=1,
                    row_max=2000, col_alpha=0.8, col_cap=10000, rank=10, factor_std=0.6, offset=3.0,
                    noise_std=0.5, quantum=1.0, vmin=1.0, vmax=5.0),
        run=dict(k=16, lambda_=0.05, maxiter=5, maxinneriter=1)),
    # 480,189 x 17,770, 100,480,507 nonzeros, 1,408,395 held out; rows capped
    # Zipf 1.0 (max 17,000, mean ~209), columns capped Zipf 1.0 (max ~230k,
    # mean ~5.6k); integer 1-5 from a planted rank-20 model + 3.0 + N(0, 0.6).
    # k=32 or 64, lambda=0.05, 20 x 1.
    "netflix_shape": dict(
        matrix=dict(m=480189, n=17770, nnz_total=100_480_507, nnz_test=1_408_395, row_alpha=1.0, row_min=1,
                    row_max=17000, col_alpha=1.0, col_cap=900000, rank=20, factor_std=0.5, planted_std=1.0,
                    offset=3.0, noise_std=0.6, quantum=1.0, vmin=1.0, vmax=5.0),
        run=dict(k=64, lambda_=0.05, maxiter=20, maxinneriter=1)),
    # 138,493 x 26,744, 20,000,263 nonzeros, >= 20 per row, rows Zipf 0.9,
    # columns Zipf 1.1, half stars 0.5-5.0 from a planted rank-16 model + 3.5
    # + N(0, 0.7), 2 % held out.  k=128, lambda=0.1, 10 x 3.
    "ml20m_shape": dict(
        matrix=dict(m=138493, n=26744, nnz_total=20_000_263, test_fraction=0.02, row_alpha=0.9, row_min=20,
                    row_max=9254, col_alpha=1.1, col_cap=67310, rank=16, factor_std=0.5, planted_std=1.0,
                    offset=3.5, noise_std=0.7, quantum=0.5, vmin=0.5, vmax=5.0),
        run=dict(k=128, lambda_=0.1, maxiter=10, maxinneriter=3)),
    # 73,421 x 100, 15-100 entries per row (uniform), column inclusion weights
    # ~ Beta(2, 1.5), continuous values in [-10, 10] from a planted rank-8
    # model scaled to std 4.5 + N(0, 2.0), clipped, 1 % held out.
    # k=10, lambda=0.5, 15 x 2.
    "jester_shape": dict(
        matrix=dict(m=73421, n=100, nnz_total=0, test_fraction=0.01, row_mode=1, row_min=15, row_max=100,
                    col_mode=1, col_beta_a=2.0, col_beta_b=1.5, rank=8, factor_std=1.0, planted_std=4.5,
                    offset=0.0, noise_std=2.0, quantum=0.0, vmin=-10.0, vmax=10.0),
        run=dict(k=10, lambda_=0.5, maxiter=15, maxinneriter=2)),
}


def generate(threads=0, seed=0, lib=None, **matrix):
    """Generates one matrix; keyword arguments are cdmf_synth_spec fields.
    `lib`: a library exporting the cdmf_synth_* functions (default: the
    engine library)."""
    lib = lib or _lib.load()
    sp = spec(seed=seed, **matrix)
    h = ctypes.c_void_p()
    _lib.check(lib.cdmf_synth_create(ctypes.byref(sp), int(threads), ctypes.byref(h)), "cdmf_synth_create")
    try:
        m, n, nnz, nt = (ctypes.c_int64() for _ in range(4))
        lib.cdmf_synth_info(h, ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nt))
        m, n, nnz, nt = m.value, n.value, nnz.value, nt.value
        u32, f32 = np.uint32, np.float32
        a = dict(csr_ptr=np.empty(m + 1, u32), csr_idx=np.empty(nnz, u32), csr_val=np.empty(nnz, f32),
                 csc_ptr=np.empty(n + 1, u32), csc_idx=np.empty(nnz, u32), csc_val=np.empty(nnz, f32),
                 te_row=np.empty(nt, u32), te_col=np.empty(nt, u32), te_val=np.empty(nt, f32))
        P, U, F = _lib.ptr, ctypes.c_uint32, ctypes.c_float
        _lib.check(lib.cdmf_synth_copy(h, P(a["csr_ptr"], U), P(a["csr_idx"], U), P(a["csr_val"], F),
                                       P(a["csc_ptr"], U), P(a["csc_idx"], U), P(a["csc_val"], F),
                                       P(a["te_row"], U), P(a["te_col"], U), P(a["te_val"], F)), "cdmf_synth_copy")
    finally:
        lib.cdmf_synth_destroy(h)
    return RatingMatrix(m, n, **a)


def config(name, threads=0, seed=0, lib=None, **overrides):
    """(matrix, run-parameters) of a named workload; overrides patch the matrix spec."""
    c = CONFIGS[name]
    mspec = dict(c["matrix"])
    mspec.update(overrides)
    return generate(threads=threads, seed=seed, lib=lib, **mspec), dict(c["run"])


def batch_specs(count=64, seed=0):
    """The uneven batch: per problem m ~ logU[1k, 200k], n ~ logU[500, 20k],
    nnz ~ logU[50k, 5M] capped at 30 % fill, Zipf 0.9 rows and columns,
    integer 1-5 from a planted rank-8 model + noise, k in {8, 16, 32},
    lambda in {0.01, 0.05, 0.1, 0.5}, 10 x 1."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(count):
        m = int(round(math.exp(rng.uniform(math.log(1000), math.log(200000)))))
        n = int(round(math.exp(rng.uniform(math.log(500), math.log(20000)))))
        nnz = int(round(math.exp(rng.uniform(math.log(50000), math.log(5000000)))))
        nnz = min(nnz, int(0.3 * m * n))
        k = int(rng.choice([8, 16, 32]))
        lam = float(rng.choice([0.01, 0.05, 0.1, 0.5]))
        matrix = dict(m=m, n=n, nnz_total=nnz, test_fraction=0.01, row_alpha=0.9, row_min=1 if nnz >= 2 * m else 0,
                      row_max=max(1, n // 2), col_alpha=0.9, col_cap=max(1, m // 2), rank=8, factor_std=0.6,
                      offset=3.0, noise_std=0.5, quantum=1.0, vmin=1.0, vmax=5.0, seed=seed * 1000 + p)
        out.append(dict(matrix=matrix, run=dict(k=k, lambda_=lam, maxiter=10, maxinneriter=1)))
    return out


def initial_w(k, m, seed=0):
    """Initial W ~ U(0, 1/sqrt(k)), float32, k x m feature-major, from a seeded
    numpy generator; H starts at zero (the reference zeroes H first,
    src/cdmf_ref.cpp:57-61)."""
    rng = np.random.default_rng(seed)
    return (rng.random((k, m), dtype=np.float64) / math.sqrt(k)).astype(np.float32)


def reference_initial_col(k, n):
    """The reference's own initial_col (src/tools.cpp:349-357), via the C library's rand()."""
    X = np.empty((k, n), np.float32)
    _lib.load().cdmf_initial_col(_lib.ptr(X, ctypes.c_float), k, n)
    return X
