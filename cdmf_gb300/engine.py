"""Python front end of the CUDA engine (include/cdmf_cuda.h through ctypes).

`cdmf_cuda(R, W, H, param)` has the shape of the reference's engine call
`cdmf_ocl_01(R, W, H, T, param, filename)` (src/cdmf.h:8, called at
src/main.cpp:43): W is read and overwritten, H is overwritten, R is left
untouched, and the reference's per-outer-iteration log line is printed.
`Engine` exposes the same engine split into upload / run / read-back, which
the tests and the benchmark use.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, ptr

RESIDUAL = {"f32": _lib.RES_F32, "bf16": _lib.RES_BF16, "f16": _lib.RES_F16}
REDUCE = {"tree": _lib.REDUCE_TREE, "sequential": _lib.REDUCE_SEQUENTIAL}


@dataclass
class parameter:
    """The reference's run parameters (src/pmf.h:4-26), same defaults."""
    threads: int = 16
    nBlocks: int = 1
    nThreadsPerBlock: int = 32
    do_ref: int = 0
    do_predict: int = 0
    maxinneriter: int = 5
    maxiter: int = 5
    k: int = 10
    lambda_: float = 0.1
    platform_id: int = 0
    verbose: int = 0
    version: int = 1
    residual: str = "f32"
    reduce: str = "tree"


def _problem(R):
    U, F = ctypes.c_uint32, ctypes.c_float
    return _lib.Problem(R.m, R.n, R.nnz, ptr(R.csr_ptr, U), ptr(R.csr_idx, U), ptr(R.csr_val, F),
                        ptr(R.csc_ptr, U), ptr(R.csc_idx, U), ptr(R.csc_val, F), R.nnz_test,
                        ptr(R.te_row, U), ptr(R.te_col, U), ptr(R.te_val, F))


def make_opts(k, lambda_, maxiter=5, maxinneriter=5, version=1, residual="f32", reduce="tree",
              rmse_each_outer=True, use_graph=False, device=0, threads_per_block=0, verbose=0, relabel=True,
              autotune=False, layout=None):
    o = _lib.Opts()
    _lib.load().cdmf_opts_default(ctypes.byref(o))
    o.k, o.lambda_, o.maxiter, o.maxinneriter = int(k), float(lambda_), int(maxiter), int(maxinneriter)
    o.version = int(version)
    o.residual = RESIDUAL[residual] if isinstance(residual, str) else int(residual)
    o.reduce = REDUCE[reduce] if isinstance(reduce, str) else int(reduce)
    o.rmse_each_outer = int(bool(rmse_each_outer))
    o.use_graph = int(bool(use_graph))
    o.device, o.threads_per_block, o.verbose = int(device), int(threads_per_block), int(verbose)
    # True / 1: relabel (on the GPU for the line layout); "host" / 2: relabel on the host
    o.relabel = 2 if relabel == "host" else int(relabel) if not isinstance(relabel, bool) else int(relabel)
    o.autotune = int(bool(autotune))
    if layout is not None:
        o.layout = {"lines": 0, "blocked": 1}[layout] if isinstance(layout, str) else int(layout)
    return o


class Engine:
    """One factorisation resident on the GPU."""

    def __init__(self, R, k, lambda_, maxiter=5, maxinneriter=5, **kw):
        self.lib = _lib.load()
        self.R = R
        self.k = int(k)
        self.opts = make_opts(k, lambda_, maxiter, maxinneriter, **kw)
        self._p = _problem(R)
        h = ctypes.c_void_p()
        check(self.lib.cdmf_cuda_create(ctypes.byref(self._p), ctypes.byref(self.opts), ctypes.byref(h)),
              "cdmf_cuda_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.cdmf_cuda_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_factors(self, W0, H0=None):
        W0 = np.ascontiguousarray(W0, np.float32)
        H0 = None if H0 is None else np.ascontiguousarray(H0, np.float32)
        assert W0.shape == (self.k, self.R.m)
        check(self.lib.cdmf_cuda_set_factors(self.h, ptr(W0, ctypes.c_float), ptr(H0, ctypes.c_float)),
              "cdmf_cuda_set_factors", self.h)

    def run(self, n_outer):
        out = np.zeros(max(1, n_outer), np.float64)
        want = self.opts.rmse_each_outer and self.R.nnz_test > 0
        check(self.lib.cdmf_cuda_run(self.h, int(n_outer), ptr(out, ctypes.c_double) if want else None),
              "cdmf_cuda_run", self.h)
        return out[:n_outer] if want else None

    def factors(self):
        W = np.empty((self.k, self.R.m), np.float32)
        H = np.empty((self.k, self.R.n), np.float32)
        check(self.lib.cdmf_cuda_get_factors(self.h, ptr(W, ctypes.c_float), ptr(H, ctypes.c_float)),
              "cdmf_cuda_get_factors", self.h)
        return W, H

    def rmse(self):
        r = ctypes.c_double()
        check(self.lib.cdmf_cuda_rmse(self.h, ctypes.byref(r)), "cdmf_cuda_rmse", self.h)
        return r.value

    def objective(self):
        """(sum of squared residuals, lambda-weighted regulariser, their sum), FP64."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(self.lib.cdmf_cuda_objective(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
              "cdmf_cuda_objective", self.h)
        return a.value, b.value, c.value

    def state(self):
        W = np.empty((self.k, self.R.m), np.float32)
        H = np.empty((self.k, self.R.n), np.float32)
        rc = np.empty(self.R.nnz, np.float32)
        rr = np.empty(self.R.nnz, np.float32)
        nxt = ctypes.c_int()
        F = ctypes.c_float
        check(self.lib.cdmf_cuda_get_state(self.h, ptr(W, F), ptr(H, F), ptr(rc, F), ptr(rr, F), ctypes.byref(nxt)),
              "cdmf_cuda_get_state", self.h)
        return dict(W=W, H=H, res_csc=rc, res_csr=rr, next_oiter=nxt.value)

    def set_state(self, W, H, res_csc, res_csr, next_oiter):
        F = ctypes.c_float
        a = [np.ascontiguousarray(x, np.float32) for x in (W, H, res_csc, res_csr)]
        check(self.lib.cdmf_cuda_set_state(self.h, *(ptr(x, F) for x in a), int(next_oiter)),
              "cdmf_cuda_set_state", self.h)

    def set_profiling(self, on=True):
        check(self.lib.cdmf_cuda_set_profiling(self.h, int(bool(on))), "cdmf_cuda_set_profiling", self.h)

    def stats(self):
        s = _lib.Stats()
        check(self.lib.cdmf_cuda_stats(self.h, ctypes.byref(s)), "cdmf_cuda_stats", self.h)
        return {f: getattr(s, f) for f, _ in _lib.Stats._fields_}

    def bincfg(self):
        c = _lib.BinCfg()
        check(self.lib.cdmf_cuda_get_bincfg(self.h, ctypes.byref(c)), "cdmf_cuda_get_bincfg", self.h)
        return {f: getattr(c, f) for f, _ in _lib.BinCfg._fields_}

    def set_bincfg(self, **kw):
        c = _lib.BinCfg(**{**self.bincfg(), **kw})
        check(self.lib.cdmf_cuda_set_bincfg(self.h, ctypes.byref(c)), "cdmf_cuda_set_bincfg", self.h)

    def autotune(self):
        c = _lib.BinCfg()
        ms = ctypes.c_double()
        check(self.lib.cdmf_cuda_autotune(self.h, ctypes.byref(c), ctypes.byref(ms)), "cdmf_cuda_autotune", self.h)
        return {f: getattr(c, f) for f, _ in _lib.BinCfg._fields_}, ms.value

    def bins(self, which):
        """which: 'csr' or 'csc' -> (lines per bin, nnz per bin) for (thread, group8, warp, cta, split)."""
        c = (ctypes.c_int64 * 5)()
        z = (ctypes.c_int64 * 5)()
        check(self.lib.cdmf_cuda_bins(self.h, 0 if which == "csr" else 1, c, z), "cdmf_cuda_bins", self.h)
        return list(c), list(z)


def train(R, W, k, lambda_, maxiter, maxinneriter, H=None, inplace=False, **kw):
    """One-shot engine call (cdmf_cuda_train): returns (W, H, rmse per outer).

    inplace=True trains the caller's W (float32, C-contiguous) in place and
    writes H into the caller's array (float32, k x n): with page-locked arrays
    (_lib.pinned_empty) the copies run at full link speed."""
    lib = _lib.load()
    o = make_opts(k, lambda_, maxiter, maxinneriter, **kw)
    p = _problem(R)
    if inplace:
        if W.dtype != np.float32 or not W.flags["C_CONTIGUOUS"] or W.shape != (k, R.m):
            raise ValueError("inplace W must be a C-contiguous float32 array of shape (k, m)")
        if H is None or H.dtype != np.float32 or not H.flags["C_CONTIGUOUS"] or H.shape != (k, R.n):
            raise ValueError("inplace needs H: a C-contiguous float32 array of shape (k, n)")
    else:
        W = np.ascontiguousarray(W, np.float32).copy()
        H = np.zeros((k, R.n), np.float32)
    rm = np.zeros(max(1, maxiter), np.float64)
    check(lib.cdmf_cuda_train(ctypes.byref(p), ctypes.byref(o), ptr(W, ctypes.c_float), ptr(H, ctypes.c_float),
                              ptr(rm, ctypes.c_double), _lib.OUTER_CB(), None), "cdmf_cuda_train")
    return W, H, rm[:maxiter]


def cdmf_cuda(R, W, H, param, log=print):
    """Drop-in for cdmf_ocl_01/02 and cdmf_csr5 (src/cdmf.h:6-10): trains in
    place (W in/out, H out) and prints the reference's per-iteration line
    (src/cdmf_ocl_1.cpp:380) and training-time line (:386)."""
    lib = _lib.load()
    o = make_opts(param.k, param.lambda_, param.maxiter, param.maxinneriter, version=param.version,
                  residual=param.residual, reduce=param.reduce, verbose=param.verbose)
    p = _problem(R)
    Wc = np.ascontiguousarray(W, np.float32)
    Hc = np.zeros((param.k, R.n), np.float32)
    lines = []

    def cb(oiter, rmse, ms, user):
        lines.append(f"[-INFO-] iteration num {oiter} \trank_time {0.0:.4f}|{ms / 1e3:.4f} s \t"
                     f"update_time {0.0:.4f}|{0.0:.4f}s \tRMSE={rmse:f} time:{0.0:f}s")
        if log:
            log(lines[-1])

    ccb = _lib.OUTER_CB(cb)
    check(lib.cdmf_cuda_train(ctypes.byref(p), ctypes.byref(o), ptr(Wc, ctypes.c_float), ptr(Hc, ctypes.c_float),
                              None, ccb, None), "cdmf_cuda_train")
    W[...] = Wc
    H[...] = Hc
    return lines


class Batch:
    """Many independent factorisations advanced together (include/cdmf_cuda.h,
    cdmf_cuda_batch_*): problems[q] is a RatingMatrix, runs[q] a dict of
    k / lambda_ (and optionally the other make_opts arguments)."""

    def __init__(self, problems, runs, maxiter, maxinneriter=1, residual="f32", use_graph=True, **kw):
        self.lib = _lib.load()
        self.R = list(problems)
        self.ks = [int(r["k"]) for r in runs]
        n = len(self.R)
        self._probs = (_lib.Problem * n)(*[_problem(R) for R in self.R])
        self._opts = (_lib.Opts * n)(*[make_opts(r["k"], r["lambda_"], maxiter, maxinneriter, residual=residual,
                                                 use_graph=use_graph, **kw) for r in runs])
        h = ctypes.c_void_p()
        st = self.lib.cdmf_cuda_batch_create(self._probs, self._opts, n, ctypes.byref(h))
        check(st, "cdmf_cuda_batch_create")
        self.h = h
        self.maxiter = maxiter

    def close(self):
        if self.h:
            self.lib.cdmf_cuda_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, where):
        if st != 0:
            msg = self.lib.cdmf_cuda_batch_last_error(self.h)
            raise _lib.CdmfError(st, where, msg.decode() if msg else "")

    def set_factors(self, W0s):
        arrs = [np.ascontiguousarray(w, np.float32) for w in W0s]
        ptrs = (ctypes.POINTER(ctypes.c_float) * len(arrs))(*[ptr(a, ctypes.c_float) for a in arrs])
        self._check(self.lib.cdmf_cuda_batch_set_factors(self.h, ptrs), "cdmf_cuda_batch_set_factors")

    def run(self, n_outer):
        out = np.zeros((len(self.R), max(1, n_outer)), np.float64)
        self._check(self.lib.cdmf_cuda_batch_run(self.h, int(n_outer), ptr(out, ctypes.c_double)),
                    "cdmf_cuda_batch_run")
        return out[:, :n_outer]

    def run_sequential(self, n_outer):
        out = np.zeros((len(self.R), max(1, n_outer)), np.float64)
        ms = ctypes.c_double()
        self._check(self.lib.cdmf_cuda_batch_run_sequential(self.h, int(n_outer), ptr(out, ctypes.c_double),
                                                            ctypes.byref(ms)), "cdmf_cuda_batch_run_sequential")
        return out[:, :n_outer], ms.value

    def factors(self):
        Ws = [np.empty((k, R.m), np.float32) for k, R in zip(self.ks, self.R)]
        Hs = [np.empty((k, R.n), np.float32) for k, R in zip(self.ks, self.R)]
        F = ctypes.POINTER(ctypes.c_float)
        pw = (F * len(Ws))(*[ptr(a, ctypes.c_float) for a in Ws])
        ph = (F * len(Hs))(*[ptr(a, ctypes.c_float) for a in Hs])
        self._check(self.lib.cdmf_cuda_batch_get_factors(self.h, pw, ph), "cdmf_cuda_batch_get_factors")
        return Ws, Hs

    def stats(self):
        s = _lib.Stats()
        self._check(self.lib.cdmf_cuda_batch_stats(self.h, ctypes.byref(s)), "cdmf_cuda_batch_stats")
        return {f: getattr(s, f) for f, _ in _lib.Stats._fields_}
