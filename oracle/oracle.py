"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

liboracle_f32.so / liboracle_f64.so: the C restatement of the reference's
CCD++ engine (oracle/ccdpp_oracle.c).  libmixed_model.so: a model of the
engine's 16-bit residual mode (oracle/mixed_model.c).  _ref/libcdmf_ref.so: the reference's
own src/cdmf_ref.cpp + src/tools.cpp (oracle/build_ref.sh), present only
where the reference sources are.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libcdmf_ref.so")


class OracleProblem(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int64), ("n", ctypes.c_int64), ("nnz", ctypes.c_int64),
        ("csr_row_ptr", ctypes.c_void_p), ("csr_col_idx", ctypes.c_void_p), ("csr_val", ctypes.c_void_p),
        ("csc_col_ptr", ctypes.c_void_p), ("csc_row_idx", ctypes.c_void_p), ("csc_val", ctypes.c_void_p),
        ("nnz_test", ctypes.c_int64),
        ("test_row", ctypes.c_void_p), ("test_col", ctypes.c_void_p), ("test_val", ctypes.c_void_p),
    ]


def build():
    """Compiles liboracle_f32/f64 (and oracle/_ref when the reference is present)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    subprocess.check_call([os.path.join(HERE, "build_ref.sh")], stdout=subprocess.DEVNULL)


_LIBS = {}


def _lib(dtype):
    key = np.dtype(dtype).name
    if key not in _LIBS:
        path = os.path.join(HERE, "liboracle_f32.so" if key == "float32" else "liboracle_f64.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.oracle_ccdpp.argtypes = [ctypes.POINTER(OracleProblem), ctypes.c_uint32, d, i, i, i, vp, vp, vp, vp, vp,
                                     vp, vp, vp]
        lib.oracle_ccdpp.restype = i
        lib.oracle_outer_iteration.argtypes = [ctypes.POINTER(OracleProblem), ctypes.c_uint32, d, i, i, i, vp, vp,
                                               vp, vp, vp, vp]
        lib.oracle_outer_iteration.restype = i
        lib.oracle_rmse.argtypes = [ctypes.POINTER(OracleProblem), ctypes.c_uint32, vp, vp]
        lib.oracle_rmse.restype = d
        _LIBS[key] = lib
    return _LIBS[key]


def _p(a):
    return None if a is None else a.ctypes.data


def problem(R):
    """OracleProblem over a RatingMatrix (arrays must stay alive)."""
    return OracleProblem(R.m, R.n, R.nnz, _p(R.csr_ptr), _p(R.csr_idx), _p(R.csr_val), _p(R.csc_ptr),
                         _p(R.csc_idx), _p(R.csc_val), R.nnz_test, _p(R.te_row), _p(R.te_col), _p(R.te_val))


def ccdpp(R, W0, k, lam, maxiter, maxinner, threads=0, dtype=np.float32, history=False, residuals=False):
    """Runs the oracle engine.  Returns dict(W, H, rmse[maxiter], times, [W_hist, H_hist], [res_csc, res_csr])."""
    lib = _lib(dtype)
    P = problem(R)
    W = np.ascontiguousarray(W0, dtype=dtype).copy()
    H = np.zeros((k, R.n), dtype=dtype)
    rmse = np.zeros(max(1, maxiter), np.float64)
    times = np.zeros(2 * max(1, maxiter), np.float64)
    Wh = np.zeros((maxiter, k, R.m), dtype) if history else None
    Hh = np.zeros((maxiter, k, R.n), dtype) if history else None
    rc = np.zeros(R.nnz, dtype) if residuals else None
    rr = np.zeros(R.nnz, dtype) if residuals else None
    st = lib.oracle_ccdpp(ctypes.byref(P), k, lam, maxiter, maxinner, threads, _p(W), _p(H), _p(rmse), _p(Wh),
                          _p(Hh), _p(rc), _p(rr), _p(times))
    if st != 0:
        raise RuntimeError("oracle_ccdpp failed")
    out = dict(W=W, H=H, rmse=rmse[:maxiter], times=times[:2 * maxiter].reshape(-1, 2))
    if history:
        out.update(W_hist=Wh, H_hist=Hh)
    if residuals:
        out.update(res_csc=rc, res_csr=rr)
    return out


def outer_iteration(R, W, H, res_csc, res_csr, k, lam, maxinner, oiter, threads=0):
    """One outer iteration in place on an explicit state (float32 or float64 arrays)."""
    lib = _lib(W.dtype)
    P = problem(R)
    st = lib.oracle_outer_iteration(ctypes.byref(P), k, lam, maxinner, oiter, threads, _p(W), _p(H), _p(res_csc),
                                    _p(res_csr), None, None)
    if st != 0:
        raise RuntimeError("oracle_outer_iteration failed")


def rmse(R, W, H, k):
    lib = _lib(W.dtype)
    P = problem(R)
    return lib.oracle_rmse(ctypes.byref(P), k, _p(W), _p(H))


def objective(R, W, H, res, lam):
    """FP64 objective of a state: (sum r^2, lambda (sum_i nnz_i |w_i|^2 + sum_j nnz_j |h_j|^2), total).

    The first term is the loss that UpdateRating accumulates over the CSC copy
    (src/cdmf_ref.cpp:20-43); the regulariser weights each line by its
    nonzero count, as RankOneUpdate scales lambda (src/cdmf_ref.cpp:8).
    """
    r = np.asarray(res, np.float64)
    sq = float(np.dot(r, r))
    nr = np.diff(R.csr_ptr.astype(np.int64)).astype(np.float64)
    nc = np.diff(R.csc_ptr.astype(np.int64)).astype(np.float64)
    W64 = np.asarray(W, np.float64)
    H64 = np.asarray(H, np.float64)
    lam = float(np.float32(lam))   # parameter.lambda is a VALUE_TYPE float (src/pmf.h:16)
    reg = lam * (float(np.dot(nr, (W64 * W64).sum(axis=0))) + float(np.dot(nc, (H64 * H64).sum(axis=0))))
    return sq, reg, sq + reg


_SYNTH = []


def synth_lib():
    """The seeded matrix generator (include/cdmf_synth.h) as oracle/libsynth.so,
    for callers that must not load the engine library (the benchmark's CPU
    reference arm); it makes the same matrices as the engine library's copy."""
    if not _SYNTH:
        path = os.path.join(HERE, "libsynth.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        vp, i = ctypes.c_void_p, ctypes.c_int
        lib.cdmf_synth_create.argtypes = [vp, i, vp]
        lib.cdmf_synth_create.restype = i
        lib.cdmf_synth_info.argtypes = [vp, vp, vp, vp, vp]
        lib.cdmf_synth_info.restype = i
        lib.cdmf_synth_copy.argtypes = [vp] * 10
        lib.cdmf_synth_copy.restype = i
        lib.cdmf_synth_destroy.argtypes = [vp]
        lib.cdmf_synth_destroy.restype = None
        _SYNTH.append(lib)
    return _SYNTH[0]


_MODEL = []
STORAGE = {"f32": 0, "bf16": 1, "f16": 2}


def mixed_model(R, W0, k, lam, maxiter, maxinner, storage="bf16", refresh_every=0, refresh_all=False, threads=0):
    """CPU model of the engine's 16-bit residual mode (oracle/mixed_model.c):
    the residual rounded to `storage` on every write, the subtract and the
    add-back fused, a refresh from FP32 at the start of every outer iteration
    after the first, and, with refresh_every > 0, every refresh_every features
    of the first (of every one with refresh_all).  With storage "f32" it is
    the reference's arithmetic.  Returns dict(W, H, rmse)."""
    if not _MODEL:
        path = os.path.join(HERE, "libmixed_model.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        vp, i = ctypes.c_void_p, ctypes.c_int
        lib.mixed_model_ccdpp.argtypes = [ctypes.POINTER(OracleProblem), ctypes.c_uint32, ctypes.c_double, i, i, i, i,
                                          i, i, vp, vp, vp]
        lib.mixed_model_ccdpp.restype = i
        _MODEL.append(lib)
    P = problem(R)
    W = np.ascontiguousarray(W0, np.float32).copy()
    H = np.zeros((k, R.n), np.float32)
    rm = np.zeros(max(1, maxiter), np.float64)
    st = _MODEL[0].mixed_model_ccdpp(ctypes.byref(P), k, lam, maxiter, maxinner, STORAGE[storage], refresh_every,
                                     int(bool(refresh_all)), threads, _p(W), _p(H), _p(rm))
    if st != 0:
        raise RuntimeError("mixed_model_ccdpp failed (CSC not the transpose of CSR, or out of memory)")
    return dict(W=W, H=H, rmse=rm[:maxiter])


def reference_available():
    return os.path.exists(REF_LIB)


def reference_run(data_dir, W0, k, lam, maxiter, maxinner, threads=1, residuals=False):
    """The reference's own cdmf_ref on a cdmf-format directory (oracle/_ref)."""
    lib = ctypes.CDLL(REF_LIB)
    m, n = ctypes.c_long(), ctypes.c_long()
    nnz, nt = ctypes.c_ulong(), ctypes.c_ulong()
    lib.ref_dims(data_dir.encode(), ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nt))
    W0 = np.ascontiguousarray(W0, np.float32)
    W = np.zeros((k, m.value), np.float32)
    H = np.zeros((k, n.value), np.float32)
    r = ctypes.c_double()
    rc = np.zeros(nnz.value, np.float32) if residuals else None
    rr = np.zeros(nnz.value, np.float32) if residuals else None
    lib.ref_run.argtypes = [ctypes.c_char_p, ctypes.c_uint, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_void_p]
    lib.ref_run(data_dir.encode(), k, lam, maxiter, maxinner, threads, _p(W0), _p(W), _p(H), ctypes.addressof(r),
                _p(rc), _p(rr))
    out = dict(W=W, H=H, rmse=r.value)
    if residuals:
        out.update(res_csc=rc, res_csr=rr)
    return out


def reference_initial_col(k, n):
    lib = ctypes.CDLL(REF_LIB)
    X = np.zeros((k, n), np.float32)
    lib.ref_initial_col.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]
    lib.ref_initial_col(_p(X), k, n)
    return X
