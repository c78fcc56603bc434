"""ctypes binding of libcdmf_cuda.so (include/cdmf_cuda.h, include/cdmf_synth.h).

Loading fails loudly: there is no fallback.  If the library is missing,
`load()` raises with the build command to run.
"""
import ctypes
import os

from . import _build

c_u32p = ctypes.POINTER(ctypes.c_uint32)
c_f32p = ctypes.POINTER(ctypes.c_float)
c_f64p = ctypes.POINTER(ctypes.c_double)
c_i64p = ctypes.POINTER(ctypes.c_int64)

CDMF_OK = 0
STATUS = {
    0: "CDMF_OK", -1: "CDMF_ERR_INVALID", -2: "CDMF_ERR_ALLOC", -3: "CDMF_ERR_CUDA",
    -4: "CDMF_ERR_NO_DEVICE", -5: "CDMF_ERR_EMPTY_TEST", -6: "CDMF_ERR_NUMERIC",
    -7: "CDMF_ERR_UNSUPPORTED", -8: "CDMF_ERR_TOO_LARGE",
}
RES_F32, RES_BF16, RES_F16 = 0, 1, 2
REDUCE_TREE, REDUCE_SEQUENTIAL = 0, 1


class Problem(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int64), ("n", ctypes.c_int64), ("nnz", ctypes.c_int64),
        ("csr_row_ptr", c_u32p), ("csr_col_idx", c_u32p), ("csr_val", c_f32p),
        ("csc_col_ptr", c_u32p), ("csc_row_idx", c_u32p), ("csc_val", c_f32p),
        ("nnz_test", ctypes.c_int64),
        ("test_row", c_u32p), ("test_col", c_u32p), ("test_val", c_f32p),
    ]


class Opts(ctypes.Structure):
    _fields_ = [
        ("k", ctypes.c_uint32), ("lambda_", ctypes.c_float), ("maxiter", ctypes.c_int32),
        ("maxinneriter", ctypes.c_int32), ("version", ctypes.c_int32), ("residual", ctypes.c_int32),
        ("reduce", ctypes.c_int32), ("rmse_each_outer", ctypes.c_int32), ("use_graph", ctypes.c_int32),
        ("threads_per_block", ctypes.c_int32), ("device", ctypes.c_int32), ("verbose", ctypes.c_int32),
        ("relabel", ctypes.c_int32), ("autotune", ctypes.c_int32), ("layout", ctypes.c_int32),
    ]


class BinCfg(ctypes.Structure):
    _fields_ = [("thread_max", ctypes.c_uint32), ("group_max", ctypes.c_uint32), ("warp_max", ctypes.c_uint32),
                ("cta_max", ctypes.c_uint32), ("chunk", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [
        ("train_ms", ctypes.c_double), ("sweep_csc_ms", ctypes.c_double), ("sweep_csr_ms", ctypes.c_double),
        ("rmse_ms", ctypes.c_double), ("refresh_ms", ctypes.c_double), ("launches", ctypes.c_int64),
        ("sweep_csc_launches", ctypes.c_int64), ("sweep_csr_launches", ctypes.c_int64),
        ("rmse_launches", ctypes.c_int64), ("refresh_launches", ctypes.c_int64), ("updates", ctypes.c_int64),
        ("bytes_per_update", ctypes.c_double), ("drift_rms", ctypes.c_double), ("nonfinite", ctypes.c_int64),
    ]


class SynthSpec(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int64), ("n", ctypes.c_int64), ("nnz_total", ctypes.c_int64), ("nnz_test", ctypes.c_int64),
        ("test_fraction", ctypes.c_double), ("row_mode", ctypes.c_int32), ("row_alpha", ctypes.c_double),
        ("row_min", ctypes.c_int64), ("row_max", ctypes.c_int64), ("col_mode", ctypes.c_int32),
        ("col_alpha", ctypes.c_double), ("col_cap", ctypes.c_int64), ("col_beta_a", ctypes.c_double),
        ("col_beta_b", ctypes.c_double), ("col_min_one", ctypes.c_int32), ("rank", ctypes.c_int32),
        ("factor_std", ctypes.c_double), ("planted_std", ctypes.c_double), ("offset", ctypes.c_double),
        ("noise_std", ctypes.c_double), ("quantum", ctypes.c_double), ("vmin", ctypes.c_double),
        ("vmax", ctypes.c_double), ("seed", ctypes.c_uint64),
    ]


OUTER_CB = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p)

# every symbol declared in include/cdmf_cuda.h and include/cdmf_synth.h
EXPORTS = {
    "cdmf_opts_default": (None, [ctypes.POINTER(Opts)]),
    "cdmf_cuda_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "cdmf_cuda_version": (ctypes.c_int, []),
    "cdmf_cuda_train": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(Opts), c_f32p, c_f32p, c_f64p,
                                       OUTER_CB, ctypes.c_void_p]),
    "cdmf_cuda_rmse_coo": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_int64, ctypes.c_int64, c_f32p, c_f32p,
                                          ctypes.c_int64, c_u32p, c_u32p, c_f64p, ctypes.c_int, c_f64p, c_i64p]),
    "cdmf_cuda_rmse_coo_noalloc": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p, c_f64p, c_i64p]),
    "cdmf_cuda_compress": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, c_u32p, c_u32p, c_f64p,
                                          ctypes.c_int, c_u32p, c_u32p, c_f32p, c_u32p, c_u32p, c_f32p, c_i64p]),
    "cdmf_spmv_create": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cdmf_spmv_destroy": (None, [ctypes.c_void_p]),
    "cdmf_spmv_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "cdmf_spmv_input_csr": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "cdmf_spmv_as_csr5": (ctypes.c_int, [ctypes.c_void_p]),
    "cdmf_spmv_as_csr": (ctypes.c_int, [ctypes.c_void_p]),
    "cdmf_spmv_set_x": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cdmf_spmv_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, c_f64p]),
    "cdmf_cuda_create": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(Opts),
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "cdmf_cuda_destroy": (None, [ctypes.c_void_p]),
    "cdmf_cuda_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "cdmf_cuda_set_factors": (ctypes.c_int, [ctypes.c_void_p, c_f32p, c_f32p]),
    "cdmf_cuda_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_f64p]),
    "cdmf_cuda_get_factors": (ctypes.c_int, [ctypes.c_void_p, c_f32p, c_f32p]),
    "cdmf_cuda_rmse": (ctypes.c_int, [ctypes.c_void_p, c_f64p]),
    "cdmf_cuda_objective": (ctypes.c_int, [ctypes.c_void_p, c_f64p, c_f64p, c_f64p]),
    "cdmf_cuda_get_state": (ctypes.c_int, [ctypes.c_void_p, c_f32p, c_f32p, c_f32p, c_f32p,
                                           ctypes.POINTER(ctypes.c_int)]),
    "cdmf_cuda_set_state": (ctypes.c_int, [ctypes.c_void_p, c_f32p, c_f32p, c_f32p, c_f32p, ctypes.c_int]),
    "cdmf_cuda_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cdmf_cuda_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "cdmf_cuda_get_bincfg": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BinCfg)]),
    "cdmf_cuda_set_bincfg": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BinCfg)]),
    "cdmf_cuda_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BinCfg), c_f64p]),
    "cdmf_cuda_host_alloc": (ctypes.c_void_p, [ctypes.c_uint64]),
    "cdmf_cuda_host_free": (None, [ctypes.c_void_p]),
    "cdmf_cuda_bins": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_i64p, c_i64p]),
    "cdmf_cuda_batch_create": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(Opts), ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_void_p)]),
    "cdmf_cuda_batch_destroy": (None, [ctypes.c_void_p]),
    "cdmf_cuda_batch_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "cdmf_cuda_batch_set_factors": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(c_f32p)]),
    "cdmf_cuda_batch_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_f64p]),
    "cdmf_cuda_batch_run_sequential": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_f64p, c_f64p]),
    "cdmf_cuda_batch_get_factors": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(c_f32p), ctypes.POINTER(c_f32p)]),
    "cdmf_cuda_batch_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "cdmf_synth_create": (ctypes.c_int, [ctypes.POINTER(SynthSpec), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cdmf_synth_info": (ctypes.c_int, [ctypes.c_void_p, c_i64p, c_i64p, c_i64p, c_i64p]),
    "cdmf_synth_copy": (ctypes.c_int, [ctypes.c_void_p, c_u32p, c_u32p, c_f32p, c_u32p, c_u32p, c_f32p,
                                       c_u32p, c_u32p, c_f32p]),
    "cdmf_synth_destroy": (None, [ctypes.c_void_p]),
    "cdmf_initial_col": (None, [c_f32p, ctypes.c_uint32, ctypes.c_uint32]),
    "cdmf_csr_to_csc": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, c_u32p, c_u32p, c_f32p,
                                       c_u32p, c_u32p, c_f32p, c_u32p]),
}

_LIB = None


class CdmfError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        name = STATUS.get(status, str(status))
        super().__init__(f"{where}: {name}" + (f" ({detail})" if detail else ""))


def load():
    """Returns the loaded library; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.environ.get("CDMF_LIB", _build.LIB)
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status, where, handle=None):
    if status != CDMF_OK:
        detail = ""
        if handle is not None:
            msg = load().cdmf_cuda_last_error(handle)
            detail = msg.decode() if msg else ""
        raise CdmfError(status, where, detail)


def ptr(a, ctype):
    """Pointer to a contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be contiguous"
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def pinned_empty(shape, dtype):
    """numpy array in page-locked host memory (freed with the returned owner)."""
    import numpy as np
    dtype = np.dtype(dtype)
    count = int(np.prod(shape))
    lib = load()
    p = lib.cdmf_cuda_host_alloc(max(1, count * dtype.itemsize))
    if not p:
        raise MemoryError("cdmf_cuda_host_alloc failed")
    buf = (ctypes.c_char * max(1, count * dtype.itemsize)).from_address(p)
    arr = np.frombuffer(buf, dtype=dtype, count=count).reshape(shape)
    owner = _Pinned(p)
    return arr, owner


class _Pinned:
    def __init__(self, p):
        self.p = p

    def __del__(self):
        if self.p and _LIB is not None:
            _LIB.cdmf_cuda_host_free(self.p)
            self.p = None
