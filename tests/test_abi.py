"""The C ABI library: loads, exports every declared entry point, rejects bad
input on the host (no GPU work in these tests)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden
from cdmf_gb300 import _lib, engine


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for line in text.split(";"):
            line = " ".join(line.split())
            if line.startswith("typedef") or "#define" in line:
                continue
            mt = re.search(r"\b(cdmf_\w+)\s*\(", line)
            if mt:
                names.add(mt.group(1))
    return names


def test_library_exports_declared_symbols():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.EXPORTS, n


def test_strerror_and_defaults():
    lib = _lib.load()
    assert lib.cdmf_cuda_strerror(0) == b"ok"
    assert lib.cdmf_cuda_strerror(-1).startswith(b"invalid")
    o = _lib.Opts()
    lib.cdmf_opts_default(ctypes.byref(o))
    assert (o.k, o.maxiter, o.maxinneriter) == (10, 5, 5) and abs(o.lambda_ - 0.1) < 1e-7


def _create(R, **kw):
    o = engine.make_opts(kw.pop("k", 4), kw.pop("lambda_", 0.1), **kw)
    p = engine._problem(R)
    h = ctypes.c_void_p()
    st = _lib.load().cdmf_cuda_create(ctypes.byref(p), ctypes.byref(o), ctypes.byref(h))
    if st == 0:
        _lib.load().cdmf_cuda_destroy(h)
    return st


def test_create_rejects_bad_structures():
    R, _ = load_golden("simple")
    bad = load_golden("simple")[0]
    bad.csr_idx = R.csr_idx.copy()
    bad.csr_idx[3] = 99                                   # column out of range
    assert _create(bad) == -1
    bad = load_golden("simple")[0]
    bad.csc_ptr = R.csc_ptr.copy()
    bad.csc_ptr[2], bad.csc_ptr[3] = bad.csc_ptr[3], bad.csc_ptr[2]   # not monotone
    assert _create(bad) == -1
    bad = load_golden("simple")[0]
    bad.te_row = R.te_row.copy()
    bad.te_row[0] = 6                                     # test row out of range
    assert _create(bad) == -1
    bad = load_golden("simple")[0]
    bad.te_col = R.te_col.copy()
    bad.te_col[-1] = R.n                                  # test column out of range
    assert _create(bad) == -1
    bad = load_golden("simple")[0]
    bad.csr_idx = R.csr_idx.copy()
    bad.csr_idx[-1] = R.n                                 # last column index one past the end
    assert _create(bad) == -1
    assert _create(R, k=0) == -1
    assert _create(R, lambda_=-1.0) == -1
    assert _create(R, residual=5) == -1


def test_null_arguments():
    lib = _lib.load()
    assert lib.cdmf_cuda_create(None, None, None) == -1
    assert lib.cdmf_cuda_run(None, 1, None) == -1
    assert lib.cdmf_cuda_get_factors(None, None, None) == -1
    lib.cdmf_cuda_destroy(None)


def test_new_entry_points_reject_bad_arguments_before_device_work():
    """Argument checks of the format builder, the dual SpMV handle and the
    objective monitor happen on the host, before any device is touched."""
    lib = _lib.load()
    n = ctypes.c_int64()
    U, F, D = ctypes.c_uint32, ctypes.c_float, ctypes.c_double
    z = np.zeros(4, np.uint32)
    zf = np.zeros(4, np.float32)
    zd = np.zeros(4, np.float64)
    p = _lib.ptr
    # negative sizes, missing outputs
    assert lib.cdmf_cuda_compress(-1, 4, 0, None, None, None, 0, p(z, U), None, None, p(z, U), None, None,
                                  ctypes.byref(n)) == -1
    assert lib.cdmf_cuda_compress(3, 3, 2, p(z, U), p(z, U), p(zd, D), 0, None, p(z, U), p(zf, F), p(z, U),
                                  p(z, U), p(zf, F), ctypes.byref(n)) == -1
    # nonzeros with an empty dimension
    assert lib.cdmf_cuda_compress(0, 3, 2, p(z, U), p(z, U), p(zd, D), 0, p(z, U), p(z, U), p(zf, F), p(z, U),
                                  p(z, U), p(zf, F), ctypes.byref(n)) == -1
    # beyond the 32-bit structure limits
    assert lib.cdmf_cuda_compress(1 << 32, 3, 2, p(z, U), p(z, U), p(zd, D), 0, p(z, U), p(z, U), p(zf, F),
                                  p(z, U), p(z, U), p(zf, F), ctypes.byref(n)) == -8
    h = ctypes.c_void_p()
    assert lib.cdmf_spmv_create(-1, 4, 0, ctypes.byref(h)) == -1
    assert lib.cdmf_spmv_create(1 << 33, 4, 0, ctypes.byref(h)) == -8
    assert lib.cdmf_spmv_create(4, 4, 0, None) == -1
    for fn, args in (("cdmf_spmv_input_csr", (None, 0, None, None, None)), ("cdmf_spmv_as_csr5", (None,)),
                     ("cdmf_spmv_as_csr", (None,)), ("cdmf_spmv_set_x", (None, None)),
                     ("cdmf_spmv_run", (None, 1.0, None, None, None)),
                     ("cdmf_cuda_objective", (None, None, None, None))):
        assert getattr(lib, fn)(*args) == -1, fn
    lib.cdmf_spmv_destroy(None)
    assert lib.cdmf_spmv_last_error(None) == b""


def test_anonymouslib_header_compiles_and_links(tmp_path):
    """The C++ face of the dual SpMV handle: a caller written against the
    reference's anonymouslibHandle calls compiles and links against the library."""
    import subprocess
    from cdmf_gb300 import _build
    src = tmp_path / "use.cpp"
    src.write_text(
        "#include <cdmf_anonymouslib.hpp>\n"
        "int main() {\n"
        "  cdmf::anonymouslibHandle<int, unsigned int, float> A(4, 5);\n"
        "  double t = 0; A.setSigma(4); (void)A.asCSR5_(&t);\n"
        "  return A.lastError() == nullptr;\n"
        "}\n")
    out = tmp_path / "use"
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(out),
                        "-L", os.path.dirname(_build.LIB), "-lcdmf_cuda", "-Wl,-rpath," + os.path.dirname(_build.LIB)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_shim_compiles_and_links(tmp_path):
    """The C++ shim a maintainer of the reference adds as
    src/cdmf_cuda_shim.cpp (tests/native/cdmf_cuda_shim.cpp) compiles against
    include/cdmf_cuda.h and stand-ins for the reference's types
    (tests/native/ref_standins), and links against the library."""
    import subprocess
    from cdmf_gb300 import _build
    native = os.path.join(ROOT, "tests", "native")
    src = tmp_path / "shim_main.cpp"
    src.write_text('#include "%s"\nint main() { return 0; }\n' % os.path.join(native, "cdmf_cuda_shim.cpp"))
    out = tmp_path / "shim"
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(native, "ref_standins"), "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(out), "-L", os.path.dirname(_build.LIB),
                        "-lcdmf_cuda", "-Wl,-rpath," + os.path.dirname(_build.LIB)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
