"""The engine's host code and the `cdmf` driver's loader under
AddressSanitizer and UndefinedBehaviorSanitizer (tests/native/host_harness.cpp,
built here without the CUDA library): the generator, the CSR->CSC
transposition, the degree relabelling and the blocked layouts on several
shapes with their invariants; the loader on a valid directory and on broken
ones (missing, truncated or oversized files, malformed meta), which must fail
with a message and no abort (the reference aborts or exits there,
src/util.h:29-32, src/tools.cpp:276-279); the text-format RMSE path (-p 1)
and the flag parser's long-flag dispatch (src/tools.cpp:390-395)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden
from cdmf_gb300 import formats

CSRC = os.path.join(ROOT, "cdmf_gb300", "csrc")
SOURCES = [os.path.join(ROOT, "tests", "native", "host_harness.cpp"), os.path.join(CSRC, "synth.cpp"),
           os.path.join(CSRC, "relabel.cpp"), os.path.join(CSRC, "blocked.cpp"),
           os.path.join(CSRC, "cli", "loader.cpp")]
SAN_ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:halt_on_error=1:abort_on_error=0",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", OMP_NUM_THREADS="4")
SAN_MARKERS = ("AddressSanitizer", "LeakSanitizer", "runtime error:", "UndefinedBehaviorSanitizer")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("san") / "host_harness")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-fopenmp", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]
    r = subprocess.run(cmd + SOURCES + ["-o", out], capture_output=True, text=True)
    if r.returncode != 0 and ("asan" in r.stderr or "ubsan" in r.stderr):
        pytest.skip("no sanitizer runtime on this host: " + r.stderr.strip().splitlines()[-1])
    assert r.returncode == 0, r.stderr
    return out


def run(harness, *args):
    r = subprocess.run([harness, *map(str, args)], capture_output=True, text=True, env=SAN_ENV, timeout=300)
    report = [m for m in SAN_MARKERS if m in r.stderr]
    assert not report, r.stderr
    return r


def test_host_code_invariants(harness):
    r = run(harness, "host")
    assert r.returncode == 0 and "host ok" in r.stdout, r.stdout + r.stderr


@pytest.fixture()
def data_dir(tmp_path):
    R, _ = load_golden("mini")
    d = tmp_path / "mini"
    formats.write_dir(str(d), R)
    return R, d


def test_loader_reads_a_valid_directory(harness, data_dir):
    R, d = data_dir
    r = run(harness, "load", d)
    assert r.returncode == 0, r.stderr
    got = r.stdout.split("loaded")[1].split()
    assert [int(x) for x in got] == [R.m, R.n, R.nnz, R.nnz_test, R.max_row_nnz, R.max_col_nnz]


def _meta_lines(d):
    return open(os.path.join(d, "meta_modified_all")).read().split("\n")


def _break(d, case):
    lines = _meta_lines(d)
    names = lines[2:11]
    if case == "missing_meta":
        os.remove(os.path.join(d, "meta_modified_all"))
    elif case == "garbage_meta":
        open(os.path.join(d, "meta_modified_all"), "w").write("not a meta file\n")
    elif case == "truncated_indices":
        path = os.path.join(d, names[4])          # CSR column indices
        data = open(path, "rb").read()
        open(path, "wb").write(data[: len(data) // 2])
    elif case == "missing_values":
        os.remove(os.path.join(d, names[8]))      # CSC values
    elif case == "missing_test_file":
        os.remove(os.path.join(d, lines[12]))
    elif case == "huge_dimensions":
        lines[0] = "4000000000 3000000000"
        open(os.path.join(d, "meta_modified_all"), "w").write("\n".join(lines))
    elif case == "nnz_beyond_files":
        lines[1] = str(int(lines[1]) * 1000)
        open(os.path.join(d, "meta_modified_all"), "w").write("\n".join(lines))
    elif case == "negative_rows":
        lines[0] = "-5 " + lines[0].split()[1]
        open(os.path.join(d, "meta_modified_all"), "w").write("\n".join(lines))


@pytest.mark.parametrize("case", ["missing_meta", "garbage_meta", "truncated_indices", "missing_values",
                                  "missing_test_file", "huge_dimensions", "nnz_beyond_files", "negative_rows"])
def test_loader_rejects_broken_directories(harness, data_dir, case):
    _, d = data_dir
    _break(str(d), case)
    r = run(harness, "load", d)
    assert r.returncode == 1, (case, r.stdout, r.stderr)
    assert (r.stdout + r.stderr).strip(), "a message names the problem"


def test_missing_directory(harness, tmp_path):
    r = run(harness, "load", tmp_path / "absent")
    assert r.returncode == 1


def test_text_rmse_path(harness, data_dir):
    """-p 1: the meta / test.txt files parsed and the RMSE of the initial
    factors reported in the reference's format."""
    R, d = data_dir
    k = 4
    r = run(harness, "rmse", d, k)
    assert r.returncode == 0, r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("[INFO] Test RMSE = ")]
    assert len(line) == 1
    got = float(line[0].split("=")[1])
    # initial_col: X[t][i] = 0.1 rand()/RAND_MAX + 0.001 after srand(0), row by row (src/tools.cpp:349-357)
    from cdmf_gb300 import synth
    W = synth.reference_initial_col(k, R.m).astype(np.float64)
    H = synth.reference_initial_col(k, R.n).astype(np.float64)
    pred = np.einsum("ti,ti->i", W[:, R.te_row], H[:, R.te_col])
    expect = float(np.sqrt(np.mean((pred - R.te_val.astype(np.float64)) ** 2)))
    assert abs(got - expect) <= 1e-6 * max(1.0, expect)


def test_text_rmse_meta_larger_than_factors(harness, data_dir):
    _, d = data_dir
    meta = os.path.join(d, "meta")
    lines = open(meta).read().split("\n")
    m, n = lines[0].split()
    lines[0] = f"{int(m) * 10} {n}"
    open(meta, "w").write("\n".join(lines))
    r = run(harness, "rmse", d, 3)
    assert r.returncode == 1


def test_flag_parser_long_flags_before_letters(harness):
    r = run(harness, "args", "-k", 7, "-l", 0.5, "-t", 3, "-T", 2, "-V", 3, "-residual", "bf16", "-reduce",
            "sequential", "-graph", 1, "-p", 1, "-r", 1, "-nBlocks", 9, "-nThreadsPerBlock", 64, "some/dir")
    assert r.returncode == 0, r.stderr
    got = dict(kv.split("=") for kv in r.stdout.strip().splitlines()[-1].split())
    assert got == {"k": "7", "lambda": "0.5", "maxiter": "3", "inner": "2", "version": "3", "residual": "1",
                   "reduce": "1", "graph": "1", "predict": "1", "ref": "1", "dir": "some/dir"}


@pytest.mark.parametrize("argv", [["-x", "1", "d"], ["-k"], ["-residual", "f64", "d"], ["-k", "3"]])
def test_flag_parser_rejects_bad_flags(harness, argv):
    r = run(harness, "args", *argv)
    assert r.returncode != 0 and "Usage: cdmf" in r.stdout


def test_harness_sources_exist():
    for s in SOURCES:
        assert os.path.exists(s), s
    assert shutil.which("g++")
