"""The `cdmf` driver (cdmf_gb300/csrc/cli): the reference's command line
(src/main.cpp, src/tools.cpp:378-465) on the CUDA engine, run on the
reference's own data/simple fixture written in cdmf's directory format."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from cdmf_gb300 import _build, formats

pytestmark = pytest.mark.gpu
ITER = re.compile(r"iteration num (\d+) .*RMSE=([0-9.]+)")


def _run(args, cwd):
    assert os.path.exists(_build.CLI), "build the driver first"
    p = subprocess.run([_build.CLI] + args, capture_output=True, text=True, cwd=cwd, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    return p.stdout


def test_simple_tree_then_reference_order(tmp_path):
    R, z = load_golden("simple")
    d = str(tmp_path / "simple")
    formats.write_dir(d, R)
    out = _run(["-k", "10", "-l", "0.05", "-t", "5", "-T", "3", "-V", "1", "-r", "1", "-p", "1", d], str(tmp_path))
    its = [(int(a), float(b)) for a, b in ITER.findall(out)]
    assert [i for i, _ in its] == [1, 2, 3, 4, 5] * 2, out
    tree, seq = np.array([r for _, r in its[:5]]), np.array([r for _, r in its[5:]])
    # the second run (-r 1) is the reference order: the reference's RMSE to
    # the printed digits; the default tree order within the FP32 budget
    assert np.max(np.abs(seq - z["rmse"])) <= 1e-6, (seq, z["rmse"])
    assert np.max(np.abs(tree - z["rmse"])) <= 1e-5, (tree, z["rmse"])
    assert out.count("Check... PASS!") == 2, out
    assert len(re.findall(r"\[INFO\] Rank-one updates/s: [0-9.]+, outer iterations/s: [0-9.]+", out)) == 2, out
    m = re.search(r"\[INFO\] Test RMSE = ([0-9.]+)", out)
    assert m and abs(float(m.group(1)) - z["rmse"][-1]) <= 1e-5, out


@pytest.mark.parametrize("flags", [["-V", "3"], ["-V", "2", "-residual", "bf16"], ["-V", "1", "-graph", "1"]])
def test_versions_and_modes_run(tmp_path, flags):
    R, z = load_golden("tricky_simple")
    d = str(tmp_path / "tricky")
    formats.write_dir(d, R)
    out = _run(["-k", "10", "-l", "0.05", "-t", "5", "-T", "3"] + flags + [d], str(tmp_path))
    its = [float(b) for _, b in ITER.findall(out)]
    assert len(its) == 5
    # flags reach the engine: 16-bit residual storage moves the RMSE of this
    # 5 x 5, 9-rating toy problem by about 1e-3 (the mixed-precision accuracy bar
    # itself is tested at realistic size in test_parity_gpu.py)
    tol = 5e-3 if "bf16" in flags else 5e-5
    assert abs(its[-1] - z["rmse"][-1]) <= tol, (its, z["rmse"])


def test_bad_directory_fails_cleanly(tmp_path):
    p = subprocess.run([_build.CLI, "-k", "4", str(tmp_path / "missing")], capture_output=True, text=True, timeout=60)
    assert p.returncode != 0
