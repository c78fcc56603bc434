"""The multi-process path of bench.py on CPU (gloo, world size 2): the
barrier and the max-over-ranks of the timings that bracket every timed
region, and the replica arithmetic of the whole-job value.  The engine's
path does not shard (one independent replica per GPU), so nothing else
crosses ranks."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(ws, rank)
    d.barrier()
    t_ms = d.max(10.0 + 5.0 * rank)          # rank 1 is the slower replica
    d.barrier()
    d.close()
    # whole-job value of the replicas: every rank's updates over the slowest time
    q.put((rank, t_ms, ws * 640 / (t_ms / 1e3)))


def test_two_rank_barrier_max_and_value():
    torch_mp = pytest.importorskip("torch.multiprocessing")
    ctx = torch_mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=30) for _ in range(2))
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(abs(r[2] - 2 * 640 / 0.015) < 1e-6 for r in res)


def test_reference_arm_other_ranks_do_no_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, timeout=120, env=env)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_reference_arm_contract_line():
    """Rank 0 of the reference arm (the oracle port of cdmf_ref on the host
    cores, whole outer iterations of the Netflix-shaped workload; k = 4 here
    to keep the test short) prints one JSON line with the keys the benchmark
    contract asks for and the GPU arm's config, and never loads the engine
    library."""
    import json
    env = dict(os.environ, RANK="0", LOCAL_RANK="0", WORLD_SIZE="1", MASTER_ADDR="127.0.0.1")
    script = ("import runpy, sys\n"
              "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', '--k', '4']\n"
              "runpy.run_path(%r, run_name='__main__')\n"
              "print('maps', open('/proc/self/maps').read().count('libcdmf_cuda'))\n" % os.path.join(ROOT, "bench.py"))
    p = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 2 and lines[1] == "maps 0", p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "rank-one updates/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert "480189x17770" in d["config"]["workload"] and "k=4" in d["config"]["workload"]
    assert set(d["config"]) == {"workload", "step", "l2", "parallelism"}
    assert 0.5 < d["test_rmse"] < 2.0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_e2e_phase_times_are_captured():
    """The e2e leg records the engine's phase times per call: the lines the
    engine prints on stderr (fd 2) with verbose options are captured around
    the call and parsed, and stderr is restored afterwards."""
    sys.path.insert(0, ROOT)
    import bench

    def fake_call():
        os.write(2, b"[cdmf] create: checks            3.7 ms\n[cdmf] create: relabel (GPU)     21.4 ms\n"
                    b"[cdmf] train: create           31.4 ms\n[cdmf] train: outer loop      578.3 ms\n"
                    b"unrelated line\n")
        return 7

    out, phases = bench.with_phase_times(fake_call)
    assert out == 7
    assert phases == {"create/checks": 3.7, "create/relabel (GPU)": 21.4, "create": 31.4, "outer loop": 578.3}
    os.write(2, b"")   # fd 2 is usable again
