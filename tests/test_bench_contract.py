"""bench.py's reference arm on the CPU: the one JSON line a harness reads,
from one process and from two gloo ranks (rank 0 alone runs and prints).
The arm times the oracle's restatement of the reference's serial
findSerialBFS / findSerialSSSP (graph.h:115-184) on host threads."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--scale", "10", "--sources", "4", "--steps", "2", "--warmup", "3"]


def _json_lines(out: str):
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def _check_line(d, gpus):
    sys.path.insert(0, ROOT)
    import bench

    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert (d["steps"], d["warmup"], d["n_gpus"]) == (2, 3, gpus)
    assert d["config"]["workload"] == "rmat10_ef16_seed2_4src_bfs+sssp"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert cb["cores"] == (os.cpu_count() or 1)  # every host thread, each taking the next traversal
    assert set(cb["latency_1core_s"]) == {"bfs", "sssp"} and min(cb["latency_1core_s"].values()) > 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same workload description the GPU arm prints
    assert sorted(d["config"]) == ["edges", "graph", "l2", "maxdeg", "parallelism", "sources", "vertices", "workload"]


def test_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    _check_line(lines[0], 1)


def test_reference_arm_does_not_load_the_gpu_library():
    """The CPU arm builds its graph with the generator compiled into
    liboracle.so; libgga.so is never mapped into the process."""
    code = ("import sys; sys.argv = ['bench.py', *%r]; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('LIBGGA', 'libgga.so' in maps, 'LIBORACLE', 'liboracle.so' in maps)") % (ARGS,)
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "LIBGGA False LIBORACLE True" in r.stdout, r.stdout[-500:]


def test_reference_arm_two_ranks_rank0_prints():
    pytest.importorskip("torch.distributed")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", *ARGS, "--gpus", "2"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    _check_line(lines[0], 2)


def _dist_rank(rank, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": "2", "LOCAL_RANK": str(rank), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    try:
        d.barrier()
        # each replica's own time and units: the job's time is the slowest
        # rank's, its units the sum over ranks
        q.put((rank, d.max(1.5 + rank), d.sum(10.0 * (rank + 1))))
    finally:
        d.close()


def test_replica_timing_reductions_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    pytest.importorskip("torch.distributed")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_dist_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(300)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5, 30.0), (1, 2.5, 30.0)]
