"""The drop-in CLI (gpugraphalgo_gb300/bin/gga_cli and its flavour
links na_/n_/da_/d_ x bfs/sssp, named like the reference's genexe outputs):
argv of bfs_sssp.cu:149-184, the Ary2File dump (myutils.h:51-62) and the
17-column result.vi row (writeResult, myutils.h:86-113)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "gpugraphalgo_gb300", "bin")
FLAVOURS = ["na_bfs", "na_sssp", "n_bfs", "n_sssp", "da_bfs", "da_sssp", "d_bfs", "d_sssp", "gga_bfs", "gga_sssp"]


def _run(name, *args, cwd=None):
    return subprocess.run([os.path.join(BIN, name), *args], capture_output=True, text=True, cwd=cwd, timeout=300)


def test_cli_built_with_every_flavour():
    for f in FLAVOURS + ["gga_cli"]:
        assert os.access(os.path.join(BIN, f), os.X_OK), f


@pytest.mark.parametrize("name,algo", [("na_sssp", "SSSP"), ("n_bfs", "BFS"), ("gga_cli", "BFS")])
def test_cli_usage_without_graph(name, algo):
    r = _run(name)
    assert r.returncode == 1
    assert r.stdout.splitlines()[0] == algo
    assert "Usage:" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("flavour", FLAVOURS)
@pytest.mark.parametrize("args", [[], ["0"], ["-1", "10"], ["4"]])
def test_cli_matches_oracle_and_writes_result_row(tmp_path, flavour, args):
    g = gga.Graph.rmat(11, 8, seed=31)
    gr = str(tmp_path / "rmat11.gr")
    g.save_gr(gr)
    sssp = "sssp" in flavour
    out = tmp_path / "dist.txt"
    argv = [gr] + args
    if args in ([], ["0"], ["4"]):
        argv = [gr, args[0] if args else "0", str(out)]
    r = _run(flavour, *argv, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "verifying: no of errors = 0." in r.stdout
    want = oracle.serial_distances(*g.csr(), "sssp" if sssp else "bfs", 0)
    if out.exists():
        got = np.loadtxt(out, dtype=np.uint64).astype(np.uint32)
        np.testing.assert_array_equal(got, want)
    rows = (tmp_path / "result.vi").read_text().strip().splitlines()
    f = rows[-1].split(",")
    assert len(f) == 17
    assert f[1] == ("SSSP" if sssp else "BFS") and f[2] == "rmat11.gr"
    info = g.info()
    assert int(f[4]) == info["nodes_orig"] and int(f[5]) == info["nedges"] and int(f[9]) == info["maxdeg"]
    assert int(f[12]) >= 1  # iterations


@pytest.mark.gpu
def test_split_sweep_writes_one_row_per_point(tmp_path):
    """The split-level sweep (the reference's mysc driver, levels then the
    histogram rule per bucket count) in one process: 17-column rows, MDA per
    level = ceil(maxdeg / level) as getSizeafterLoadBalance computes it
    (graph.h:386-397)."""
    from gpugraphalgo_gb300 import sweep

    g = gga.Graph.rmat(12, 8, seed=33)
    gr = str(tmp_path / "r12.gr")
    g.save_gr(gr)
    out = str(tmp_path / "result.vi")
    rc = sweep.main([gr, "--flavours", "na,gga,d", "--algos", "bfs,sssp", "--levels", "1-3", "--buckets", "2,10",
                     "--out", out])
    assert rc == 0
    rows = [r.split(",") for r in open(out).read().strip().splitlines()]
    assert len(rows) == 3 * 2 * 5 and all(len(r) == 17 for r in rows)
    maxdeg = g.info()["maxdeg"]
    for r in rows:
        level = int(r[10])
        if r[0].startswith(("na_", "gga_")) and level < 2**31:
            assert int(r[11]) == -(-maxdeg // level)
        assert float(r[14]) > 0 and int(r[12]) >= 1


def test_sweep_points_follow_the_reference_driver():
    """mysc:20-51 runs levels 1..40 (no bucket argument, so the default 10)
    and then the histogram rule (level -1) with buckets 2, 5, 10, 15."""
    from gpugraphalgo_gb300 import sweep

    pts = sweep.sweep_points(sweep._levels("1-40"), [2, 5, 10, 15])
    assert pts == [(i, 10) for i in range(1, 41)] + [(-1, 2), (-1, 5), (-1, 10), (-1, 15)]
    assert sweep._levels("1-3,7,9-10") == [1, 2, 3, 7, 9, 10]
    assert sweep._levels("-1") == [-1]
    assert sweep.VARIANT == {"na": "topo_atomic", "n": "topo_plain", "da": "cdp_atomic", "d": "cdp_plain",
                             "gga": "frontier"}


@pytest.mark.parametrize("exe", FLAVOURS)
def test_cli_usage_without_arguments(exe):
    """The algorithm line (bfs_sssp.cu:106-111), then the usage line and exit
    status 1 when no graph is given (bfs_sssp.cu:149-152).  The reference
    prints its device lines in between; this CLI reaches the usage check
    without touching a device."""
    r = subprocess.run([os.path.join(BIN, exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    lines = r.stdout.splitlines()
    assert lines[0] == ("SSSP" if "sssp" in exe else "BFS")
    assert lines[1].startswith("Usage: ") and lines[1].endswith(" <file>")


def test_cli_algorithm_override():
    r = subprocess.run([os.path.join(BIN, "d_sssp")], capture_output=True, text=True, timeout=60,
                       env={**os.environ, "GGA_ALGO": "bfs"})
    assert r.returncode == 1 and r.stdout.splitlines()[0] == "BFS"


def test_conv_log_format_matches_reference_lines():
    """conv.vi lines as convergence.h:81-159 writes them: a header after
    three blank lines and an 88-dash rule, `Iteration:` with the iteration
    left-aligned in 3 columns and the norm printed like a C++ stream double,
    and the footer."""
    from gpugraphalgo_gb300 import conv

    assert conv.header(-1, 1234, "rmat20.gr", "SSSP") == "\n\n\n" + "-" * 88 + "\nDist_Level_-1_MaxDeg_1234_rmat20.gr_SSSP\n"
    assert conv.iteration_line(1, 123456.789, 42) == "Iteration:1   = 123457(42)\n"
    assert conv.iteration_line(12, 0.0, 0) == "Iteration:12  = 0(0)\n"
    assert conv.iteration_line(1234, 1.5e-7, 3) == "Iteration:1234 = 1.5e-07(3)\n"
    assert conv.iteration_line(7, 65536.0 ** 2, 1) == "Iteration:7   = 4.29497e+09(1)\n"
    assert conv.footer(17, 254) == "Total Iteration : 17     Max Dist : 254\n" + "-" * 88 + "\n"


@pytest.mark.gpu
@pytest.mark.parametrize("flavour", ["na", "d"])
def test_conv_tool_writes_a_converging_log(tmp_path, flavour):
    g = gga.Graph.rmat(10, 8, seed=3)
    gr = str(tmp_path / "rmat10.gr")
    g.save_gr(gr)
    from gpugraphalgo_gb300 import conv

    out = tmp_path / "conv.vi"
    assert conv.main([gr, "--flavour", flavour, "--algo", "sssp", "--level", "2", "--out", str(out)]) == 0
    lines = out.read_text().split("\n")
    assert lines[:3] == ["", "", ""] and lines[3] == "-" * 88
    assert lines[4] == f"Dist_Level_2_MaxDeg_{g.info()['maxdeg']}_rmat10.gr_SSSP"
    its = [x for x in lines if x.startswith("Iteration:")]
    assert its and its[-1].endswith(" = 0(0)")
    want = oracle.serial_distances(*g.csr(), "sssp", 0)
    assert f"Total Iteration : {len(its)}     Max Dist : {int(want[want < gga.INFINITY].max())}" in lines
