"""Pins the oracle (oracle/gga_oracle.c) and the generators to the REFERENCE.

tests/golden/* were produced by the reference's own graph.h/myutils.h
(oracle/_ref, see tests/golden/make_golden.py).  Here the C restatement must
reproduce every recorded output bit for bit: serial BFS/SSSP distances
(graph.h:115-184), NodeSplit arrays (graph.h:415-522), the split rules
(graph.h:338-414), verifysolution counts (myutils.h:1-18) and the Ary2File
text (myutils.h:51-62).  The generated graphs must also hash to the recorded
CSR digests, which pins the generators across machines.
"""
from __future__ import annotations

import hashlib
import os
import tempfile

import numpy as np
import pytest

import oracle
from conftest import build_golden_graph
from _util import csr_digest, digest, expand_to_split


def _graphs(golden):
    meta, arrays = golden
    return [(name, e, arrays) for name, e in sorted(meta["graphs"].items())]


def test_golden_has_cases(golden):
    meta, _ = golden
    assert len(meta["graphs"]) >= 7
    crashes = [k for e in meta["graphs"].values() for k, s in e["split"].items() if s.get("crash")]
    assert crashes, "the reference's divide-by-zero cases must be recorded"


def test_generated_graphs_match_recorded_digest(golden):
    for name, e, arrays in _graphs(golden):
        g = build_golden_graph(name, e, arrays)
        off, col, wt = g.csr()
        assert csr_digest(off, col, wt) == e["csr_sha256"], name
        assert (len(off) - 1, len(col)) == (e["n"], e["m"]), name


def test_oracle_serial_matches_reference(golden):
    for name, e, arrays in _graphs(golden):
        g = build_golden_graph(name, e, arrays)
        og = oracle.OracleGraph.from_csr(*g.csr())
        assert og.max_degree() == e["maxdeg"]
        for key, rec in e["dist"].items():
            algo, src = key.split("/")
            d, _ = og.serial(algo, int(src))
            assert digest(d) == rec["sha256"], (name, key)
            np.testing.assert_array_equal(d, arrays[f"{name}/dist/{key}"])
            finite = d[d < oracle.INF]
            assert (finite.max() if len(finite) else 0) == rec["max_dist"] or rec["max_dist"] == 0


def test_oracle_split_matches_reference(golden):
    for name, e, arrays in _graphs(golden):
        g = build_golden_graph(name, e, arrays)
        off, col, wt = g.csr()
        for key, rec in e["split"].items():
            level, buckets = map(int, key.split("/"))
            og = oracle.OracleGraph.from_csr(off, col, wt)
            rc = og.node_split(level, buckets)
            if rec.get("crash"):
                assert rc == 4, (name, key)  # the reference raised SIGFPE here
                continue
            assert rc == 0, (name, key)
            a = og.arrays()
            d = og.dims()
            assert d["mda"] == rec["mda"] and d["nnodes"] == rec["nnodes"], (name, key)
            for k in ("psrc", "noutgoing", "childCount", "IsParent", "parentNode"):
                assert digest(a[k]) == rec[f"{k}_sha256"], (name, key, k)
            assert digest(a["edgessrcdst"][1:]) == rec["edgessrcdst_sha256"], (name, key)


def test_oracle_split_rules_and_verify(golden):
    for name, e, arrays in _graphs(golden):
        g = build_golden_graph(name, e, arrays)
        off, col, wt = g.csr()
        for key, rec in e["split"].items():
            level, buckets = map(int, key.split("/"))
            og = oracle.OracleGraph.from_csr(off, col, wt)
            rc, mda, cnt = og.size_after_split(level, buckets)
            if rec.get("crash"):
                assert rc == 4
                continue
            assert (mda, cnt) == (rec["mda"], rec["nnodes"])
            og.node_split(level, buckets)
            a = og.arrays()
            src = rec["src"]
            dist = arrays[f"{name}/dist/sssp/{src}"]
            assert og.verify("sssp", expand_to_split(dist, a["parentNode"])) == rec["nerr_sssp"] == 0


def test_oracle_child_index_and_init(golden):
    """bfs_sssp.cu:256-283 child lists and :301-318 dist initialisation."""
    meta, arrays = golden
    e = meta["graphs"]["hub40_oddm"]
    g = build_golden_graph("hub40_oddm", e, arrays)
    og = oracle.OracleGraph.from_csr(*g.csr())
    og.node_split(3, 10)
    a = og.arrays()
    idx, cnt = og.child_index()
    np.testing.assert_array_equal(idx, np.nonzero(a["childCount"])[0])
    np.testing.assert_array_equal(cnt, a["childCount"][idx])
    hd = og.init_dist(0)
    first_parent = 0
    assert hd[first_parent] == 0
    assert (hd[1:1 + a["childCount"][0]] == 0).all()
    assert (hd[1 + a["childCount"][0]:] == oracle.INF).all()


def test_oracle_ary2file_matches_reference(golden):
    meta, arrays = golden
    for name in ("hub40_oddm", "rmat10", "grid64"):
        e = meta["graphs"][name]
        g = build_golden_graph(name, e, arrays)
        og = oracle.OracleGraph.from_csr(*g.csr())
        for key, rec in e["dist"].items():
            d = arrays[f"{name}/dist/{key}"]
            with tempfile.TemporaryDirectory() as t:
                p = os.path.join(t, "a.txt")
                a = og.arrays()
                oracle.load().oracle_ary2file(p.encode(), oracle._p(np.ascontiguousarray(d, np.uint32)),
                                              oracle._p(a["IsParent"]), len(d))
                assert hashlib.sha256(open(p, "rb").read()).hexdigest() == rec["ary_txt_sha256"]


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build exists only on the development host")
def test_reference_build_agrees_with_oracle_on_fresh_graph():
    """Direct cross-check against oracle/_ref on a graph not in the fixtures."""
    import gpugraphalgo_gb300 as gga

    g = gga.Graph.rmat(11, 16, seed=99)
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "g.gr")
        g.save_gr(p)
        og = oracle.OracleGraph.from_csr(*g.csr())
        for algo in ("bfs", "sssp"):
            r = oracle.run_reference(p, algo, -1, 10, 3)
            assert r["returncode"] == 0
            np.testing.assert_array_equal(r["dist"], og.serial(algo, 3)[0])


def test_oracle_shortest_matches_reference(golden):
    """The second exact method (FIFO BFS / Dijkstra) that checks the graphs too
    deep for the reference's sweeps gives the reference's own distances on
    every golden graph and source."""
    for name, e, arrays in _graphs(golden):
        g = build_golden_graph(name, e, arrays)
        og = oracle.OracleGraph.from_csr(*g.csr())
        for key in e["dist"]:
            algo, src = key.split("/")
            np.testing.assert_array_equal(og.shortest(algo, int(src)), arrays[f"{name}/dist/{key}"],
                                          err_msg=f"{name} {key}")


def test_oracle_generators_build_the_library_graphs(golden):
    """oracle.OracleGraph.gen_rmat / gen_grid (the benchmark's CPU legs, which
    do not load the GPU library) build the same graphs as gga.Graph."""
    meta, arrays = golden
    for name, e in sorted(meta["graphs"].items()):
        p = e.get("params")
        if e["kind"] == "rmat":
            og = oracle.OracleGraph.gen_rmat(p["scale"], p["edge_factor"], seed=p["seed"], wmin=p["wmin"],
                                             wmax=p["wmax"])
        elif e["kind"] == "grid":
            og = oracle.OracleGraph.gen_grid(p["width"], p["height"], p["del_prob"], p["longrange_frac"],
                                             seed=p["seed"], wmin=p["wmin"], wmax=p["wmax"])
        else:
            continue
        a = og.arrays()
        off = np.concatenate([a["psrc"][:-1] - 1, [len(a["edgessrcdst"]) - 1]]).astype(np.uint32)
        assert csr_digest(off, a["edgessrcdst"][1:], a["edgessrcwt"][1:]) == e["csr_sha256"], name
        np.testing.assert_array_equal(og.degrees(), np.diff(off.astype(np.int64)))
