"""Host-side logic of libgga.so (no GPU): .gr I/O, generators, split rules,
verifier and writers, checked against the reference's recorded outputs."""
from __future__ import annotations

import hashlib
import os
import struct
import tempfile

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle
from conftest import build_golden_graph


def test_gr_roundtrip_and_reference_reader(golden):
    meta, arrays = golden
    for name in ("hub40_oddm", "rmat10", "grid64"):
        g = build_golden_graph(name, meta["graphs"][name], arrays)
        with tempfile.TemporaryDirectory() as t:
            p = os.path.join(t, "g.gr")
            g.save_gr(p)
            h = gga.Graph.readFromGR(p)
            for a, b in zip(g.csr(), h.csr()):
                np.testing.assert_array_equal(a, b)
            # the oracle's reader (readFromGR restated) sees the same graph
            og = oracle.OracleGraph.load_gr(p)
            oa = og.arrays()
            off = g.csr()[0]
            np.testing.assert_array_equal(oa["psrc"][:-1], off[:-1] + 1)
            assert oa["psrc"][-1] == len(g.csr()[1])  # graph.h:254 quirk


def _write_raw(path, header, idx, outs, pad, data):
    with open(path, "wb") as f:
        f.write(struct.pack("<4Q", *header))
        f.write(np.asarray(idx, "<u8").tobytes())
        f.write(np.asarray(outs, "<u4").tobytes())
        if pad:
            f.write(b"\0" * 4)
        f.write(np.asarray(data, "<u4").tobytes())


@pytest.mark.parametrize(
    "case,status",
    [
        ("version", gga.ERR_FORMAT),
        ("truncated", gga.ERR_FORMAT),
        ("bad_dst", gga.ERR_FORMAT),
        ("non_monotone", gga.ERR_FORMAT),
        ("missing", gga.ERR_IO),
    ],
)
def test_gr_malformed(case, status):
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "bad.gr")
        if case == "version":
            _write_raw(p, (2, 4, 2, 1), [1, 1], [1], True, [5])
        elif case == "truncated":
            _write_raw(p, (1, 4, 3, 4), [2, 4, 4], [1, 2, 0, 0], False, [1, 1])
        elif case == "bad_dst":
            _write_raw(p, (1, 4, 2, 1), [1, 1], [7], True, [5])
        elif case == "non_monotone":
            _write_raw(p, (1, 4, 3, 2), [2, 1, 2], [1, 2], False, [1, 1])
        else:
            p = os.path.join(t, "does_not_exist.gr")
        with pytest.raises(gga.GGAError) as e:
            gga.Graph.readFromGR(p)
        assert e.value.status == status


def test_from_csr_validation():
    with pytest.raises(gga.GGAError):
        gga.Graph.from_csr([0, 2, 1], [0, 1])  # decreasing offsets
    with pytest.raises(gga.GGAError):
        gga.Graph.from_csr([0, 1], [5])  # dst out of range
    g = gga.Graph.from_csr([0, 0, 0], [])  # edgeless graph is fine
    assert g.info()["maxdeg"] == 0


def test_host_split_rules_match_reference(golden):
    meta, arrays = golden
    for name, e in meta["graphs"].items():
        g = build_golden_graph(name, e, arrays)
        assert g.getMaxdeg() == e["maxdeg"]
        for key, rec in e["split"].items():
            level, buckets = map(int, key.split("/"))
            if rec.get("crash"):
                with pytest.raises(gga.GGAError) as ex:
                    g.getSizeafterLoadBalance(level, buckets)
                assert ex.value.status == gga.ERR_SPLIT_RULE
                continue
            assert g.getSizeafterLoadBalance(level, buckets) == (rec["mda"], rec["nnodes"]), (name, key)
            if level < 0:
                assert g.getMaxAllowedOutDegree(buckets) == rec["mda"]


def test_verify_counts_like_reference(golden):
    meta, arrays = golden
    for name in ("hub40_oddm", "chain64_zero_w", "rmat10"):
        e = meta["graphs"][name]
        g = build_golden_graph(name, e, arrays)
        og = oracle.OracleGraph.from_csr(*g.csr())
        for key in e["dist"]:
            algo, _ = key.split("/")
            d = arrays[f"{name}/dist/{key}"].copy()
            assert g.verifysolution(d, algo) == 0
            rng = np.random.default_rng(len(d))
            bad = rng.choice(len(d), size=max(1, len(d) // 7), replace=False)
            d[bad] = np.minimum(d[bad], 10**9) + 3
            assert g.verifysolution(d, algo) == og.verify(algo, d)


def test_ary2file_text_matches_reference(golden):
    meta, arrays = golden
    for name in ("hub40_oddm", "grid64", "c1_rmat14"):
        e = meta["graphs"][name]
        g = build_golden_graph(name, e, arrays)
        for key, rec in e["dist"].items():
            with tempfile.TemporaryDirectory() as t:
                p = os.path.join(t, "d.txt")
                g.Ary2File(p, arrays[f"{name}/dist/{key}"])
                assert hashlib.sha256(open(p, "rb").read()).hexdigest() == rec["ary_txt_sha256"]


def test_write_result_row_format():
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "result.vi")
        kw = dict(exename="./na_bfs.exe", algo="BFS", graphfile="rmat20.gr", bucket_size=0, nnode=1048576,
                  nedge=8259994, ns_nnode=1048576, ns_nedge=8259994, extranode=0, maxdeg=1181, splitlevel=1,
                  max_edges_allowed=1181, iterations=8, runtime=100, time=104.660957, ktime=104.321053, sktime=0.0)
        gga.writeResult(p, **kw)
        gga.writeResult(p, **kw)
        lines = open(p).read().splitlines()
        # the row shape of the reference's own result.vi (Kepler_BFS_SSSP/result.vi:241)
        assert lines[0] == "./na_bfs.exe,BFS,rmat20.gr,0,1048576,8259994,1048576,8259994,0,1181,1,1181,8,100,104.660957,104.321053,0.000000"
        assert len(lines) == 2


def test_rmat_generator_properties():
    g = gga.Graph.rmat(12, 8, seed=3)
    off, col, wt = g.csr()
    n = len(off) - 1
    src = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
    assert (src != col).all(), "self loops removed"
    key = src.astype(np.int64) * n + col
    assert len(np.unique(key)) == len(key), "duplicates removed"
    for u in range(0, n, 97):
        assert np.all(np.diff(col[off[u]:off[u + 1]].astype(np.int64)) > 0), "adjacency sorted"
    rev = col.astype(np.int64) * n + src
    order = np.argsort(key)
    pos = np.searchsorted(key[order], rev)
    assert np.array_equal(key[order][pos], rev), "symmetric"
    assert np.array_equal(wt[order][pos], wt), "same weight both ways"
    info = g.info()
    assert info["symmetric"] == 1 and info["wsymmetric"] == 1, "known symmetric with equal weights"
    assert gga.Graph.from_csr(off, col, wt).info()["wsymmetric"] == 0, "user arrays: checked on the device"
    assert wt.min() >= 1 and wt.max() <= 255
    deg = np.diff(off.astype(np.int64))
    assert deg.max() > 20 * deg.mean(), "skewed degrees"
    h = gga.Graph.rmat(12, 8, seed=3)
    for a, b in zip(g.csr(), h.csr()):
        np.testing.assert_array_equal(a, b)


def test_grid_generator_properties():
    g = gga.Graph.grid(100, 80, 0.05, 0.001, seed=3, wmin=1, wmax=1000)
    off, col, wt = g.csr()
    n = len(off) - 1
    assert n == 8000
    deg = np.diff(off.astype(np.int64))
    assert deg.max() <= 6
    grid_edges = 2 * (100 * 79 + 99 * 80)
    assert 0.9 * grid_edges < len(col) < 0.99 * grid_edges
    assert wt.min() >= 1 and wt.max() <= 1000


def test_maxweight_rejected_for_sssp_only():
    g = gga.Graph.from_csr([0, 1, 1], [1], [gga.MAX_WEIGHT + 1])
    assert g.info()["max_weight"] == gga.MAX_WEIGHT + 1


def test_combine_clocks_matches_reference_rule():
    """metrics.h:68-84: blocks in order onto the least-loaded SM (first index
    on ties); the estimate is the busiest SM's total."""
    import gpugraphalgo_gb300 as gga

    assert gga.combine_clocks([5, 3, 4, 1, 2], sms=2) == (8, [0, 1, 1, 0, 0])
    assert gga.combine_clocks([1, 1, 1], sms=3) == (1, [0, 1, 2])
    assert gga.combine_clocks([7] * 14) == (7, list(range(14)))
    assert gga.combine_clocks([7] * 15)[0] == 14
    assert gga.combine_clocks([], sms=4) == (0, [])


def test_combine_clocks_matches_reference_fixture():
    """Against the reference's own combineClocks (metrics.h:68-84, 14 SMs),
    run by tests/golden/make_golden_clocks.py."""
    import json
    import os

    import gpugraphalgo_gb300 as gga

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "clocks.json")) as f:
        cases = json.load(f)["cases"]
    assert len(cases) >= 10
    for c in cases:
        assert gga.combine_clocks(c["clocks"]) == (c["estimate"], c["sm"]), len(c["clocks"])
