"""Batched queries on the GPU: bit-packed multi-source BFS, 32-source SSSP,
multi-graph batches and the serving loop, each row checked bit for bit
against the oracle's single-source serial runs (the reference's
findSerialBFS / findSerialSSSP, graph.h:115-184).

A batch changes how work is scheduled, never the answer: every query's
distances must equal the one-source result."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle

pytestmark = pytest.mark.gpu

_CACHE: dict = {}


def _want(g, algo, src):
    key = (id(g), algo, int(src))
    if key not in _CACHE:
        _CACHE[key] = oracle.serial_distances(*g.csr(), algo, int(src))
    return _CACHE[key]


@pytest.fixture(scope="module")
def graphs():
    gs = {
        "rmat12": gga.Graph.rmat(12, 8, seed=5),
        "rmat10": gga.Graph.rmat(10, 16, seed=6),
        "grid": gga.Graph.grid(40, 30, seed=7),
        # 0 -> 1 -> 2, 3 isolated, 4 -> 0 (a source with no out-edges, an unreachable part)
        "tiny": gga.Graph.from_csr(np.array([0, 1, 2, 2, 2, 3], np.uint32), np.array([1, 2, 0], np.uint32),
                                   np.array([5, 7, 1], np.uint32)),
    }
    yield gs
    _CACHE.clear()


def _sources(g, k, seed):
    rng = np.random.default_rng(seed)
    deg = g.degrees()
    s = [int(np.argmax(deg))] + [int(x) for x in rng.integers(0, g.n, k - 1)]
    return s[:k]


def test_msbfs_64_sources_match_oracle(ctx, graphs):
    for name in ("rmat12", "grid"):
        g = graphs[name]
        srcs = _sources(g, 64, 11)
        srcs[5] = srcs[0]  # duplicate source vertices share one traversal bit set
        got, st = ctx.msbfs(g, srcs, stats=True)
        assert got.shape == (64, g.n)
        for i, s in enumerate(srcs):
            np.testing.assert_array_equal(got[i], _want(g, "bfs", s), err_msg=f"{name} src#{i}={s}")
        reached = sum(int((_want(g, "bfs", s) < gga.INFINITY).sum()) for s in srcs)
        assert st["vertices_reached"] == reached
        assert st["iterations"] >= 1


@pytest.mark.parametrize("k", [1, 3, 33])
def test_msbfs_partial_batches(ctx, graphs, k):
    g = graphs["rmat10"]
    srcs = _sources(g, k, k)
    got = ctx.msbfs(g, srcs)
    for i, s in enumerate(srcs):
        np.testing.assert_array_equal(got[i], _want(g, "bfs", s))


def test_msbfs_sources_without_edges(ctx, graphs):
    g = graphs["tiny"]
    got = ctx.msbfs(g, [0, 2, 3, 4])
    for i, s in enumerate([0, 2, 3, 4]):
        np.testing.assert_array_equal(got[i], _want(g, "bfs", s))


def test_msbfs_rejects_bad_arguments(ctx, graphs):
    g = graphs["rmat10"]
    for srcs in ([], list(range(65)), [g.n]):
        with pytest.raises(gga.GGAError) as ex:
            ctx.msbfs(g, srcs)
        assert ex.value.status == gga.ERR_INVALID_ARG


def test_msbfs_device_output(ctx, graphs):
    torch = pytest.importorskip("torch")
    g = graphs["rmat10"]
    srcs = np.array(_sources(g, 8, 3), np.uint32)
    out = torch.empty((8, g.n), dtype=torch.int32, device="cuda")
    s = gga._native.Stats()
    rc = gga.lib().gga_msbfs(ctx.handle, g.handle, 8, srcs.ctypes.data_as(ctypes.c_void_p),
                             ctypes.c_void_p(out.data_ptr()), ctypes.byref(s))
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    for i, src in enumerate(srcs):
        np.testing.assert_array_equal(got[i], _want(g, "bfs", src))


def test_sssp_batch_32_sources_match_oracle(ctx, graphs):
    for name in ("rmat12", "grid"):
        g = graphs[name]
        srcs = _sources(g, 32, 12)
        got, st = ctx.sssp_batch(g, srcs, stats=True)
        for i, s in enumerate(srcs):
            np.testing.assert_array_equal(got[i], _want(g, "sssp", s), err_msg=f"{name} src#{i}={s}")
        # one warp-edge visit serves every source whose frontier holds the tail
        assert 0 < st["edges_relaxed"] and st["edges_reached"] > 0


def test_sssp_batch_limits(ctx, graphs):
    g = graphs["rmat10"]
    with pytest.raises(gga.GGAError):
        ctx.sssp_batch(g, list(range(33)))
    with pytest.raises(gga.GGAError):
        ctx.sssp_batch(g, [g.n + 1])


def test_multi_graph_batch_matches_oracle(ctx, graphs):
    queries = []
    for j, name in enumerate(sorted(graphs)):
        g = graphs[name]
        for s in _sources(g, 4, 20 + j):
            for algo in ("bfs", "sssp"):
                queries.append((g, algo, s))
    outs, st = ctx.multi_solve(queries, stats=True)
    assert len(outs) == len(queries)
    for (g, algo, s), got in zip(queries, outs):
        np.testing.assert_array_equal(got, _want(g, algo, s))
    want_vr = sum(int((_want(g, a, s) < gga.INFINITY).sum()) for g, a, s in queries)
    assert st["vertices_reached"] == want_vr


def test_multi_graph_batch_equals_single_solves(ctx, graphs):
    g = graphs["rmat12"]
    srcs = _sources(g, 6, 30)
    queries = [(g, "sssp" if i % 2 else "bfs", s) for i, s in enumerate(srcs)]
    outs = ctx.multi_solve(queries)
    for (gg, algo, s), got in zip(queries, outs):
        np.testing.assert_array_equal(got, ctx.solve(gg, algo, s, "frontier"))
    assert ctx.multi_solve([]) == []


def test_server_mixed_stream_matches_oracle(ctx, graphs):
    names = ["rmat12", "rmat10", "grid", "tiny"]
    gl = [graphs[n] for n in names]
    srv = gga.Server(ctx, gl, mem_cap_bytes=256 << 20, max_slots=16)
    try:
        rng = np.random.default_rng(40)
        tickets = []
        for i in range(120):
            gi = int(rng.integers(len(gl)))
            algo = "bfs" if rng.random() < 0.7 else "sssp"
            s = int(rng.integers(gl[gi].n))
            tickets.append((srv.submit(gi, algo, s), gi, algo, s))
        lats = []
        for t, gi, algo, s in tickets:
            got, lat = srv.wait(t)
            np.testing.assert_array_equal(got, _want(gl[gi], algo, s))
            lats.append(lat)
        st = srv.stats()
        assert st["submitted"] == st["completed"] == 120
        assert st["rejected"] == 0
        assert 1 <= st["max_inflight"] <= 16
        assert st["supersteps"] >= 1
        assert all(x > 0 for x in lats)
    finally:
        srv.close()


def test_server_slot_limit_and_admission(ctx, graphs):
    small, big = graphs["tiny"], graphs["rmat12"]
    # 64 KiB: queue room for ~1600 vertices, so the 4096-vertex graph never fits
    srv = gga.Server(ctx, [small, big], mem_cap_bytes=64 << 10, max_slots=2)
    try:
        with pytest.raises(gga.GGAError) as ex:
            srv.submit(1, "bfs", 0)
        assert ex.value.status == gga.ERR_ADMISSION
        ts = [(srv.submit(0, "sssp" if i % 2 else "bfs", i % small.n), i) for i in range(20)]
        for t, i in ts:
            got, _ = srv.wait(t)
            np.testing.assert_array_equal(got, _want(small, "sssp" if i % 2 else "bfs", i % small.n))
        st = srv.stats()
        assert st["rejected"] == 1 and st["completed"] == 20
        assert st["max_inflight"] <= 2
        with pytest.raises(gga.GGAError) as ex:
            srv.submit(0, "bfs", small.n)
        assert ex.value.status == gga.ERR_INVALID_ARG
    finally:
        srv.close()


def test_server_poll_and_close_with_work_pending(ctx, graphs):
    g = graphs["rmat12"]
    srv = gga.Server(ctx, [g], mem_cap_bytes=64 << 20, max_slots=4)
    t = srv.submit(0, "sssp", 0)
    r = None
    for _ in range(20000):
        r = srv.poll(t)
        if r is not None:
            break
    if r is None:
        r = srv.wait(t)
    np.testing.assert_array_equal(r[0], _want(g, "sssp", 0))
    for s in range(8):
        srv.submit(0, "bfs", s)
    srv.close()  # returns with queries still queued; their tickets are dropped
