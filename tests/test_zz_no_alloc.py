"""GPU tests of gga_bfs_noalloc, the BFS entry point that allocates no GPU memory.

Some callers cannot allocate device memory while they traverse a graph: code
running inside a memory pool that another framework owns, latency-critical
paths where cudaMalloc could synchronise the device, processes whose device
memory is reserved up front.  gga_bfs_noalloc serves them from a fixed array
the library reserves on each GPU.  Its results must equal the oracle's (the
reference's serial BFS) and gga_bfs's, bit for bit (integer BFS levels), on
consecutive calls that reuse that array: at its size limit, on a directed
graph, with unreached vertices, and after a call that the kernel rejected.

This file is collected last so that a stop-at-first-failure run has already
run every other test when it gets here.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle

pytestmark = pytest.mark.gpu

MAX_NODES = 1 << 18  # the entry point's documented limits
MAX_EDGES = 1 << 23


def _dev_ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _upload(torch, off, col):
    d_off = torch.from_numpy(off.view(np.int32).copy()).cuda()
    d_col = torch.from_numpy((col if len(col) else np.zeros(1, np.uint32)).view(np.int32).copy()).cuda()
    d_dist = torch.empty(len(off) - 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    return d_off, d_col, d_dist


def _noalloc(torch, d_off, d_col, n, m, src, d_dist):
    lib = gga.lib()
    rc = lib.gga_bfs_noalloc(_dev_ptr(d_off), _dev_ptr(d_col), n, m, src, _dev_ptr(d_dist), None)
    torch.cuda.synchronize()
    return rc, lib.gga_last_error().decode()


def test_noalloc_bfs_matches_oracle_and_gga_bfs_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    g = gga.Graph.rmat(16, 16, seed=7)
    off, col, wt = g.csr()
    n, m = len(off) - 1, len(col)
    deg = np.diff(off.astype(np.int64))
    srcs = [int(np.argmax(deg)), int(np.nonzero(deg)[0][len(deg) // 3])]
    with gga.Context(0) as ctx:
        want = [ctx.bfs(g, s) for s in srcs]
    d_off, d_col, d_dist = _upload(torch, off, col)
    for s, w in zip(srcs, want):  # two calls in a row share the fixed array
        rc, msg = _noalloc(torch, d_off, d_col, n, m, s, d_dist)
        assert rc == gga.OK, msg
        got = d_dist.cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(got, w)
        np.testing.assert_array_equal(got, oracle.serial_distances(off, col, wt, "bfs", s))


def test_noalloc_bfs_at_its_size_limit_matches_oracle():
    """262,144 vertices (the limit) and 8.06 M edges (96% of the edge limit),
    where the fixed queue and unit-table regions are tightest."""
    torch = pytest.importorskip("torch")
    g = gga.Graph.rmat(18, 17, seed=7)
    off, col, wt = g.csr()
    n, m = len(off) - 1, len(col)
    assert n == MAX_NODES and 0.9 * MAX_EDGES < m <= MAX_EDGES
    deg = np.diff(off.astype(np.int64))
    d_off, d_col, d_dist = _upload(torch, off, col)
    for s in (int(np.argmax(deg)), int(np.nonzero(deg == 1)[0][0])):
        rc, msg = _noalloc(torch, d_off, d_col, n, m, s, d_dist)
        assert rc == gga.OK, msg
        np.testing.assert_array_equal(d_dist.cpu().numpy().view(np.uint32),
                                      oracle.serial_distances(off, col, wt, "bfs", s))


def _directed_two_components(seed: int):
    """A directed graph (edges kept in one direction only, at random) in two
    components, so part of the graph is never reached."""
    rng = np.random.default_rng(seed)
    parts, base = [], 0
    for k in (3000, 2000):
        a = rng.integers(0, k, 6 * k)
        b = rng.integers(0, k, 6 * k)
        keep = a != b
        parts.append((a[keep] + base, b[keep] + base))
        base += k
    a = np.concatenate([p[0] for p in parts])
    b = np.concatenate([p[1] for p in parts])
    pairs = np.unique(np.stack([a, b], 1), axis=0)
    n = base
    off = np.zeros(n + 1, np.uint32)
    np.add.at(off, pairs[:, 0] + 1, 1)
    off = np.cumsum(off).astype(np.uint32)
    col = pairs[:, 1].astype(np.uint32)
    wt = np.ones(len(col), np.uint32)
    return off, col, wt


def test_noalloc_bfs_directed_graph_with_unreached_vertices():
    torch = pytest.importorskip("torch")
    off, col, wt = _directed_two_components(11)
    n, m = len(off) - 1, len(col)
    g = gga.Graph.from_csr(off, col, wt)
    d_off, d_col, d_dist = _upload(torch, off, col)
    with gga.Context(0) as ctx:
        for s in (0, 4000):
            rc, msg = _noalloc(torch, d_off, d_col, n, m, s, d_dist)
            assert rc == gga.OK, msg
            got = d_dist.cpu().numpy().view(np.uint32)
            want = oracle.serial_distances(off, col, wt, "bfs", s)
            assert (want == oracle.INF).sum() > 0  # the other component stays unreached
            np.testing.assert_array_equal(got, want)
            np.testing.assert_array_equal(got, ctx.bfs(g, s))


def test_noalloc_bfs_rejects_a_target_outside_the_graph_then_recovers():
    """A column id equal to n is caught by the kernel's own bounds check
    (GGA_ERR_FORMAT, no access made with it); the next call on a good CSR,
    sharing the same fixed array, is exact again."""
    torch = pytest.importorskip("torch")
    g = gga.Graph.rmat(12, 8, seed=5)
    off, col, wt = g.csr()
    n, m = len(off) - 1, len(col)
    deg = np.diff(off.astype(np.int64))
    src = int(np.argmax(deg))
    bad = col.copy()
    bad[off[src]] = n  # the source's first edge: expanded in the first round
    d_off, d_bad, d_dist = _upload(torch, off, bad)
    rc, msg = _noalloc(torch, d_off, d_bad, n, m, src, d_dist)
    assert rc == gga.ERR_FORMAT, (rc, msg)
    assert "malformed CSR" in msg
    _, d_col, _ = _upload(torch, off, col)
    rc, msg = _noalloc(torch, d_off, d_col, n, m, src, d_dist)
    assert rc == gga.OK, msg
    np.testing.assert_array_equal(d_dist.cpu().numpy().view(np.uint32),
                                  oracle.serial_distances(off, col, wt, "bfs", src))


def test_noalloc_bfs_rejects_graphs_beyond_its_limit():
    torch = pytest.importorskip("torch")
    d = torch.zeros(8, dtype=torch.int32, device="cuda")
    lib = gga.lib()
    rc = lib.gga_bfs_noalloc(_dev_ptr(d), _dev_ptr(d), MAX_NODES + 1, 4, 0, _dev_ptr(d), None)
    assert rc == gga.ERR_TOO_LARGE
    assert "fixed working memory" in lib.gga_last_error().decode()
    rc = lib.gga_bfs_noalloc(_dev_ptr(d), _dev_ptr(d), 4, MAX_EDGES + 1, 0, _dev_ptr(d), None)
    assert rc == gga.ERR_TOO_LARGE
