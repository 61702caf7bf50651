"""GPU test of gga_bfs_noalloc, the BFS entry point that allocates no GPU memory.

Some callers cannot allocate device memory while they traverse a graph: code
running inside a memory pool that another framework owns, latency-critical
paths where cudaMalloc could synchronise the device, processes whose device
memory is reserved up front.  gga_bfs_noalloc serves them from a fixed array
the library reserves on each GPU.  Its results must equal gga_bfs's, bit for
bit (integer BFS levels), on consecutive calls that reuse that array.

This file is collected last so that a stop-at-first-failure run has already
run every other test when it gets here.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga

pytestmark = pytest.mark.gpu


def _dev_ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_bfs_matches_gga_bfs_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    g = gga.Graph.rmat(16, 16, seed=7)
    off, col, _ = g.csr()
    n, m = len(off) - 1, len(col)
    deg = np.diff(off.astype(np.int64))
    srcs = [int(np.argmax(deg)), int(np.nonzero(deg)[0][len(deg) // 3])]
    with gga.Context(0) as ctx:
        want = [ctx.bfs(g, s) for s in srcs]
    d_off = torch.from_numpy(off.view(np.int32).copy()).cuda()
    d_col = torch.from_numpy(col.view(np.int32).copy()).cuda()
    d_dist = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    lib = gga.lib()
    for s, w in zip(srcs, want):  # two calls in a row share the fixed array
        rc = lib.gga_bfs_noalloc(_dev_ptr(d_off), _dev_ptr(d_col), n, m, s, _dev_ptr(d_dist), None)
        assert rc == gga.OK, lib.gga_last_error().decode()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_dist.cpu().numpy().view(np.uint32), w)


def test_noalloc_bfs_rejects_graphs_beyond_its_limit():
    torch = pytest.importorskip("torch")
    d = torch.zeros(8, dtype=torch.int32, device="cuda")
    lib = gga.lib()
    rc = lib.gga_bfs_noalloc(_dev_ptr(d), _dev_ptr(d), (1 << 18) + 1, 4, 0, _dev_ptr(d), None)
    assert rc == gga.ERR_TOO_LARGE
    assert "fixed working memory" in lib.gga_last_error().decode()
    rc = lib.gga_bfs_noalloc(_dev_ptr(d), _dev_ptr(d), 4, (1 << 23) + 1, 0, _dev_ptr(d), None)
    assert rc == gga.ERR_TOO_LARGE
