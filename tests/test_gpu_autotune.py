"""The autotuner: per graph it picks CTA size, SSSP bucket width, BFS
direction thresholds, the expansion strategy (edge units over the unsplit or
the node-split CSR, or the CDP variant) and the batch engine's bucket width
from timed trials, stores the pick on the graph, and every strategy it can
pick gives the oracle's distances (the reference's serial BFS/SSSP,
graph.h:115-184)."""
from __future__ import annotations

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle

pytestmark = pytest.mark.gpu


def _want(g, algo, s):
    return oracle.serial_distances(*g.csr(), algo, s)


def test_autotune_picks_per_graph_and_keeps_answers(ctx):
    graphs = [gga.Graph.rmat(12, 16, seed=3), gga.Graph.grid(48, 40, seed=9)]
    picks = []
    try:
        for g in graphs:
            g.cudaCopy(ctx)
            p = ctx.autotune(g, 1)
            rep = ctx.autotune_report()
            picks.append(p)
            assert p["expansion"] in (0, 1, 2)
            assert p["block_threads"] in (256, 512)
            assert any(k.startswith("sssp_bs") for k in rep) and "bfs_alpha8_beta18" in rep
            assert "expansion_edges_unsplit" in rep and any(k.startswith("batch_sssp8_delta") for k in rep)
            assert any(k.startswith("expansion_cdp") for k in rep)  # small graph: CDP is a candidate
            assert all(v > 0 for v in rep.values())
        ctx.reset_params()  # each graph's solves now use its own tuned parameters
        qs = []
        for g in graphs:
            s = int(np.argmax(g.degrees()))
            for algo in ("bfs", "sssp"):
                np.testing.assert_array_equal(ctx.solve(g, algo, s, "auto"), _want(g, algo, s))
                qs.append((g, algo, s))
        # the batch engine takes each graph's tuned bucket width
        for got, (g, algo, s) in zip(ctx.multi_solve(qs), qs):
            np.testing.assert_array_equal(got, _want(g, algo, s))
    finally:
        ctx.reset_params()
        for g in graphs:
            g.NodeSplit(ctx, 0)


@pytest.mark.parametrize("expansion,level", [(1, -1), (1, 4), (2, -1), (2, 1)])
def test_every_expansion_strategy_matches_oracle(ctx, expansion, level):
    """What GGA_VARIANT_AUTO runs for each pick: edge units over the split
    CSR (expansion 1, the graph split at `level`) or the CDP variant
    (expansion 2 with that heavy-vertex threshold)."""
    g = gga.Graph.rmat(13, 16, seed=17)
    try:
        if expansion == 1:
            g.NodeSplit(ctx, level, 10)
        ctx.set_params(expansion=expansion, split_level=level, split_buckets=10)
        for s in (int(np.argmax(g.degrees())), 7):
            for algo in ("bfs", "sssp"):
                np.testing.assert_array_equal(ctx.solve(g, algo, s, "auto"), _want(g, algo, s),
                                              err_msg=f"expansion {expansion} level {level} {algo} src {s}")
    finally:
        ctx.reset_params()
        g.NodeSplit(ctx, 0)
