"""GPU parity: every engine and split configuration against the reference's
recorded outputs (tests/golden) and the oracle, bit for bit.

Integer distances are unique, so all variants must agree exactly: BFS levels
and SSSP distances of the reference's serial code (graph.h:115-184), the
split arrays of NodeSplit (graph.h:415-522) and zero verifysolution errors
(myutils.h:1-18)."""
from __future__ import annotations

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle
from conftest import build_golden_graph
from _util import digest

pytestmark = pytest.mark.gpu

VARIANTS = ["frontier", "topo_atomic", "topo_plain", "cdp_atomic", "cdp_plain"]


def _golden_items(golden):
    meta, arrays = golden
    for name, e in sorted(meta["graphs"].items()):
        yield name, e, arrays


def test_unsplit_all_variants_match_reference(golden, ctx):
    for name, e, arrays in _golden_items(golden):
        g = build_golden_graph(name, e, arrays)
        for key, rec in e["dist"].items():
            algo, src = key.split("/")
            want = arrays[f"{name}/dist/{key}"]
            for v in VARIANTS:
                got = ctx.solve(g, algo, int(src), v)
                assert digest(got) == rec["sha256"], (name, key, v, np.nonzero(got != want)[0][:5])
            assert g.verifysolution(got, algo) == 0


def test_device_split_matches_reference(golden, ctx):
    for name, e, arrays in _golden_items(golden):
        g = build_golden_graph(name, e, arrays)
        for key, rec in e["split"].items():
            level, buckets = map(int, key.split("/"))
            if rec.get("crash"):
                with pytest.raises(gga.GGAError) as ex:
                    g.NodeSplit(ctx, level, buckets)
                assert ex.value.status == gga.ERR_SPLIT_RULE, (name, key)
                assert g.info()["split_level"] == 0
                continue
            g.NodeSplit(ctx, level, buckets)
            info = g.info()
            assert (info["mda"], info["nnodes"]) == (rec["mda"], rec["nnodes"]), (name, key)
            maps = g.split_maps(ctx)
            for k in ("psrc", "noutgoing", "childCount", "IsParent", "parentNode"):
                assert digest(maps[k]) == rec[f"{k}_sha256"], (name, key, k)
            assert digest(maps["edgessrcdst"][1:]) == rec["edgessrcdst_sha256"], (name, key)
            idx, cnt = g.child_index(ctx)
            np.testing.assert_array_equal(idx, np.nonzero(maps["childCount"])[0])
            np.testing.assert_array_equal(cnt, maps["childCount"][idx])
            assert info["parents_with_children"] == len(idx)
        g.NodeSplit(ctx, 0)
        assert g.info()["split_level"] == 0


def test_split_graph_all_variants_match_reference(golden, ctx):
    for name, e, arrays in _golden_items(golden):
        g = build_golden_graph(name, e, arrays)
        for key, rec in e["split"].items():
            if rec.get("crash"):
                continue
            level, buckets = map(int, key.split("/"))
            g.NodeSplit(ctx, level, buckets)
            for dkey, drec in e["dist"].items():
                algo, src = dkey.split("/")
                for v in ("frontier", "topo_atomic", "topo_plain"):
                    got = ctx.solve(g, algo, int(src), v)
                    assert digest(got) == drec["sha256"], (name, key, dkey, v)
                try:  # the frontier engine over the split view too
                    ctx.set_params(use_split=1)
                    got = ctx.solve(g, algo, int(src), "frontier")
                    assert digest(got) == drec["sha256"], (name, key, dkey, "frontier/split view")
                finally:
                    ctx.reset_params()
        g.NodeSplit(ctx, 0)


@pytest.mark.parametrize("bs", [256, 512, 1024])
@pytest.mark.parametrize("iters", [2, 4, 8])
@pytest.mark.parametrize("delta", [0, 1, 37, 100000])
def test_frontier_parameters_do_not_change_answers(golden, ctx, bs, iters, delta):
    meta, arrays = golden
    name = "c1_rmat14"
    e = meta["graphs"][name]
    g = build_golden_graph(name, e, arrays)
    ctx.set_params(block_threads=bs, unit_iters=iters, sssp_delta=delta, use_split=1)
    if bs * iters > 4096:  # a unit must fit the CTA's shared memory
        with pytest.raises(gga.GGAError) as ex:
            ctx.solve(g, "bfs", 0, "frontier")
        assert ex.value.status == gga.ERR_INVALID_ARG
        ctx.reset_params()
        return
    try:
        for key, rec in e["dist"].items():
            algo, src = key.split("/")
            assert digest(ctx.solve(g, algo, int(src), "frontier")) == rec["sha256"], key
        g.NodeSplit(ctx, -1, 10)
        for key, rec in e["dist"].items():
            algo, src = key.split("/")
            assert digest(ctx.solve(g, algo, int(src), "frontier")) == rec["sha256"], key
        g.NodeSplit(ctx, 0)
    finally:
        ctx.reset_params()


def _oracle_dist(g, algo, src):
    return oracle.serial_distances(*g.csr(), algo, src)


@pytest.mark.parametrize("seed", [21, 22])
def test_random_rmat_against_oracle(ctx, seed):
    g = gga.Graph.rmat(16, 16, seed=seed)
    deg = g.degrees()
    rng = np.random.default_rng(seed)
    srcs = [int(np.argmax(deg)), int(rng.integers(g.n))]
    for algo in ("bfs", "sssp"):
        for s in srcs:
            want = _oracle_dist(g, algo, s)
            for v in ("frontier", "topo_atomic"):
                np.testing.assert_array_equal(ctx.solve(g, algo, s, v), want)
    g.NodeSplit(ctx, -1, 10)
    for algo in ("bfs", "sssp"):
        want = _oracle_dist(g, algo, srcs[0])
        for v in ("frontier", "topo_plain", "cdp_atomic"):
            np.testing.assert_array_equal(ctx.solve(g, algo, srcs[0], v), want)
        try:
            ctx.set_params(use_split=1)
            np.testing.assert_array_equal(ctx.solve(g, algo, srcs[0], "frontier"), want)
        finally:
            ctx.reset_params()


def test_grid_deep_against_oracle(ctx):
    g = gga.Graph.grid(256, 256, 0.05, 0.001, seed=3, wmin=1, wmax=1000)
    for algo in ("bfs", "sssp"):
        want = _oracle_dist(g, algo, 0)
        got, st = ctx.solve(g, algo, 0, "frontier", stats=True)
        np.testing.assert_array_equal(got, want)
        assert st["iterations"] > 50


def test_edge_cases(ctx):
    # single vertex, no edges
    g = gga.Graph.from_csr([0, 0], [])
    assert ctx.bfs(g, 0).tolist() == [0]
    # zero-degree source: everything else unreachable
    g = gga.Graph.from_csr([0, 0, 1, 2], [2, 1], [5, 5])
    for v in VARIANTS:
        assert ctx.sssp(g, 0, v).tolist() == [0, gga.INFINITY, gga.INFINITY]
    # self loops and parallel edges (allowed by from_csr)
    off, col, wt = [0, 3, 4, 4], [0, 1, 1, 2], [4, 9, 2, 1]
    g = gga.Graph.from_csr(off, col, wt)
    for v in VARIANTS:
        assert ctx.sssp(g, 0, v).tolist() == [0, 2, 3]
        assert ctx.bfs(g, 0, v).tolist() == [0, 1, 2]
    # directed (asymmetric) graph and zero weights
    g = gga.Graph.from_csr([0, 2, 3, 3, 4], [1, 2, 3, 1], [0, 7, 0, 0])
    for v in VARIANTS:
        assert ctx.sssp(g, 0, v).tolist() == [0, 0, 7, 0]
        assert ctx.bfs(g, 3, v).tolist() == [gga.INFINITY, 1, gga.INFINITY, 0]
    # weight limit: the heaviest accepted weight cannot wrap; above MYINFINITY
    # the target stays unreached, as the reference's compare leaves it
    g = gga.Graph.from_csr([0, 1, 1], [1], [gga.MAX_WEIGHT])
    for v in VARIANTS:
        assert ctx.sssp(g, 0, v).tolist() == [0, gga.INFINITY]
    g = gga.Graph.from_csr([0, 1, 1], [1], [gga.MAX_WEIGHT + 1])
    with pytest.raises(gga.GGAError) as e:
        ctx.sssp(g, 0)
    assert e.value.status == gga.ERR_INVALID_ARG
    assert ctx.bfs(g, 0).tolist() == [0, 1]
    # bad source
    with pytest.raises(gga.GGAError):
        ctx.bfs(g, 5)


def test_distances_above_infinity_stay_unreached(ctx):
    """A path longer than MYINFINITY is not relaxed (alt < dist fails at 1e9),
    exactly as the reference's unsigned compare behaves."""
    w = [600000000, 600000000]
    g = gga.Graph.from_csr([0, 1, 2, 2], [1, 2], w)
    want = _oracle_dist(g, "sssp", 0)
    assert want.tolist() == [0, 600000000, gga.INFINITY]
    for v in VARIANTS:
        np.testing.assert_array_equal(ctx.sssp(g, 0, v), want)


def test_source_is_split_parent(golden, ctx):
    meta, arrays = golden
    e = meta["graphs"]["hub40_oddm"]
    g = build_golden_graph("hub40_oddm", e, arrays)
    g.NodeSplit(ctx, 7, 10)
    assert g.split_maps(ctx)["childCount"][0] > 0  # vertex 0 (the hub) has children
    for key, rec in e["dist"].items():
        algo, src = key.split("/")
        if src == "0":
            for v in ("frontier", "topo_atomic", "topo_plain"):
                assert digest(ctx.solve(g, algo, 0, v)) == rec["sha256"]
            try:  # the split source as the frontier engine's split view sees it
                ctx.set_params(use_split=1)
                assert digest(ctx.solve(g, algo, 0, "frontier")) == rec["sha256"]
            finally:
                ctx.reset_params()


def test_cdp_modes_and_fallback(ctx):
    g = gga.Graph.rmat(14, 16, seed=5)
    s = int(np.argmax(g.degrees()))
    want = {a: _oracle_dist(g, a, s) for a in ("bfs", "sssp")}
    try:
        for mode in (0, 1, 2):
            ctx.set_params(cdp_level=20, cdp_mode=mode)
            for a in ("bfs", "sssp"):
                for v in ("cdp_atomic", "cdp_plain"):
                    got, st = ctx.solve(g, a, s, v, stats=True)
                    np.testing.assert_array_equal(got, want[a])
                    if mode == 2:
                        assert st["cdp_children"] == 0
                    else:
                        assert st["cdp_children"] + st["cdp_fallbacks"] > 0
        # the reference's shape with a tiny pending-launch budget: launches
        # that do not fit fall back to inline relaxation (cudaKernels.h:483-512)
        ctx.set_params(cdp_level=40, cdp_mode=1, cdp_pending_limit=4)
        for a in ("bfs", "sssp"):
            got, st = ctx.solve(g, a, s, "cdp_atomic", stats=True)
            np.testing.assert_array_equal(got, want[a])
    finally:
        ctx.set_params(cdp_pending_limit=2048)
        ctx.reset_params()


def test_device_output_buffer(ctx):
    torch = pytest.importorskip("torch")
    g = gga.Graph.rmat(12, 8, seed=4)
    want = ctx.bfs(g, 1)
    out = torch.empty(g.n, dtype=torch.int32, device="cuda")
    lib = gga.lib()
    import ctypes

    s = gga._native.Stats()
    rc = lib.gga_solve(ctx.handle, g.handle, gga.BFS, 1, 1, ctypes.c_void_p(out.data_ptr()), ctypes.byref(s))
    assert rc == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want)


def test_stats_report_reached(ctx):
    g = gga.Graph.rmat(14, 8, seed=1)
    try:
        ctx.set_params(bfs_direction=1)  # top-down only
        d, st = ctx.bfs(g, 0, stats=True)
    finally:
        ctx.reset_params()
    vr, er = g.reached(d)
    assert st["vertices_reached"] == vr and st["edges_reached"] == er
    assert st["edges_relaxed"] == er  # top-down BFS expands each reached vertex once
    assert st["kernel_ms"] > 0 and st["kernel_launches"] >= 1


@pytest.mark.parametrize("alpha,beta", [(0, 0), (1000, 1000), (1, 2), (1000, 1)])
def test_bfs_bottom_up_rounds_match_oracle(ctx, alpha, beta):
    """Direction-optimising BFS (bottom-up rounds where the frontier is large)
    gives the same levels for every mix of top-down and bottom-up rounds."""
    for g in (gga.Graph.rmat(16, 16, seed=23), gga.Graph.grid(128, 96, seed=5)):
        deg = g.degrees()
        srcs = [int(np.argmax(deg)), 17, int(np.nonzero(deg == 0)[0][0]) if (deg == 0).any() else 3]
        try:
            ctx.set_params(bfs_direction=0, bfs_alpha=alpha, bfs_beta=beta)
            for s in srcs:
                np.testing.assert_array_equal(ctx.bfs(g, s), _oracle_dist(g, "bfs", s))
        finally:
            ctx.reset_params()
        assert g.info()["symmetric"] == 1


def test_bottom_up_checks_fewer_edges(ctx):
    g = gga.Graph.rmat(16, 16, seed=3)
    s = int(np.argmax(g.degrees()))
    try:
        ctx.set_params(bfs_direction=1)
        d1, st1 = ctx.bfs(g, s, stats=True)
    finally:
        ctx.reset_params()
    d0, st0 = ctx.bfs(g, s, stats=True)
    np.testing.assert_array_equal(d0, d1)
    assert st0["edges_relaxed"] < st1["edges_relaxed"] == st1["edges_reached"]


def test_bfs_on_directed_graph_stays_top_down(ctx):
    """Bottom-up rounds need every edge's reverse: a directed CSR is detected
    on the device (symmetric = -1) and walked top-down only."""
    off, col, wt = gga.Graph.rmat(12, 8, seed=9).csr()
    u = np.repeat(np.arange(len(off) - 1, dtype=np.uint32), np.diff(off.astype(np.int64)))
    keep = u < col
    u, v, w = u[keep], col[keep], wt[keep]
    noff = np.zeros(len(off), np.uint32)
    np.add.at(noff, u + 1, 1)
    noff = np.cumsum(noff, dtype=np.uint64).astype(np.uint32)
    g = gga.Graph.from_csr(noff, v.astype(np.uint32), w.astype(np.uint32))
    assert g.info()["symmetric"] == 0
    for s in (0, 5, int(np.argmax(g.degrees()))):
        np.testing.assert_array_equal(ctx.bfs(g, s), _oracle_dist(g, "bfs", s))
    assert g.info()["symmetric"] == -1


@pytest.mark.parametrize("delta", [1, 7, 33, 100, 5000])
def test_sssp_light_heavy_classes_match_oracle(ctx, delta):
    """Delta-stepping's light/heavy edge classes (light-first rows, heavy
    edges relaxed once per bucket) give the same distances as relaxing every
    edge in every near round, for every bucket width."""
    for g in (gga.Graph.rmat(15, 16, seed=41), gga.Graph.grid(96, 80, seed=6)):
        srcs = [int(np.argmax(g.degrees())), 11]
        for s in srcs:
            want = _oracle_dist(g, "sssp", s)
            try:
                for lh in (0, 1):
                    ctx.set_params(sssp_delta=delta, sssp_light_heavy=lh)
                    got, st = ctx.sssp(g, s, stats=True)
                    np.testing.assert_array_equal(got, want, err_msg=f"delta={delta} lh={lh} src={s}")
            finally:
                ctx.reset_params()


def test_sssp_light_heavy_relaxes_fewer_edges(ctx):
    g = gga.Graph.rmat(16, 16, seed=8)
    s = int(np.argmax(g.degrees()))
    res = {}
    try:
        for lh in (0, 1):
            ctx.set_params(sssp_delta=32, sssp_light_heavy=lh)
            res[lh] = ctx.sssp(g, s, stats=True)
    finally:
        ctx.reset_params()
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert res[0][1]["edges_relaxed"] < res[1][1]["edges_relaxed"]


@pytest.mark.parametrize("delta", [1, 7, 33, 100])
def test_sssp_pull_bucket_close_matches_oracle(ctx, delta):
    """Closing a bucket by pull (each unsettled vertex takes the smallest
    d(u) + w over its heavy edges to settled vertices) gives the same
    distances as pushing the bucket's heavy edges: with the cost rule (0),
    never (1) and at every bucket (2)."""
    for g in (gga.Graph.rmat(15, 16, seed=41), gga.Graph.grid(96, 80, seed=6)):
        assert g.info()["wsymmetric"] == 1
        for s in (int(np.argmax(g.degrees())), 11):
            want = _oracle_dist(g, "sssp", s)
            try:
                for pull in (0, 1, 2):
                    ctx.set_params(sssp_delta=delta, sssp_pull=pull)
                    np.testing.assert_array_equal(ctx.sssp(g, s), want, err_msg=f"delta={delta} pull={pull} src={s}")
            finally:
                ctx.reset_params()


def test_sssp_pull_relaxes_fewer_edges(ctx):
    """On R-MAT the first bucket holds the hubs: its heavy edges far
    outnumber the unsettled vertices', so the cost rule pulls there."""
    g = gga.Graph.rmat(16, 16, seed=8)
    s = int(np.argmax(g.degrees()))
    res, kinds = {}, {}
    try:
        ctx.trace(True)
        for pull in (0, 1):
            ctx.set_params(sssp_delta=32, sssp_pull=pull)
            res[pull] = ctx.sssp(g, s, stats=True)
            kinds[pull] = {r["kind"] for r in ctx.last_trace()["rounds"]}
    finally:
        ctx.trace(False)
        ctx.reset_params()
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert res[0][1]["edges_relaxed"] < res[1][1]["edges_relaxed"]
    assert {"pull_scan", "pull"} <= kinds[0]
    assert "pull" not in kinds[1] and "heavy" in kinds[1]


def test_sssp_pull_needs_equal_reverse_weights(ctx):
    """A graph whose every edge has its reverse, but with another weight,
    must not pull (the pull reads w(v, u) for w(u, v)): the device check
    marks it and the bucket closes push, so the distances stay right even
    with sssp_pull = 2."""
    off, col, wt = gga.Graph.rmat(13, 8, seed=17).csr()
    u = np.repeat(np.arange(len(off) - 1, dtype=np.uint32), np.diff(off.astype(np.int64)))
    wt2 = (wt + (u < col)).astype(np.uint32)
    g = gga.Graph.from_csr(off, col, wt2)
    assert g.info()["wsymmetric"] == 0
    s = int(np.argmax(g.degrees()))
    try:
        ctx.set_params(sssp_delta=16, sssp_pull=2)
        ctx.trace(True)
        np.testing.assert_array_equal(ctx.sssp(g, s), _oracle_dist(g, "sssp", s))
        kinds = {r["kind"] for r in ctx.last_trace()["rounds"]}
    finally:
        ctx.trace(False)
        ctx.reset_params()
    info = g.info()
    assert info["symmetric"] == 1 and info["wsymmetric"] == -1
    assert "pull" not in kinds
    with pytest.raises(gga.GGAError):
        ctx.set_params(sssp_pull=3)


@pytest.mark.parametrize("algo", ["bfs", "sssp"])
def test_solve_many_matches_single_solves(ctx, algo):
    """gga_solve_many: back-to-back traversals with the copies on a second
    stream give each source's single-solve distances and stats, into pinned
    or pageable host memory, on split and unsplit graphs."""
    for g in (gga.Graph.rmat(14, 16, seed=12), gga.Graph.grid(64, 50, seed=3)):
        srcs = [int(np.argmax(g.degrees())), 0, 17, 5, 0, 999 % g.n, 33]  # repeats and more than the ring
        pinned = gga.pinned_empty((len(srcs), g.n))
        got, st = ctx.solve_many(g, algo, srcs, out=pinned, stats=True)
        assert got is pinned
        page = ctx.solve_many(g, algo, srcs)
        for i, s in enumerate(srcs):
            want, ws = ctx.solve(g, algo, s, "frontier", stats=True)
            np.testing.assert_array_equal(got[i], want, err_msg=f"src #{i}={s}")
            np.testing.assert_array_equal(page[i], want)
            assert st[i]["vertices_reached"] == ws["vertices_reached"]
            assert st[i]["edges_reached"] == ws["edges_reached"]
            assert st[i]["kernel_ms"] > 0
            if algo == "bfs":  # BFS rounds are the levels; SSSP's depend on relaxation timing
                assert st[i]["iterations"] == ws["iterations"]
        np.testing.assert_array_equal(got[0], _oracle_dist(g, algo, srcs[0]))
    gs = gga.Graph.rmat(12, 8, seed=4)
    gs.cudaCopy(ctx)
    gs.NodeSplit(ctx, 4)
    try:
        srcs = [0, 3, 100, 7]
        for us in (0, 1):
            ctx.set_params(use_split=us)
            got = ctx.solve_many(gs, algo, srcs)
            for i, s in enumerate(srcs):
                np.testing.assert_array_equal(got[i], _oracle_dist(gs, algo, s), err_msg=f"use_split={us}")
    finally:
        ctx.reset_params()
        gs.NodeSplit(ctx, 0)


def test_solve_many_edges(ctx):
    g = gga.Graph.rmat(10, 8, seed=2)
    assert ctx.solve_many(g, "bfs", []).shape == (0, g.n)
    with pytest.raises(gga.GGAError) as ex:
        ctx.solve_many(g, "sssp", [0, g.n])
    assert ex.value.status == gga.ERR_INVALID_ARG
    torch = pytest.importorskip("torch")
    out = torch.empty((3, g.n), dtype=torch.int32, device="cuda")
    ctx.solve_many(g, "sssp", [1, 2, 3], out=out)
    got = out.cpu().numpy().view(np.uint32)
    for i, s in enumerate([1, 2, 3]):
        np.testing.assert_array_equal(got[i], _oracle_dist(g, "sssp", s))


@pytest.mark.parametrize("tail", [0, 1, 2, 64])
def test_sssp_tail_matches_oracle(ctx, tail):
    """Ending the buckets early (the rest as one label-correcting frontier
    over whole rows) gives the same distances, with and without light/heavy
    classes and pulled bucket closes."""
    for g in (gga.Graph.rmat(15, 16, seed=41), gga.Graph.grid(96, 80, seed=6)):
        for s in (int(np.argmax(g.degrees())), 11):
            want = _oracle_dist(g, "sssp", s)
            try:
                for delta, lh, pull in ((16, 0, 0), (33, 0, 2), (100, 1, 1), (1, 0, 1)):
                    ctx.set_params(sssp_delta=delta, sssp_tail=tail, sssp_light_heavy=lh, sssp_pull=pull)
                    np.testing.assert_array_equal(ctx.sssp(g, s), want,
                                                  err_msg=f"tail={tail} delta={delta} lh={lh} pull={pull} src={s}")
            finally:
                ctx.reset_params()


def test_sssp_tail_cuts_rounds(ctx):
    g = gga.Graph.rmat(16, 16, seed=8)
    s = int(np.argmax(g.degrees()))
    res = {}
    try:
        for tail in (0, 1):
            ctx.set_params(sssp_delta=16, sssp_tail=tail)
            res[tail] = ctx.sssp(g, s, stats=True)
    finally:
        ctx.reset_params()
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert res[0][1]["iterations"] < res[1][1]["iterations"]


@pytest.mark.parametrize("variant", ["topo_atomic", "topo_plain", "cdp_atomic"])
@pytest.mark.parametrize("algo", ["bfs", "sssp"])
def test_convergence_log(ctx, variant, algo):
    """printConv_rtime (convergence.h:100-159) after every relax launch: the
    vertices still differing from the final answer shrink to none, and the
    reference's norm (squares of 32-bit unsigned differences) is exact."""
    g = gga.Graph.rmat(11, 8, seed=41)
    if variant == "topo_plain":
        g.node_split(ctx, -1, 10)
    want = _oracle_dist(g, algo, 7)
    recs, got = ctx.convergence(g, algo, 7, want, variant)
    np.testing.assert_array_equal(got, want)
    assert [r["iteration"] for r in recs] == list(range(1, len(recs) + 1))
    diffs = [r["diff_count"] for r in recs]
    assert diffs == sorted(diffs, reverse=True) and diffs[-1] == 0 and recs[-1]["norm2"] == 0.0
    reached = want < gga.INFINITY
    n = int(reached.sum())
    # against a final answer off by a known amount the converged state shows it
    for off, per_vertex in ((1, 1), (-1, 1), (65536, 0), (3, 9)):
        fin = want.astype(np.int64)
        fin[reached] += off
        fin = (fin % (1 << 32)).astype(np.uint32)
        recs, _ = ctx.convergence(g, algo, 7, fin, variant)
        assert recs[-1]["diff_count"] == n
        assert recs[-1]["norm2"] == pytest.approx((n * per_vertex) ** 0.5, rel=1e-12, abs=0)


def test_convergence_rejects_frontier(ctx):
    g = gga.Graph.rmat(8, 4, seed=2)
    with pytest.raises(gga.GGAError) as ex:
        ctx.convergence(g, "bfs", 0, np.zeros(g.n, np.uint32), "frontier")
    assert ex.value.status == gga.ERR_INVALID_ARG


def test_release_and_upload_again_reuses_the_pool(ctx):
    """gga_graph_release_device returns the device arrays (the CSR and the
    light/heavy order) to the stream-ordered pool and the next upload takes
    them again; over several cycles, with a mesh refinement using the same
    pool in between, every traversal still equals the oracle's."""
    g = gga.Graph.rmat(15, 16, seed=8)
    off, col, wt = g.csr()
    og = oracle.OracleGraph.from_csr(off, col, wt)
    srcs = [int(s) for s in np.nonzero(np.diff(off.astype(np.int64)) > 0)[0][:3]]
    want = {(a, s): og.shortest(a, s) for a in ("bfs", "sssp") for s in srcs}
    g.pin(True)
    for cycle in range(4):
        g.release_device()
        g.cudaCopy(ctx)
        ctx.prepare(g, "bfs")
        ctx.prepare(g, "sssp")
        for (a, s), w in want.items():
            np.testing.assert_array_equal(ctx.solve(g, a, s), w, err_msg=f"cycle {cycle} {a} {s}")
        out = gga.pinned_empty((len(srcs), g.n))
        ctx.solve_many(g, "sssp", srcs, out=out)
        for i, s in enumerate(srcs):
            np.testing.assert_array_equal(out[i], want[("sssp", s)])
        if cycle == 1:
            m = gga.Mesh.random(3000, seed=cycle)
            ctx.refine(m)
            assert m.check()["bad_triangles"] == 0
    g.pin(False)
