"""The persistent kernels' own source text, run on the CPU against the oracle.

tests/emu/gen_kernels.py turns a kernel file (frontier.cu, sssp32.cu,
msbfs.cu, batch.cu) into host C++ and tests/emu/prelude.h emulates the CUDA
constructs it uses: one host thread per CUDA thread, real barriers for
__syncthreads (which also check that every thread of the block arrived from
the same call site) and for warp collectives (so a collective reached by
part of a warp hangs here instead of passing), host atomics, and grid
barriers between
2-4 emulated blocks that interleave freely.  Each case checks bit-exact
distances against the oracle (the reference's serial BFS/SSSP,
graph.h:115-184) and that the kernel's error word stays clear.  This is how
every change to a persistent kernel's synchronisation is checked before it
runs on a GPU; it needs only g++ (C++20)."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle

EMU = os.path.join(os.path.dirname(os.path.abspath(__file__)), "emu")


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    root = tmp_path_factory.mktemp("emu")
    rng = np.random.default_rng(1)
    graphs = {"r10": gga.Graph.rmat(10, 8, seed=5), "grid": gga.Graph.grid(24, 20, seed=7)}
    for name, g in graphs.items():
        d = root / name
        d.mkdir()
        off, col, wt = g.csr()
        deg = g.degrees()
        srcs = [int(np.argmax(deg))] + [int(x) for x in rng.integers(0, g.n, 63)]
        srcs[5] = srcs[0]  # a repeated source vertex
        for arr, f in ((off, "off"), (col, "col"), (wt, "wt")):
            arr.astype(np.uint32).tofile(d / f"{f}.bin")
        np.array(srcs, np.uint32).tofile(d / "srcs.bin")
        np.stack([oracle.serial_distances(off, col, wt, "bfs", s) for s in srcs]).astype(np.uint32).tofile(d / "want_bfs.bin")
        np.stack([oracle.serial_distances(off, col, wt, "sssp", s) for s in srcs[:32]]).astype(np.uint32).tofile(
            d / "want_sssp.bin")
        algos = [i % 2 for i in range(16)]
        np.array(algos, np.uint32).tofile(d / "algos.bin")
        np.stack([oracle.serial_distances(off, col, wt, "sssp" if a else "bfs", s) for s, a in zip(srcs[:16], algos)]
                 ).astype(np.uint32).tofile(d / "want_mix.bin")
    shutil.copy(os.path.join(EMU, "prelude.h"), root / "prelude.h")
    bins = {}
    for k in ("frontier", "sssp32", "msbfs", "mq", "dmr"):
        harness = os.path.join(EMU, f"emu_{k}.cpp")
        if not os.path.exists(harness):
            continue
        subprocess.run(["python3", os.path.join(EMU, "gen_kernels.py"), k, str(root / f"kernel_{k}.inc")], check=True)
        shutil.copy(harness, root / f"emu_{k}.cpp")
        exe = str(root / f"emu_{k}")
        subprocess.run(["g++", "-std=c++20", "-O1", "-pthread", "-w", "-ffp-contract=off", "-I", str(root),
                        str(root / f"emu_{k}.cpp"),
                        "-o", exe], check=True)
        bins[k] = exe
    if "dmr" in bins:  # the refinement predicates alone, from the same generated text
        shutil.copy(os.path.join(EMU, "emu_dmr_predicates.cpp"), root / "emu_dmr_predicates.cpp")
        exe = str(root / "emu_dmr_predicates")
        subprocess.run(["g++", "-std=c++20", "-O2", "-pthread", "-w", "-ffp-contract=off", "-I", str(root),
                        str(root / "emu_dmr_predicates.cpp"), "-o", exe], check=True)
        bins["dmr_predicates"] = exe
    return root, bins


def _run(emu, kernel, *args):
    root, bins = emu
    if kernel not in bins:
        pytest.skip(f"no harness for {kernel}")
    r = subprocess.run([bins[kernel], str(root / args[0]), *map(str, args[1:])], capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " bad=0" in r.stdout and "err=0" in r.stdout, r.stdout


# graph, blocks, source row, sssp, unit_iters, delta, bottom-up, alpha, beta, light/heavy,
# pulling bucket closes (0 never, 1 cost rule, 2 always), far-pile size that ends the buckets
FRONTIER = [
    ("r10", 4, 0, 0, 8, 0, 1, 15, 18, 0, 0, 0),
    ("r10", 3, 3, 0, 2, 0, 0, 15, 18, 0, 0, 0),
    ("grid", 4, 2, 0, 16, 0, 1, 1000, 1000, 0, 0, 0),
    ("r10", 4, 0, 1, 4, 33, 0, 15, 18, 1, 0, 0),
    ("r10", 2, 9, 1, 2, 64, 0, 15, 18, 1, 1, 64),
    ("grid", 4, 1, 1, 8, 100, 0, 15, 18, 1, 0, 30),
    ("grid", 3, 4, 1, 16, 0, 0, 15, 18, 0, 0, 0),
    ("r10", 4, 7, 1, 4, 1, 0, 15, 18, 1, 0, 0),
    ("r10", 4, 0, 1, 4, 33, 0, 15, 18, 1, 2, 0),
    ("grid", 3, 1, 1, 8, 100, 0, 15, 18, 1, 2, 0),
    ("r10", 2, 7, 1, 2, 1, 0, 15, 18, 1, 2, 200),
    ("r10", 4, 11, 1, 4, 20, 0, 15, 18, 1, 1, 64),
    ("r10", 4, 3, 1, 4, 8, 0, 15, 18, 1, 1, 1024),
    ("grid", 4, 5, 1, 4, 50, 0, 15, 18, 0, 0, 100),
]


@pytest.mark.parametrize("case", FRONTIER, ids=lambda c: "-".join(map(str, c)))
def test_frontier_kernel_text(emu, case):
    _run(emu, "frontier", *case)


@pytest.mark.parametrize("case", [("r10", 4, 32), ("grid", 3, 5)], ids=lambda c: "-".join(map(str, c)))
def test_sssp32_kernel_text(emu, case):
    _run(emu, "sssp32", *case)


# graph, blocks, sources, bottom-up levels allowed
@pytest.mark.parametrize("case", [("r10", 4, 64, 0), ("grid", 2, 7, 0), ("r10", 4, 64, 1), ("r10", 3, 5, 1),
                                  ("grid", 4, 33, 1)], ids=lambda c: "-".join(map(str, c)))
def test_msbfs_kernel_text(emu, case):
    _run(emu, "msbfs", *case)


# graph, blocks, rounds per launch, queries admitted per launch, SSSP delta, pile size that ends a
# query's buckets[, server supersteps]
MQ = [
    ("r10", 4, 1000000, 0, 0, 0),
    ("r10", 4, 1000000, 0, 33, 0),
    ("grid", 4, 1000000, 0, 100, 0),
    ("r10", 3, 2, 3, 16, 0),
    ("grid", 4, 5, 1, 300, 0),
    ("grid", 3, 3, 2, 1, 0),
    ("r10", 4, 1000000, 0, 16, 256),
    ("grid", 3, 3, 2, 50, 120),
    # the server's supersteps: stop at the first finished query, remaining work counted in the launch
    ("r10", 4, 128, 3, 16, 0, 1),
    ("grid", 3, 64, 2, 50, 120, 1),
    ("r10", 2, 1000000, 0, 0, 0, 1),
    # stop once 3 queries finished
    ("r10", 3, 1000000, 0, 16, 0, 3),
    # the server's flow: 4 or 3 slots (20, 19) reused as queries retire
    ("r10", 4, 128, 0, 16, 0, 20),
    ("grid", 3, 64, 0, 50, 120, 19),
]


@pytest.mark.parametrize("case", MQ, ids=lambda c: "-".join(map(str, c)))
def test_batch_kernel_text(emu, case):
    _run(emu, "mq", *case)


# Mesh refinement kernels (dmr.cu): every round's kernels run as emulated
# threads (3 blocks of 64 for the compactions, 2 x 32 planning and commit
# threads, one block of 64 for the tail kernel), and the refined mesh must
# equal the oracle's serial restatement of the same schedule bit for bit:
# points, triangles and neighbours.  tail_max 0 keeps every round on the
# multi-kernel path, 2048 hands the small rounds to the one-block tail
# kernel, 12 makes it hand back and take over again; pf 8 plans rounds of
# more than 8 bad triangles with the lean variant of k_plan.
DMR_CASES = [("jittered", 1 << 20, 0, 32768), ("jittered", 7, 2048, 32768), ("random", 1 << 20, 0, 8),
             ("random", 1 << 20, 12, 8), ("random", 1 << 20, 2048, 32768)]


@pytest.mark.parametrize("case", DMR_CASES, ids=[f"{m}-cap{c}-tail{t}-pf{f}" for m, c, t, f in DMR_CASES])
def test_dmr_kernel_text(emu, case):
    root, bins = emu
    kind, bcap, tail, pf = case
    mesh = oracle.mesh_gen_jittered(14, 12, 0.35, 2) if kind == "jittered" else oracle.mesh_gen_random(120, 5)
    d = root / f"dmr_{kind}_{bcap}_{tail}_{pf}"
    d.mkdir()
    for k in ("x", "y", "tri", "nbr"):
        mesh[k].tofile(d / f"{k}.bin")
    tcap = 4 * (len(mesh["tri"]) // 3) + 65536
    r = subprocess.run([bins["dmr"], str(d), "3", "64", "32", str(bcap), str(tcap), oracle.cos_bound(25.0).hex(),
                        str(tail), str(pf)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = dict(zip(r.stdout.split()[0::2], r.stdout.split()[1::2]))
    want = oracle.mesh_refine(mesh, batch_cap=bcap)
    assert want["status"] == "ok" and want["bad_out"] == 0
    assert fields["stop"] == "1" and fields["err"] == "0"  # done, no index error
    assert (fields["tails"] != "0") == (tail > 0)
    assert int(fields["rounds"]) == want["rounds"] and int(fields["ins"]) == want["insertions"]
    assert int(fields["splits"]) == want["boundary_splits"] and int(fields["bad_in"]) == want["bad_in"]
    for k, dt in (("x", np.float64), ("y", np.float64), ("tri", np.uint32), ("nbr", np.uint32)):
        np.testing.assert_array_equal(np.fromfile(d / f"out_{k}.bin", dt), want[k], err_msg=k)


def test_dmr_filtered_predicates_equal_the_double_ones(emu):
    """The kernels' single-precision predicate filters never decide against the
    double expressions the oracle evaluates, on 400,000 near-degenerate cases
    (points within relative 1e-3 .. 1e-9 of a circumcircle or a line, flat
    triangles, features down to 3e-5, meshes 1000 units from the origin)."""
    root, bins = emu
    r = subprocess.run([bins["dmr_predicates"], "400000", "3"], capture_output=True, text=True, timeout=300)
    f = dict(zip(r.stdout.split()[0::2], r.stdout.split()[1::2]))
    assert r.returncode == 0, r.stdout
    assert f["orient_wrong"] == f["incircle_wrong"] == f["angle_wrong"] == "0"
    assert int(f["orient_fallback_random"]) < 40000 // 20  # float decides almost every ordinary case
