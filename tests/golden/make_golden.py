"""Generates the golden fixtures in this folder from the REFERENCE's own code.

Runs only on the development host, where the reference sources exist: it
builds oracle/_ref (``make -C oracle ref``, which compiles the reference's
graph.h and myutils.h in place), writes each fixture graph as a Galois .gr,
runs the reference's readFromGR -> findSerialBFS/SSSP -> NodeSplit ->
verifysolution -> Ary2File through oracle/_ref/ref_{bfs,sssp}, and records
the outputs.  Graphs are either tiny hand-built CSRs (stored whole) or
seeded generator graphs (stored as generator parameters plus a digest of the
CSR, so a generator change is detected).

    python tests/golden/make_golden.py

Outputs: golden.json (metadata, digests) and golden_arrays.npz (arrays).
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import gpugraphalgo_gb300 as gga  # noqa: E402  (host generator only, no GPU)
import oracle  # noqa: E402


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def csr_digest(off, col, wt) -> str:
    h = hashlib.sha256()
    for a in (off, col, wt):
        h.update(np.ascontiguousarray(a, dtype="<u4").tobytes())
    return h.hexdigest()


def hand_graphs():
    """Small hand-built CSRs (directed)."""
    out = {}
    # analogue of Graph::testgraph (graph.h:557-598): 0->{1,2,3}, 2->{4..8}, 3->{9,10}
    adj = {0: [1, 2, 3], 2: [4, 5, 6, 7, 8], 3: [9, 10]}
    off, col = [0], []
    for u in range(11):
        col += adj.get(u, [])
        off.append(len(col))
    out["testgraph11"] = (np.array(off), np.array(col), np.arange(1, len(col) + 1))
    # hub graph with zero-degree vertices and an unreachable island; odd m
    rng = np.random.default_rng(5)
    n = 40
    edges = set()
    for v in range(1, 30):
        edges.add((0, v))
        edges.add((v, 0))
    for _ in range(60):
        a, b = rng.integers(1, 34, 2)
        if a != b:
            edges.add((int(a), int(b)))
    edges.add((36, 37))
    edges.add((37, 38))
    edges.add((5, 0))
    edges = sorted(edges)
    if len(edges) % 2 == 0:
        edges.append((38, 36))
    off = np.zeros(n + 1, np.int64)
    for a, _ in edges:
        off[a + 1] += 1
    off = np.cumsum(off)
    col = np.array([b for _, b in edges])
    wt = rng.integers(1, 255, len(col))
    out["hub40_oddm"] = (off, col, wt)
    # zero weights and a chain (deep BFS)
    n = 64
    e = [(i, i + 1) for i in range(n - 1)] + [(i + 1, i) for i in range(n - 1)] + [(0, 63), (10, 50)]
    e = sorted(set(e))
    off = np.zeros(n + 1, np.int64)
    for a, _ in e:
        off[a + 1] += 1
    off = np.cumsum(off)
    col = np.array([b for _, b in e])
    wt = np.array([(a * 7 + b * 3) % 5 for a, b in e])  # includes zeros
    out["chain64_zero_w"] = (off, col, wt)
    return out


GEN_GRAPHS = {
    # name: (kind, params)
    "rmat10": ("rmat", dict(scale=10, edge_factor=8, seed=7, wmin=1, wmax=255)),
    "c1_rmat14": ("rmat", dict(scale=14, edge_factor=8, seed=1, wmin=1, wmax=255)),
    "rmat12_ef16": ("rmat", dict(scale=12, edge_factor=16, seed=11, wmin=1, wmax=255)),
    "grid64": ("grid", dict(width=64, height=64, del_prob=0.05, longrange_frac=0.001, seed=3, wmin=1, wmax=1000)),
}

SPLITS = [(0, 10), (1, 10), (2, 10), (3, 10), (7, 10), (40, 10), (-1, 10), (-1, 2), (-1, 5), (-1, 15)]


def make_graph(kind, p):
    if kind == "rmat":
        return gga.Graph.rmat(p["scale"], p["edge_factor"], seed=p["seed"], wmin=p["wmin"], wmax=p["wmax"])
    return gga.Graph.grid(p["width"], p["height"], p["del_prob"], p["longrange_frac"], seed=p["seed"], wmin=p["wmin"], wmax=p["wmax"])


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so", "ref"], check=True)
    assert oracle.ref_available(), "oracle/_ref not built"
    meta = {"graphs": {}}
    arrays = {}
    work = tempfile.mkdtemp(prefix="gga_golden_")
    graphs = {}
    for name, (off, col, wt) in hand_graphs().items():
        graphs[name] = ("csr", None, gga.Graph.from_csr(off, col, wt))
    for name, (kind, p) in GEN_GRAPHS.items():
        graphs[name] = (kind, p, make_graph(kind, p))
    for name, (kind, p, g) in graphs.items():
        off, col, wt = g.csr()
        n, m = len(off) - 1, len(col)
        deg = np.diff(off.astype(np.int64))
        gr = os.path.join(work, f"{name}.gr")
        g.save_gr(gr)
        entry = {"kind": kind, "params": p, "n": n, "m": m, "maxdeg": int(deg.max()),
                 "csr_sha256": csr_digest(off, col, wt), "dist": {}, "split": {}}
        if kind == "csr":
            arrays[f"{name}/off"] = off.astype(np.uint32)
            arrays[f"{name}/col"] = col.astype(np.uint32)
            arrays[f"{name}/wt"] = wt.astype(np.uint32)
        srcs = sorted({0, int(np.argmax(deg))})
        for algo in ("bfs", "sssp"):
            for src in srcs:
                r = oracle.run_reference(gr, algo, 0, 10, src)
                assert r["returncode"] == 0, r["stdout"][-500:]
                key = f"{algo}/{src}"
                entry["dist"][key] = {"sha256": digest(r["dist"]), "max_dist": r["max_dist"], "nerr": r["nerr"],
                                      "ary_txt_sha256": hashlib.sha256(r["ary_txt"].encode()).hexdigest()}
                arrays[f"{name}/dist/{key}"] = r["dist"]
        for level, buckets in SPLITS:
            if level == 0:
                continue
            src = srcs[-1]
            r = oracle.run_reference(gr, "sssp", level, buckets, src)
            key = f"{level}/{buckets}"
            if r["returncode"] != 0:
                entry["split"][key] = {"returncode": r["returncode"],
                                       "crash": "SIGFPE" if r["returncode"] == -8 else "other"}
                continue
            rec = {"returncode": 0, "mda": r["mda"], "nnodes": r["nnodes"], "nerr_sssp": r["nerr"], "src": src,
                   "ary_txt_sha256": hashlib.sha256(r["ary_txt"].encode()).hexdigest()}
            for k in ("psrc", "noutgoing", "childCount", "IsParent", "parentNode"):
                rec[f"{k}_sha256"] = digest(r[k])
            rec["edgessrcdst_sha256"] = digest(r["edgessrcdst"][1:])  # slot 0 is uninitialised in the reference
            if n <= 5000:
                for k in ("psrc", "noutgoing", "childCount", "IsParent", "parentNode"):
                    arrays[f"{name}/split/{key}/{k}"] = r[k]
            entry["split"][key] = rec
        meta["graphs"][name] = entry
        print(name, n, m, "maxdeg", entry["maxdeg"], "splits",
              {k: v.get("mda", v.get("crash")) for k, v in entry["split"].items()})
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_arrays.npz"), **arrays)
    subprocess.run(["rm", "-rf", work])


if __name__ == "__main__":
    main()
