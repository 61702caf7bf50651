"""Split-level sweep: the counterpart of the reference's `mysc` driver script
(K/mysc:20-51), which runs every flavour (d_/da_/n_/na_ x bfs/sssp) on each
graph for node-split levels 1..40 and then for the histogram rule with
buckets 2, 5, 10 and 15, one process per point, each appending its row to
result.vi (writeResult, K/myutils.h:86-113).

Here one process keeps the graph resident and re-splits it on the device per
point (gga_node_split), so a 40-level sweep costs seconds, and the rows have
the reference's 17 columns.  The frontier engine ("gga") can be swept beside
the reference's flavours, and with --autotune each point also records the
parameters gga_autotune picks for the split graph.

    python -m gpugraphalgo_gb300.sweep graph.gr [--flavours na,n,da,d,gga]
        [--algos bfs,sssp] [--levels 1-40] [--buckets 2,5,10,15]
        [--out result.vi] [--src 0] [--autotune]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import GGAError, Context, Graph, ERR_SPLIT_RULE, writeResult

VARIANT = {"na": "topo_atomic", "n": "topo_plain", "da": "cdp_atomic", "d": "cdp_plain", "gga": "frontier"}


def _levels(spec: str):
    out = []
    for part in spec.split(","):
        if "-" in part[1:]:
            a, b = part.split("-", 1)
            out += list(range(int(a), int(b) + 1))
        elif part:
            out.append(int(part))
    return out


def sweep_points(levels, buckets):
    """(level, buckets) pairs in the reference's order: levels first, then the
    histogram rule (level -1) per bucket count."""
    return [(lv, 10) for lv in levels] + [(-1, b) for b in buckets]


def run_point(ctx: Context, g: Graph, flavour: str, algo: str, level: int, buckets: int, src: int = 0,
              graph_name: str = "graph", autotune: bool = False) -> dict:
    """One sweep point; returns the result-row fields (plus 'error')."""
    variant = VARIANT[flavour]
    cdp = variant.startswith("cdp")
    info0 = g.info()
    row = {"exename": f"{flavour}_{algo}", "algo": algo.upper(), "graphfile": graph_name,
           "bucket_size": buckets if level < 0 else 0, "nnode": info0["nodes_orig"], "nedge": info0["nedges"],
           "maxdeg": info0["maxdeg"], "splitlevel": level & 0xFFFFFFFF}
    try:
        if cdp:
            g.NodeSplit(ctx, 0)
            ctx.set_params(cdp_level=level, cdp_buckets=buckets)
            mda = 0
        else:
            g.NodeSplit(ctx, level, buckets)
            mda = g.info()["mda"]
        if autotune:
            row["params"] = ctx.autotune(g, 1)
            if not cdp:  # the tuner's trials re-split the graph: back to this point's split
                g.NodeSplit(ctx, level, buckets)
        _, st = ctx.solve(g, algo, src, variant, stats=True)
    except GGAError as e:
        row["error"] = "split rule divides by zero" if e.status == ERR_SPLIT_RULE else str(e)
        return row
    finally:
        if not autotune:
            ctx.reset_params()
    info = g.info()
    row.update(ns_nnode=info["nnodes"], ns_nedge=info["nedges"], extranode=info["nnodes"] - info0["nodes_orig"],
               max_edges_allowed=mda, iterations=st["iterations"], runtime=int(st["total_ms"]),
               time=st["kernel_ms"] + st["aux_ms"], ktime=st["kernel_ms"], sktime=st["aux_ms"])
    return row


ROW_KEYS = ("exename", "algo", "graphfile", "bucket_size", "nnode", "nedge", "ns_nnode", "ns_nedge", "extranode",
            "maxdeg", "splitlevel", "max_edges_allowed", "iterations", "runtime", "time", "ktime", "sktime")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("graph")
    ap.add_argument("--flavours", default="d,da,n,na")
    ap.add_argument("--algos", default="bfs,sssp")
    ap.add_argument("--levels", default="1-40")
    ap.add_argument("--buckets", default="2,5,10,15")
    ap.add_argument("--out", default="result.vi")
    ap.add_argument("--src", type=int, default=0)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--autotune", action="store_true")
    a = ap.parse_args(argv)
    g = Graph.readFromGR(a.graph)
    name = os.path.basename(a.graph)
    ctx = Context(a.device)
    g.cudaCopy(ctx)
    points = sweep_points(_levels(a.levels), [int(b) for b in a.buckets.split(",") if b])
    failures = 0
    for flavour in a.flavours.split(","):
        for algo in a.algos.split(","):
            best = None
            for level, buckets in points:
                r = run_point(ctx, g, flavour, algo, level, buckets, a.src, name, a.autotune)
                if "error" in r:
                    print(f"{flavour}_{algo} level {level} buckets {buckets}: {r['error']}")
                    failures += "split rule" not in r["error"]
                    continue
                writeResult(a.out, **{k: r[k] for k in ROW_KEYS})
                print(f"{flavour}_{algo} level {level:3d} buckets {buckets:2d} MDA {r['max_edges_allowed']:8d} "
                      f"nodes {r['ns_nnode']:9d} iterations {r['iterations']:5d} time {r['time']:9.3f} ms")
                if best is None or r["time"] < best["time"]:
                    best = r
            if best:
                print(f"best {flavour}_{algo}: level {best['splitlevel'] if best['splitlevel'] < 2**31 else -1} "
                      f"MDA {best['max_edges_allowed']} time {best['time']:.3f} ms")
    g.NodeSplit(ctx, 0)
    ctx.close()
    return 1 if failures else 0


if __name__ == "__main__":
    sys.exit(main())
