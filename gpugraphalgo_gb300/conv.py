"""Convergence log in the reference's conv.vi format.

The reference's ENABLE_IT_DIST + ENABLE_RTIME_DIST build copies the distances
back after every relax launch and appends to conv.vi: a header naming the
split level, maximum degree, graph and algorithm (printConv_rtime_init,
convergence.h:81-90, called at bfs_sssp.cu:247-249), one line per iteration
with the norm of the difference to the serial answer and the count of
differing vertices (printConv_rtime, convergence.h:100-159, called at
bfs_sssp.cu:420-424), and a footer with the iteration count and the largest
distance (printConv_rtime_final, convergence.h:91-99, bfs_sssp.cu:510-517).

Here the per-iteration figures come from gga_convergence, computed on the
device; the final answer is the frontier engine's (bit-identical to the
serial one).  The reference also lists each differing vertex when fewer than
100 differ; gga_convergence returns counts only, so those lines are not
written.

    python -m gpugraphalgo_gb300.conv graph.gr [--flavour na|n|da|d]
        [--algo bfs|sssp] [--level 0] [--buckets 10] [--src 0] [--out conv.vi]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import INFINITY, Context, Graph

DASHES = "-" * 88
VARIANT = {"na": "topo_atomic", "n": "topo_plain", "da": "cdp_atomic", "d": "cdp_plain"}


def header(level: int, maxdeg: int, graph_name: str, algo: str) -> str:
    """printConv_rtime_init: three blank lines, a rule, the run's name."""
    return "\n\n\n" + DASHES + "\n" + f"Dist_Level_{level}_MaxDeg_{maxdeg}_{graph_name}_{algo}\n"


def iteration_line(it: int, norm2: float, diff_count: int) -> str:
    """printConv_rtime's line: the iteration left-aligned in 3 columns, the
    norm as a C++ stream prints a double (6 significant digits, like %g)."""
    return f"Iteration:{it:<3} = {norm2:g}({diff_count})\n"


def footer(total_iterations: int, max_dist: int) -> str:
    """printConv_rtime_final."""
    return f"Total Iteration : {total_iterations}     Max Dist : {max_dist}\n" + DASHES + "\n"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("graph")
    ap.add_argument("--flavour", default="na", choices=sorted(VARIANT))
    ap.add_argument("--algo", default="sssp", choices=["bfs", "sssp"])
    ap.add_argument("--level", type=int, default=0)
    ap.add_argument("--buckets", type=int, default=10)
    ap.add_argument("--src", type=int, default=0)
    ap.add_argument("--out", default="conv.vi")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    g = Graph.readFromGR(a.graph)
    ctx = Context(a.device)
    try:
        g.cudaCopy(ctx)
        maxdeg = g.info()["maxdeg"]  # of the graph as read, as the reference's header has it
        if a.level and a.flavour in ("na", "n"):
            g.node_split(ctx, a.level, a.buckets)
        elif a.level:  # the CDP flavours take their heavy-vertex threshold from the level
            ctx.set_params(cdp_level=a.level, cdp_buckets=a.buckets)
        final = ctx.solve(g, a.algo, a.src, "frontier")
        recs, _ = ctx.convergence(g, a.algo, a.src, final, VARIANT[a.flavour])
        reached = final[final < INFINITY]
        with open(a.out, "a") as f:
            f.write(header(a.level, maxdeg, os.path.basename(a.graph), a.algo.upper()))
            for r in recs:
                f.write(iteration_line(r["iteration"], r["norm2"], r["diff_count"]))
            f.write(footer(len(recs), int(reached.max()) if len(reached) else 0))
    finally:
        ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
