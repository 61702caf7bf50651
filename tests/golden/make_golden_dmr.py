"""Generates tests/golden/dmr_io.json from the REFERENCE DMR program's own host
code: its mesh readers (readNodes / readTriangles, Kepler_DMR/helpers.h:5-63)
and its result row (getname / writeResult, Kepler_DMR/myresult.h:13-52),
compiled in place into oracle/_ref/ref_dmr_io (``make -C oracle ref_dmr``).

Runs only on the development host, where the reference sources exist.  Each
fixture mesh is written by this library's saver (plus a .poly listing its
boundary edges, which the reference's reader requires); the file texts, what
the reference parsed from them and the row its writeResult appended are
stored, so tests/test_mesh_host.py can check this library's loader and CLI row
against them anywhere.

    python tests/golden/make_golden_dmr.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import gpugraphalgo_gb300 as gga  # noqa: E402  (host mesh code only, no GPU)

REF = os.path.join(ROOT, "oracle", "_ref", "ref_dmr_io")
NONE = 0xFFFFFFFF


def boundary_edges(a: dict):
    tri, nbr = a["tri"].reshape(-1, 3), a["nbr"].reshape(-1, 3)
    out = []
    for t in range(len(tri)):
        for i in range(3):
            if nbr[t, i] == NONE:
                out.append((int(tri[t, (i + 1) % 3]), int(tri[t, (i + 2) % 3])))
    return out


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref_dmr"], check=True)
    cases = {"jittered6x5": gga.Mesh.jittered(6, 5, 0.3, seed=1), "random60": gga.Mesh.random(60, seed=2)}
    fixtures = {}
    with tempfile.TemporaryDirectory() as td:
        for name, mesh in cases.items():
            base = os.path.join(td, name)
            mesh.save(base)
            a = mesh.arrays()
            segs = boundary_edges(a)
            with open(base + ".poly", "w") as f:
                f.write("0 2 0 0\n%d 1\n" % len(segs))
                for i, (p, q) in enumerate(segs):
                    f.write("%d %d %d 1\n" % (i, p, q))
            fields = [len(a["tri"]) // 3, 7, 3 * (len(a["tri"]) // 3), 0, 5, "12.5", "3.25"]
            out = os.path.join(td, name + "_ref")
            subprocess.run([REF, base, out, "/opt/bin/r_dmr"] + [str(x) for x in fields], cwd=td, check=True,
                           stdout=subprocess.DEVNULL)
            meta = dict(line.strip().split("=") for line in open(out + ".meta"))
            nn, nt = int(meta["nnodes"]), int(meta["ntriangles"])
            fixtures[name] = {
                "node": open(base + ".node").read(), "ele": open(base + ".ele").read(),
                "poly": open(base + ".poly").read(),
                "ref_nnodes": nn, "ref_ntriangles": nt,
                "ref_x": np.fromfile(out + ".x", "<f4").tolist(), "ref_y": np.fromfile(out + ".y", "<f4").tolist(),
                "ref_tri": np.fromfile(out + ".tri", "<u4").tolist(),
                "row_fields": fields,
            }
        fixtures["result_vi"] = open(os.path.join(td, "result.vi")).read()
    with open(os.path.join(HERE, "dmr_io.json"), "w") as f:
        json.dump(fixtures, f)
    print("wrote", os.path.join(HERE, "dmr_io.json"), {k: len(v) if isinstance(v, str) else None for k, v in fixtures.items()})


if __name__ == "__main__":
    main()
