"""Generates clocks.json from the REFERENCE's own combineClocks (metrics.h:68-84).

Runs only on the development host, where the reference sources exist: it
builds oracle/_ref/ref_clocks (``make -C oracle ref_clocks``, which compiles
the reference's metrics.h in place) and records its estimate and SM
assignment for seeded per-block clock arrays (the reference fixes 14 SMs).

    python tests/golden/make_golden_clocks.py
"""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref_clocks"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_clocks")
    rng = np.random.default_rng(68)
    arrays = [[], [7], [3] * 14, [3] * 15, [5, 3, 4, 1, 2]]
    for n in (13, 14, 15, 100, 608):
        arrays.append([int(x) for x in rng.integers(0, 1 << 31, n)])
        arrays.append([int(x) for x in rng.integers(0, 4, n)])  # many ties
    cases = []
    for a in arrays:
        r = subprocess.run([exe], input=f"{len(a)}\n" + " ".join(map(str, a)) + "\n", capture_output=True, text=True,
                           check=True)
        lines = r.stdout.split("\n")
        cases.append({"clocks": a, "estimate": int(lines[0]),
                      "sm": [int(x) for x in lines[1].split()] if len(lines) > 1 else []})
    with open(os.path.join(HERE, "clocks.json"), "w") as f:
        json.dump({"source": "reference combineClocks, metrics.h:68-84 (14 SMs)", "cases": cases}, f)


if __name__ == "__main__":
    main()
