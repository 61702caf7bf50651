"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: large graphs")


def _ensure_built():
    lib = os.path.join(ROOT, "gpugraphalgo_gb300", "libgga.so")
    if not os.path.exists(lib):
        subprocess.run(["make", "-s", "-j", "-C", os.path.join(ROOT, "gpugraphalgo_gb300", "csrc")], check=True)
    if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)


_ensure_built()


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, "golden_arrays.npz")))
    return meta, arrays


def build_golden_graph(name, entry, arrays):
    import gpugraphalgo_gb300 as gga

    if entry["kind"] == "csr":
        return gga.Graph.from_csr(arrays[f"{name}/off"], arrays[f"{name}/col"], arrays[f"{name}/wt"])
    p = entry["params"]
    if entry["kind"] == "rmat":
        return gga.Graph.rmat(p["scale"], p["edge_factor"], seed=p["seed"], wmin=p["wmin"], wmax=p["wmax"])
    return gga.Graph.grid(p["width"], p["height"], p["del_prob"], p["longrange_frac"], seed=p["seed"],
                          wmin=p["wmin"], wmax=p["wmax"])


@pytest.fixture(scope="session")
def ctx():
    import gpugraphalgo_gb300 as gga

    c = gga.Context(0)
    yield c
    c.close()
