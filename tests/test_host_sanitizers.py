"""The host mesh code (csrc/mesh_host.c, with csrc/graph_host.c's helpers) and
the oracle's refinement (oracle/mesh_oracle.c) built with AddressSanitizer
and UndefinedBehaviorSanitizer and run over a sweep of generated meshes, a
file round trip and refinements (tests/asan/mesh_sweep.c).  A heap overflow
in the jittered generator's flip stack was found this way; the sweep keeps
the host side free of out-of-bounds accesses."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CS = os.path.join(ROOT, "gpugraphalgo_gb300", "csrc")


def test_mesh_host_and_oracle_under_sanitizers(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    exe = str(tmp_path / "mesh_sweep")
    cmd = ["gcc", "-g", "-O1", "-std=c11", "-pthread", "-ffp-contract=off", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer", "-I", CS,
           os.path.join(ROOT, "tests", "asan", "mesh_sweep.c"), os.path.join(CS, "mesh_host.c"),
           os.path.join(CS, "graph_host.c"), os.path.join(ROOT, "oracle", "mesh_oracle.c"), "-lm", "-o", exe]
    b = subprocess.run(cmd, capture_output=True, text=True)
    if b.returncode != 0 and "sanitize" in b.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert b.returncode == 0, b.stderr[-2000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe, str(tmp_path / "m")], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, (r.stdout + r.stderr)[-3000:]
    assert "ok" in r.stdout
