"""Host code built with AddressSanitizer and UndefinedBehaviorSanitizer and run
over sweeps of inputs: the mesh code (csrc/mesh_host.c) with the oracle's
refinement (oracle/mesh_oracle.c) over generated meshes, a file round trip
and refinements (tests/asan/mesh_sweep.c); the graph code (csrc/graph_host.c)
with the BFS/SSSP oracle over R-MAT and grid graphs, .gr round trips,
truncated .gr files, split rules, node splits and traversals
(tests/asan/graph_sweep.c).  A heap overflow in the jittered generator's flip
stack was found this way; the sweeps keep the host side free of
out-of-bounds accesses and undefined behaviour."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CS = os.path.join(ROOT, "gpugraphalgo_gb300", "csrc")


SWEEPS = {
    "mesh": ["tests/asan/mesh_sweep.c", "gpugraphalgo_gb300/csrc/mesh_host.c", "gpugraphalgo_gb300/csrc/graph_host.c",
             "oracle/mesh_oracle.c"],
    "graph": ["tests/asan/graph_sweep.c", "gpugraphalgo_gb300/csrc/graph_host.c", "oracle/gga_oracle.c",
              "oracle/gen_inputs.c"],
}


@pytest.mark.parametrize("which", sorted(SWEEPS))
def test_host_code_under_sanitizers(tmp_path, which):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    exe = str(tmp_path / f"{which}_sweep")
    cmd = ["gcc", "-g", "-O1", "-std=c11", "-pthread", "-ffp-contract=off", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer", "-I", CS] + \
        [os.path.join(ROOT, f) for f in SWEEPS[which]] + ["-lm", "-o", exe]
    b = subprocess.run(cmd, capture_output=True, text=True)
    if b.returncode != 0 and "sanitize" in b.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert b.returncode == 0, b.stderr[-2000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe, str(tmp_path / "m")], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, (r.stdout + r.stderr)[-3000:]
    assert "ok" in r.stdout
