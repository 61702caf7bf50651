"""Delaunay mesh refinement on the GPU (the reference's DMR program,
Kepler_DMR/dmr.cu) against the oracle's serial restatement of the same round
schedule (oracle/mesh_oracle.c): the refined points, triangles and neighbour
links must be identical bit for bit, and the refined mesh must have the
properties the reference's verification checks (dverify, dmr.cu:371-391: no
bad triangle left) plus those of a valid Delaunay mesh (counter-clockwise
triangles, mutual neighbour links, every interior edge locally Delaunay, the
domain's area unchanged)."""
from __future__ import annotations

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle

pytestmark = pytest.mark.gpu


def _assert_same(got: dict, want: dict):
    for k in ("x", "y", "tri", "nbr"):
        assert len(got[k]) == len(want[k]), k
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)


def _assert_valid(mesh: gga.Mesh, area: float, min_angle: float = 25.0):
    c = mesh.check(min_angle)
    assert c["bad_triangles"] == 0
    assert c["bad_orientation"] == 0 and c["bad_neighbors"] == 0 and c["non_delaunay_edges"] == 0
    assert abs(c["area"] - area) < 1e-9
    a = mesh.arrays()
    # the neighbour links are exactly the ones derived from the triangles
    assert oracle.mesh_check(a, min_angle)["nbr_consistent"]


@pytest.mark.parametrize("kind,size,bcap", [("random", 20000, 0), ("random", 3000, 5), ("jittered", 120, 0),
                                            ("jittered", 60, 1)])
def test_refine_matches_oracle_bit_for_bit(ctx, kind, size, bcap):
    mesh = gga.Mesh.random(size, seed=11) if kind == "random" else gga.Mesh.jittered(size, size, 0.35, seed=4)
    before = mesh.arrays()
    area = mesh.check()["area"]
    st = ctx.refine(mesh, batch_cap=bcap)
    want = oracle.mesh_refine(before, batch_cap=bcap or (1 << 20))
    assert want["status"] == "ok"
    _assert_same(mesh.arrays(), want)
    assert st["bad_out"] == 0 and st["bad_in"] == want["bad_in"] > 0
    assert st["rounds"] == want["rounds"]
    assert st["insertions"] == want["insertions"] and st["boundary_splits"] == want["boundary_splits"]
    assert st["triangles_out"] == len(want["tri"]) // 3 and st["points_out"] == len(want["x"])
    assert st["device_ms"] > 0 and st["total_ms"] >= st["device_ms"]
    _assert_valid(mesh, area)


@pytest.mark.parametrize("tail_max,prefetch_max", [(0xFFFFFFFF, 0), (16, 0), (0, 1), (0, 1 << 30), (7, 1)],
                         ids=["no-tail", "tail-hand-back", "lean-plans", "prefetch-plans", "hand-back-lean"])
def test_refine_schedule_knobs_never_change_the_result(ctx, tail_max, prefetch_max):
    """Every round on the multi-kernel path, the one-block tail kernel taking
    over and handing back, and either planning variant: the same mesh as the
    oracle's."""
    mesh = gga.Mesh.random(12000, seed=21)
    before = mesh.arrays()
    st = ctx.refine(mesh, tail_max=tail_max, prefetch_max=prefetch_max)
    want = oracle.mesh_refine(before)
    _assert_same(mesh.arrays(), want)
    assert st["rounds"] == want["rounds"] and st["bad_out"] == 0


def test_refine_is_repeatable(ctx):
    a, b = gga.Mesh.random(5000, seed=2), gga.Mesh.random(5000, seed=2)
    ctx.refine(a)
    ctx.refine(b)
    _assert_same(a.arrays(), b.arrays())


@pytest.mark.parametrize("angle", [20.0, 28.0])
def test_refine_other_angle_bounds(ctx, angle):
    mesh = gga.Mesh.random(4000, seed=7)
    before = mesh.arrays()
    area = mesh.check()["area"]
    ctx.refine(mesh, min_angle_deg=angle)
    want = oracle.mesh_refine(before, min_angle_deg=angle)
    _assert_same(mesh.arrays(), want)
    _assert_valid(mesh, area, angle)


def test_refine_capacity_limit_keeps_last_complete_round(ctx):
    mesh = gga.Mesh.random(3000, seed=3)
    before = mesh.arrays()
    ntri = len(before["tri"]) // 3
    cap = ntri + 3000
    with pytest.raises(gga.GGAError) as ex:
        ctx.refine(mesh, max_triangles=cap)
    assert ex.value.status == gga.ERR_TOO_LARGE
    want = oracle.mesh_refine(before, max_triangles=cap)
    assert want["status"] == "capacity"
    _assert_same(mesh.arrays(), want)
    c = mesh.check()
    assert c["bad_orientation"] == 0 and c["bad_neighbors"] == 0 and c["non_delaunay_edges"] == 0
    assert 0 < c["bad_triangles"] and len(mesh.arrays()["tri"]) // 3 <= cap
    # a second call with room finishes the job from there
    ctx.refine(mesh)
    assert mesh.check()["bad_triangles"] == 0


def test_refine_loaded_triangle_files(ctx, tmp_path):
    src = gga.Mesh.random(2500, seed=9)
    base = str(tmp_path / "r2500")
    src.save(base)
    mesh = gga.Mesh.load(base)
    before = mesh.arrays()
    ctx.refine(mesh)
    _assert_same(mesh.arrays(), oracle.mesh_refine(before))
    out = str(tmp_path / "refined")
    mesh.save(out)
    again = gga.Mesh.load(out)
    _assert_same(again.arrays(), mesh.arrays())


def test_refine_mesh_without_bad_triangles_is_unchanged(ctx):
    # an equilateral-ish strip: every angle near 60 degrees
    x = np.array([0.0, 1.0, 0.5, 1.5], np.float64)
    y = np.array([0.0, 0.0, 0.8660254, 0.8660254], np.float64)
    mesh = gga.Mesh.from_arrays(x, y, np.array([0, 1, 2, 1, 3, 2], np.uint32))
    before = mesh.arrays()
    st = ctx.refine(mesh)
    assert st["bad_in"] == 0 and st["rounds"] == 0
    _assert_same(mesh.arrays(), before)


def test_refine_larger_random_mesh(ctx):
    """200k random points (400k triangles, about a third of them bad)."""
    mesh = gga.Mesh.random(200000, seed=1)
    before = mesh.arrays()
    st = ctx.refine(mesh)
    want = oracle.mesh_refine(before)
    _assert_same(mesh.arrays(), want)
    assert st["bad_out"] == 0 and st["failed_plans"] == want["failed_plans"]
    _assert_valid(mesh, 1.0)


def test_refine_rejects_bad_arguments(ctx):
    mesh = gga.Mesh.random(100, seed=1)
    with pytest.raises(gga.GGAError) as ex:
        ctx.refine(mesh, min_angle_deg=75.0)
    assert ex.value.status == gga.ERR_INVALID_ARG
    with pytest.raises(gga.GGAError) as ex:
        ctx.refine(mesh, max_triangles=10)
    assert ex.value.status == gga.ERR_INVALID_ARG


def test_dmr_cli_drop_in(tmp_path):
    """r_dmr <basefilename> (dmr.cu:81-84): the reference's summary lines and
    its 9-column result.vi row; GGA_DMR_OUT writes the refined mesh, which
    equals the oracle's refinement of the input."""
    import os
    import subprocess

    src = gga.Mesh.random(3000, seed=12)
    base = str(tmp_path / "r3000")
    src.save(base)
    before = src.arrays()
    exe = os.path.join(os.path.dirname(gga.__file__), "bin", "r_dmr")
    env = dict(os.environ, GGA_DMR_OUT=str(tmp_path / "out"))
    r = subprocess.run([exe, base], cwd=tmp_path, capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "reading graphs..." and lines[1].strip() == "3004 nodes"
    assert lines[2].strip() == f"{2 * 3004 - 6} triangles."
    assert "verification succeeded: 0 bad triangles exist." in lines
    want = oracle.mesh_refine(before)
    row = (tmp_path / "result.vi").read_text().strip().split(",")
    assert row[:7] == ["r_dmr", "r3000", str(2 * 3004 - 6), str(want["bad_in"]), str(len(want["tri"]) // 3), "0",
                       str(want["rounds"])]
    assert float(row[7]) >= float(row[8]) > 0 and row[9] == ""
    got = gga.Mesh.load(str(tmp_path / "out")).arrays()
    for k in ("x", "y", "tri"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
