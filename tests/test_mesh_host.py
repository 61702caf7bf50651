"""Host side of Delaunay mesh refinement, no GPU: the mesh generators, the
Triangle-format reader and writer (readNodes / readTriangles of the
reference's Kepler_DMR/helpers.h:5-63), the mesh checker, and the oracle's
serial refinement (oracle/mesh_oracle.c), which the GPU is compared with bit
for bit.

The reference ships no mesh files and no expected outputs for DMR, and its
own result depends on its thread schedule (which of two conflicting cavities
wins), so the oracle is pinned by the properties the reference verifies
(no triangle with an angle below MINANGLE, dmr.cu:371-391) and by those of a
valid refinement: counter-clockwise triangles, mutual neighbour links, every
interior edge locally Delaunay, the domain's area unchanged."""
from __future__ import annotations

import math

import numpy as np
import pytest

import gpugraphalgo_gb300 as gga
import oracle


def _angles_deg(m: dict) -> np.ndarray:
    """Every triangle's three angles by arccos, in numpy (independent of the C code)."""
    t = m["tri"].reshape(-1, 3).astype(np.int64)
    P = np.stack([m["x"], m["y"]], 1)
    out = []
    for i in range(3):
        p, q, r = P[t[:, i]], P[t[:, (i + 1) % 3]], P[t[:, (i + 2) % 3]]
        u, w = q - p, r - p
        c = (u * w).sum(1) / np.sqrt((u * u).sum(1) * (w * w).sum(1))
        out.append(np.degrees(np.arccos(np.clip(c, -1, 1))))
    return np.stack(out, 1)


def _valid(m: dict, min_angle: float = 25.0, area: float = 1.0) -> dict:
    c = oracle.mesh_check(m, min_angle)
    assert c["valid"] and c["tri_ccw"] and c["nbr_consistent"]
    assert c["bad_orientation"] == 0 and c["bad_neighbors"] == 0 and c["non_delaunay_edges"] == 0
    assert abs(c["area"] - area) < 1e-9
    return c


@pytest.mark.parametrize("kind", ["random", "jittered"])
def test_generators_give_delaunay_meshes_and_match_the_oracle_build(kind):
    if kind == "random":
        g, o = gga.Mesh.random(3000, seed=4), oracle.mesh_gen_random(3000, 4)
        assert g.info() == {"npoints": 3004, "ntriangles": 2 * 3004 - 6}
    else:
        g, o = gga.Mesh.jittered(40, 30, 0.3, seed=4), oracle.mesh_gen_jittered(40, 30, 0.3, 4)
        assert g.info() == {"npoints": 1200, "ntriangles": 2 * 39 * 29}
    a = g.arrays()
    for k in ("x", "y", "tri", "nbr"):
        np.testing.assert_array_equal(a[k], o[k])
    c = _valid(a)
    assert c["bad_triangles"] > 0
    assert c == {**c, **{k: v for k, v in g.check().items() if k != "area"}}


def test_generators_reject_bad_arguments():
    with pytest.raises(gga.GGAError) as ex:
        gga.Mesh.jittered(1, 5)
    assert ex.value.status == gga.ERR_INVALID_ARG
    with pytest.raises(gga.GGAError):
        gga.Mesh.jittered(10, 10, jitter=0.5)


def test_bad_triangle_count_matches_angles_computed_independently():
    m = oracle.mesh_gen_random(20000, 8)
    ang = _angles_deg(m).min(1)
    keep = np.abs(ang - 25.0) > 1e-6  # leave out triangles within rounding of the bound
    bad = gga.Mesh.from_arrays(m["x"], m["y"], m["tri"]).check(25.0)["bad_triangles"]
    want = int((ang < 25.0).sum())
    assert abs(bad - want) <= int((~keep).sum())
    assert oracle.mesh_count_bad(m) == bad


def test_triangle_files_round_trip(tmp_path):
    m = gga.Mesh.random(500, seed=2)
    base = str(tmp_path / "m")
    m.save(base)
    (tmp_path / "m.poly").write_text("0 2 0 0\n4 0\n0 0 1 0\n")  # a .poly beside it is ignored
    back = gga.Mesh.load(base)
    a, b = m.arrays(), back.arrays()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    first = (tmp_path / "m.node").read_text().splitlines()[0].split()
    assert first[0] == "504" and (tmp_path / "m.ele").read_text().splitlines()[0].split()[0] == str(2 * 504 - 6)


def _write(tmp_path, name, nodes, eles):
    base = tmp_path / name
    (tmp_path / f"{name}.node").write_text(f"{len(nodes)} 2 0 0\n" + "".join(
        f"{i} {x!r} {y!r}\n" for i, (x, y) in enumerate(nodes)))
    (tmp_path / f"{name}.ele").write_text(f"{len(eles)} 3 0\n" + "".join(
        f"{i} {a} {b} {c}\n" for i, (a, b, c) in enumerate(eles)))
    return str(base)


SQUARE = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]


def test_loader_orders_triangles_counter_clockwise_and_links_neighbours(tmp_path):
    base = _write(tmp_path, "sq", SQUARE, [(0, 2, 1), (0, 2, 3)])  # the first is clockwise
    m = gga.Mesh.load(base)
    a = m.arrays()
    np.testing.assert_array_equal(a["tri"], [0, 1, 2, 0, 2, 3])
    np.testing.assert_array_equal(a["nbr"], [gga.MESH_NONE, 1, gga.MESH_NONE, gga.MESH_NONE, gga.MESH_NONE, 0])
    c = m.check()
    assert c["boundary_edges"] == 4 and c["area"] == 1.0 and c["bad_triangles"] == 0


@pytest.mark.parametrize("nodes,eles,what", [
    (SQUARE, [(0, 1, 7)], "point id out of range"),
    (SQUARE, [(0, 1, 1)], "degenerate triangle"),
    ([(0.0, 0.0), (1.0, 0.0), (2.0, 0.0)], [(0, 1, 2)], "collinear points"),
    (SQUARE + [(0.5, -1.0)], [(0, 1, 2), (0, 2, 3), (0, 4, 1), (1, 0, 3)], "edge shared by three triangles"),
])
def test_loader_rejects_malformed_meshes(tmp_path, nodes, eles, what):
    base = _write(tmp_path, "bad", nodes, eles)
    with pytest.raises(gga.GGAError) as ex:
        gga.Mesh.load(base)
    assert ex.value.status == gga.ERR_FORMAT, what


def test_loader_reports_missing_and_truncated_files(tmp_path):
    with pytest.raises(gga.GGAError) as ex:
        gga.Mesh.load(str(tmp_path / "none"))
    assert ex.value.status == gga.ERR_IO
    (tmp_path / "t.node").write_text("4 2 0 0\n0 0 0\n1 1 0\n")  # two of four points
    (tmp_path / "t.ele").write_text("1 3 0\n0 0 1 2\n")
    with pytest.raises(gga.GGAError) as ex:
        gga.Mesh.load(str(tmp_path / "t"))
    assert ex.value.status == gga.ERR_FORMAT


def test_from_arrays_checks_ids():
    with pytest.raises(gga.GGAError) as ex:
        gga.Mesh.from_arrays([0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [0, 1, 3])
    assert ex.value.status == gga.ERR_FORMAT


@pytest.mark.parametrize("kind,size", [("random", 4000), ("jittered", 70)])
def test_oracle_refinement_leaves_a_valid_mesh_without_bad_triangles(kind, size):
    m = oracle.mesh_gen_random(size, 6) if kind == "random" else oracle.mesh_gen_jittered(size, size, 0.35, 6)
    bad0 = oracle.mesh_count_bad(m)
    r = oracle.mesh_refine(m)
    assert r["status"] == "ok" and r["bad_in"] == bad0 > 0 and r["bad_out"] == 0
    c = _valid(r)
    assert c["bad_triangles"] == 0
    assert _angles_deg(r).min() >= 25.0 - 1e-9
    # every inserted point is new (one per insertion or boundary split)
    assert len(r["x"]) == len(m["x"]) + r["insertions"] + r["boundary_splits"]
    assert len(r["tri"]) // 3 == len(m["tri"]) // 3 + 2 * r["insertions"] + r["boundary_splits"]
    # the input points are kept, and boundary splits land on the unit square's sides
    np.testing.assert_array_equal(r["x"][:len(m["x"])], m["x"])
    nb = r["nbr"] == gga.MESH_NONE
    t = r["tri"].reshape(-1, 3)
    bpts = np.unique(np.concatenate([t[np.nonzero(nb.reshape(-1, 3)[:, i])[0], (i + 1) % 3] for i in range(3)]))
    on_side = (np.isin(r["x"][bpts], [0.0, 1.0])) | (np.isin(r["y"][bpts], [0.0, 1.0]))
    assert on_side.all()


def test_oracle_refinement_is_deterministic_and_batch_cap_changes_only_the_schedule():
    m = oracle.mesh_gen_random(1500, 3)
    a, b = oracle.mesh_refine(m), oracle.mesh_refine(m)
    for k in ("x", "y", "tri", "nbr"):
        np.testing.assert_array_equal(a[k], b[k])
    small = oracle.mesh_refine(m, batch_cap=3)
    assert small["status"] == "ok" and small["rounds"] > a["rounds"]
    assert _valid(small)["bad_triangles"] == 0


def test_oracle_capacity_stop_keeps_the_last_complete_round():
    m = oracle.mesh_gen_random(1500, 3)
    ntri = len(m["tri"]) // 3
    r = oracle.mesh_refine(m, max_triangles=ntri + 1500)
    assert r["status"] == "capacity" and ntri < len(r["tri"]) // 3 <= ntri + 1500
    c = _valid(r)
    assert c["bad_triangles"] == r["bad_out"] > 0


@pytest.mark.parametrize("angle", [15.0, 20.0, 30.0])
def test_oracle_refinement_other_angle_bounds(angle):
    m = oracle.mesh_gen_random(1500, 9)
    r = oracle.mesh_refine(m, min_angle_deg=angle)
    assert r["status"] == "ok"
    assert _valid(r, angle)["bad_triangles"] == 0
    assert _angles_deg(r).min() >= angle - 1e-9
    assert math.isclose(oracle.cos_bound(angle), math.cos(math.radians(angle)), rel_tol=1e-15)


def test_dmr_cli_usage_and_missing_input_need_no_device(tmp_path):
    import os
    import subprocess

    exe = os.path.join(os.path.dirname(gga.__file__), "bin", "r_dmr")
    if not os.path.exists(exe):
        pytest.skip("gga_dmr not built")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and r.stdout.startswith("Usage: ")
    r = subprocess.run([exe, str(tmp_path / "none")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "cannot open" in r.stderr


def _golden_dmr():
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dmr_io.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", ["jittered6x5", "random60"])
def test_loader_matches_the_reference_readers(tmp_path, name):
    """tests/golden/dmr_io.json holds what the reference's own readNodes /
    readTriangles (helpers.h:5-63, compiled from its sources) parsed from these
    files: the same points (the reference reads them as float), the same
    triangles, and its .poly segments are this library's boundary edges."""
    fx = _golden_dmr()[name]
    for ext in ("node", "ele", "poly"):
        (tmp_path / f"m.{ext}").write_text(fx[ext])
    a = gga.Mesh.load(str(tmp_path / "m")).arrays()
    nele = len(a["tri"]) // 3
    assert fx["ref_nnodes"] == len(a["x"])
    np.testing.assert_array_equal(a["x"].astype(np.float32), np.array(fx["ref_x"], np.float32))
    np.testing.assert_array_equal(a["y"].astype(np.float32), np.array(fx["ref_y"], np.float32))
    ref_tri = np.array(fx["ref_tri"], np.uint32).reshape(-1, 3)
    np.testing.assert_array_equal(ref_tri[:nele].ravel(), a["tri"])
    segs = ref_tri[nele:]
    assert fx["ref_ntriangles"] == nele + len(segs) and (segs[:, 2] == 1234567890).all()  # INVALIDID third node
    t, n = a["tri"].reshape(-1, 3), a["nbr"].reshape(-1, 3)
    ours = {tuple(sorted((int(t[k, (i + 1) % 3]), int(t[k, (i + 2) % 3]))))
            for k in range(nele) for i in range(3) if n[k, i] == gga.MESH_NONE}
    assert ours == {tuple(sorted(map(int, s[:2]))) for s in segs}


def test_cli_result_row_matches_the_reference_writer():
    """The row format of gga_dmr.c's result.vi line, applied to the fields the
    fixture gave the reference's own getname / writeResult (myresult.h:13-52),
    reproduces the rows that writer appended."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(gga.__file__), "csrc", "gga_dmr.c")).read()
    fmt = re.search(r'fprintf\(fp, "([^"]*)\\n"', src).group(1).replace("%llu", "%u")
    fx = _golden_dmr()
    rows = fx["result_vi"].splitlines()
    for line, name in zip(rows, ["jittered6x5", "random60"]):
        f = fx[name]["row_fields"]
        assert fmt % ("r_dmr", name, *f[:5], float(f[5]), float(f[6])) == line
