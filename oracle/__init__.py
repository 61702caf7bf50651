"""ORACLE — test infrastructure, not product code.

ctypes binding of ``oracle/liboracle.so`` (the C restatement of the
reference's host algorithms in ``gga_oracle.c``) and a runner for the
reference's own host code built into ``oracle/_ref/`` (development host only).
Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, always as the checker or the CPU baseline,
never as part of the GPU path being measured.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
INF = 1000000000

_lib = None


def build(quiet: bool = True) -> None:
    """Compiles liboracle.so (gcc only); the reference build is `make ref`."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = C.CDLL(LIB_PATH)
    P, U = C.c_void_p, C.c_uint32
    lib.oracle_load_gr.restype = P
    lib.oracle_load_gr.argtypes = [C.c_char_p]
    lib.oracle_from_csr.restype = P
    lib.oracle_from_csr.argtypes = [U, U, P, P, P]
    lib.oracle_free.argtypes = [P]
    lib.oracle_dims.argtypes = [P, P, P, P, P]
    lib.oracle_arrays.argtypes = [P] * 8
    lib.oracle_max_degree.restype = U
    lib.oracle_max_degree.argtypes = [P]
    lib.oracle_max_allowed_out_degree.restype = U
    lib.oracle_max_allowed_out_degree.argtypes = [P, C.c_int]
    lib.oracle_size_after_split.restype = C.c_int
    lib.oracle_size_after_split.argtypes = [P, C.c_int, C.c_int, P, P]
    lib.oracle_node_split.restype = C.c_int
    lib.oracle_node_split.argtypes = [P, C.c_int, C.c_int]
    lib.oracle_child_index.restype = U
    lib.oracle_child_index.argtypes = [P, P, P]
    lib.oracle_serial.restype = U
    lib.oracle_serial.argtypes = [P, C.c_int, U, P]
    lib.oracle_init_dist.argtypes = [P, U, P]
    lib.oracle_verify.restype = C.c_uint64
    lib.oracle_verify.argtypes = [P, C.c_int, P]
    lib.oracle_ary2file.restype = C.c_int
    lib.oracle_ary2file.argtypes = [C.c_char_p, P, P, U]
    lib.oracle_shortest.restype = C.c_int
    lib.oracle_shortest.argtypes = [P, C.c_int, U, P]
    D = C.c_double
    lib.oracle_gen_rmat.restype = P
    lib.oracle_gen_rmat.argtypes = [U, U, D, D, D, C.c_uint64, U, U]
    lib.oracle_gen_grid.restype = P
    lib.oracle_gen_grid.argtypes = [U, U, D, D, C.c_uint64, U, U]
    lib.oracle_mesh_refine.restype = C.c_int
    lib.oracle_mesh_refine.argtypes = [P, P, P, P, P, P, U, U, D, U, U, P]
    lib.oracle_mesh_refine_log.restype = C.c_int
    lib.oracle_mesh_refine_log.argtypes = [P, P, P, P, P, P, U, U, D, U, U, P, P, U]
    lib.oracle_mesh_count_bad.restype = C.c_uint64
    lib.oracle_mesh_count_bad.argtypes = [U, P, P, P, D]
    lib.gga_mesh_gen_jittered.restype = C.c_int
    lib.gga_mesh_gen_jittered.argtypes = [U, U, D, C.c_uint64, P]
    lib.gga_mesh_gen_random.restype = C.c_int
    lib.gga_mesh_gen_random.argtypes = [U, C.c_uint64, P]
    lib.gga_mesh_from_arrays.restype = C.c_int
    lib.gga_mesh_from_arrays.argtypes = [U, P, P, U, P, P]
    lib.gga_mesh_check.restype = C.c_int
    lib.gga_mesh_check.argtypes = [P, D, P]
    lib.gga_mesh_get_info.argtypes = [P, P]
    lib.gga_mesh_arrays.argtypes = [P, P, P, P, P]
    lib.gga_mesh_free.argtypes = [P]
    _lib = lib
    return lib


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class OracleGraph:
    """The reference's struct Graph, restated (1-based psrc layout)."""

    def __init__(self, handle):
        if not handle:
            raise RuntimeError("oracle: could not load graph")
        self._h = C.c_void_p(handle)

    @classmethod
    def from_csr(cls, off, col, wt):
        off = np.ascontiguousarray(off, np.uint32)
        col = np.ascontiguousarray(col, np.uint32)
        wt = np.ascontiguousarray(wt, np.uint32)
        if len(col) == 0:
            col = np.zeros(1, np.uint32)
            wt = np.zeros(1, np.uint32)
            m = 0
        else:
            m = len(col)
        return cls(load().oracle_from_csr(len(off) - 1, m, _p(off), _p(col), _p(wt)))

    @classmethod
    def load_gr(cls, path: str):
        return cls(load().oracle_load_gr(path.encode()))

    @classmethod
    def gen_rmat(cls, scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1, wmin=1, wmax=255):
        """The library's seeded R-MAT generator, run inside liboracle.so (the
        GPU library is not loaded): the same graph gga.Graph.rmat returns."""
        return cls(load().oracle_gen_rmat(scale, edge_factor, a, b, c, seed, wmin, wmax))

    @classmethod
    def gen_grid(cls, width, height, del_prob=0.05, longrange_frac=0.001, seed=1, wmin=1, wmax=1000):
        """The library's seeded grid generator, run inside liboracle.so."""
        return cls(load().oracle_gen_grid(width, height, del_prob, longrange_frac, seed, wmin, wmax))

    def __del__(self):
        try:
            if self._h:
                load().oracle_free(self._h)
                self._h = None
        except Exception:
            pass

    def dims(self):
        n, m, nb, mda = (C.c_uint32() for _ in range(4))
        load().oracle_dims(self._h, C.byref(n), C.byref(m), C.byref(nb), C.byref(mda))
        return {"nnodes": n.value, "nedges": m.value, "nodes_b4_ns": nb.value, "mda": mda.value}

    def arrays(self) -> dict:
        d = self.dims()
        n, m = d["nnodes"], d["nedges"]
        out = {
            "psrc": np.zeros(n + 1, np.uint32),
            "noutgoing": np.zeros(max(n, 1), np.uint32),
            "edgessrcdst": np.zeros(m + 1, np.uint32),
            "edgessrcwt": np.zeros(m + 1, np.uint32),
            "childCount": np.zeros(max(n, 1), np.uint32),
            "IsParent": np.zeros(max(n, 1), np.uint32),
            "parentNode": np.zeros(max(n, 1), np.uint32),
        }
        load().oracle_arrays(self._h, *[_p(out[k]) for k in
                                        ("psrc", "noutgoing", "edgessrcdst", "edgessrcwt", "childCount", "IsParent", "parentNode")])
        for k in ("noutgoing", "childCount", "IsParent", "parentNode"):
            out[k] = out[k][:n]
        return out

    def max_degree(self) -> int:
        return load().oracle_max_degree(self._h)

    def max_allowed_out_degree(self, buckets: int) -> int:
        return load().oracle_max_allowed_out_degree(self._h, buckets)

    def size_after_split(self, level: int, buckets: int):
        mda, cnt = C.c_uint32(), C.c_uint32()
        rc = load().oracle_size_after_split(self._h, level, buckets, C.byref(mda), C.byref(cnt))
        return rc, mda.value, cnt.value

    def node_split(self, level: int, buckets: int = 10) -> int:
        return load().oracle_node_split(self._h, level, buckets)

    def child_index(self):
        n = self.dims()["nnodes"]
        idx = np.zeros(max(n, 1), np.uint32)
        cnt = np.zeros(max(n, 1), np.uint32)
        p = load().oracle_child_index(self._h, _p(idx), _p(cnt))
        return idx[:p], cnt[:p]

    def serial(self, algo: str, src: int):
        """findSerialBFS / findSerialSSSP: (dist, passes)."""
        n = self.dims()["nnodes"]
        d = np.zeros(n, np.uint32)
        passes = load().oracle_serial(self._h, 1 if algo == "sssp" else 0, src, _p(d))
        return d, passes

    def shortest(self, algo: str, src: int) -> np.ndarray:
        """Exact distances by a second method (FIFO BFS / Dijkstra), for
        graphs too large or too deep for the reference's sweeps."""
        n = self.dims()["nnodes"]
        d = np.zeros(max(n, 1), np.uint32)
        if load().oracle_shortest(self._h, 1 if algo == "sssp" else 0, src, _p(d)):
            raise MemoryError("oracle_shortest")
        return d[:n]

    def degrees(self) -> np.ndarray:
        """Out-degree per vertex (noutgoing)."""
        n = self.dims()["nnodes"]
        d = np.zeros(max(n, 1), np.uint32)
        load().oracle_arrays(self._h, None, _p(d), None, None, None, None, None)
        return d[:n]

    def init_dist(self, parent_src: int):
        n = self.dims()["nnodes"]
        d = np.zeros(n, np.uint32)
        load().oracle_init_dist(self._h, parent_src, _p(d))
        return d

    def verify(self, algo: str, dist_split) -> int:
        d = np.ascontiguousarray(dist_split, np.uint32)
        return int(load().oracle_verify(self._h, 1 if algo == "sssp" else 0, _p(d)))


MESH_STATUS = {0: "ok", 1: "capacity", 2: "stalled", 3: "rounds", 4: "no_memory"}


def cos_bound(min_angle_deg: float) -> float:
    """cos(MINANGLE * (PI / 180)) as the refinement compares it (helpers.h:171)."""
    return math.cos(min_angle_deg * (math.pi / 180.0))


def _mesh_dict(lib, h_) -> dict:
    info = (C.c_uint32 * 2)()
    lib.gga_mesh_get_info(h_, info)
    npts, ntri = int(info[0]), int(info[1])
    px, py, pt, pn = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
    lib.gga_mesh_arrays(h_, C.byref(px), C.byref(py), C.byref(pt), C.byref(pn))

    def grab(ptr, n, ct, dt):
        if n == 0:
            return np.zeros(0, dt)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), (n,)).astype(dt, copy=True)
    return {"x": grab(px, npts, C.c_double, np.float64), "y": grab(py, npts, C.c_double, np.float64),
            "tri": grab(pt, 3 * ntri, C.c_uint32, np.uint32), "nbr": grab(pn, 3 * ntri, C.c_uint32, np.uint32)}


def _mesh_call(fn, *args) -> dict:
    lib = load()
    h_ = C.c_void_p()
    if fn(*args, C.byref(h_)) != 0:
        raise RuntimeError("oracle: mesh construction failed")
    try:
        return _mesh_dict(lib, h_)
    finally:
        lib.gga_mesh_free(h_)


def mesh_gen_jittered(w: int, h: int, jitter: float, seed: int) -> dict:
    """The library's seeded jittered-grid Delaunay mesh, built inside
    liboracle.so (the GPU library is not loaded): the same mesh that
    gga.Mesh.jittered returns.  Arrays x, y (float64), tri, nbr (uint32)."""
    return _mesh_call(load().gga_mesh_gen_jittered, w, h, jitter, seed)


def mesh_gen_random(npoints: int, seed: int) -> dict:
    """The library's seeded random-point Delaunay mesh (gga.Mesh.random)."""
    return _mesh_call(load().gga_mesh_gen_random, npoints, seed)


def mesh_check(mesh: dict, min_angle_deg: float = 25.0) -> dict:
    """Checks a mesh's arrays: its neighbour array must equal the one derived
    from its triangles, every triangle must be counter-clockwise (the
    derivation would reorder it otherwise), and the derived mesh's check
    counts (gga_mesh_check) are returned."""
    lib = load()
    x = np.ascontiguousarray(mesh["x"], np.float64)
    y = np.ascontiguousarray(mesh["y"], np.float64)
    tri = np.ascontiguousarray(mesh["tri"], np.uint32)
    h_ = C.c_void_p()
    if lib.gga_mesh_from_arrays(len(x), _p(x), _p(y), len(tri) // 3, _p(tri), C.byref(h_)) != 0:
        return {"valid": False}
    try:
        d = _mesh_dict(lib, h_)
        r = (C.c_char * 48)()  # gga_mesh_check_result: 5 x uint64, then double area
        lib.gga_mesh_check(h_, min_angle_deg, r)
        u = np.frombuffer(bytes(r), np.uint64, 5)
        area = float(np.frombuffer(bytes(r), np.float64, 1, 40)[0])
    finally:
        lib.gga_mesh_free(h_)
    return {"valid": True, "tri_ccw": bool(np.array_equal(d["tri"], tri)),
            "nbr_consistent": bool(np.array_equal(d["nbr"], np.asarray(mesh["nbr"], np.uint32))),
            "bad_triangles": int(u[0]), "bad_orientation": int(u[1]), "bad_neighbors": int(u[2]),
            "non_delaunay_edges": int(u[3]), "boundary_edges": int(u[4]), "area": area}


def mesh_refine(mesh: dict, min_angle_deg: float = 25.0, max_triangles: int = 0, batch_cap: int = 1 << 20,
                max_rounds: int = 65536) -> dict:
    """Serial refinement in the GPU's round schedule (mesh_oracle.c).  Takes
    and returns dicts of x, y, tri, nbr; adds 'status' and the stats."""
    x, y = mesh["x"], mesh["y"]
    tri, nbr = mesh["tri"], mesh["nbr"]
    npts, ntri = len(x), len(tri) // 3
    tcap = max_triangles or min(4 * ntri + 65536, 0x3FFFFFFF)
    pcap = npts + (tcap - ntri)  # each insertion adds one point and at least one triangle
    X = np.zeros(pcap, np.float64); X[:npts] = x
    Y = np.zeros(pcap, np.float64); Y[:npts] = y
    T = np.zeros(3 * tcap, np.uint32); T[:3 * ntri] = tri
    N = np.zeros(3 * tcap, np.uint32); N[:3 * ntri] = nbr
    np_, nt_ = C.c_uint32(npts), C.c_uint32(ntri)
    st = np.zeros(6, np.uint64)
    log = np.zeros(3 * 4096, np.uint32)
    rc = load().oracle_mesh_refine_log(C.byref(np_), C.byref(nt_), _p(X), _p(Y), _p(T), _p(N), pcap, tcap,
                                       cos_bound(min_angle_deg), batch_cap, max_rounds, _p(st), _p(log), 4096)
    P, Tn = np_.value, nt_.value
    return {"x": X[:P].copy(), "y": Y[:P].copy(), "tri": T[:3 * Tn].copy(), "nbr": N[:3 * Tn].copy(),
            "status": MESH_STATUS.get(rc, str(rc)), "rounds": int(st[0]), "insertions": int(st[1]),
            "boundary_splits": int(st[2]), "failed_plans": int(st[3]), "bad_in": int(st[4]), "bad_out": int(st[5]),
            "round_log": log[:3 * min(int(st[0]), 4096)].reshape(-1, 3).copy()}


def mesh_count_bad(mesh: dict, min_angle_deg: float = 25.0) -> int:
    tri = np.ascontiguousarray(mesh["tri"], np.uint32)
    return int(load().oracle_mesh_count_bad(len(tri) // 3, _p(mesh["x"]), _p(mesh["y"]), _p(tri),
                                            cos_bound(min_angle_deg)))


def serial_distances(off, col, wt, algo: str, src: int) -> np.ndarray:
    """Oracle BFS levels / SSSP distances on the unsplit graph."""
    return OracleGraph.from_csr(off, col, wt).serial(algo, src)[0]


# ---------------------------------------------------------------- reference build

def ref_available() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, f"ref_{a}")) for a in ("bfs", "sssp"))


def run_reference(gr_path: str, algo: str, level: int, buckets: int, src: int, workdir: str | None = None) -> dict:
    """Runs oracle/_ref/ref_<algo> (the reference's own host code) and reads
    its dumps.  Returns {"returncode", "stdout", arrays..., meta...}."""
    exe = os.path.join(REF_DIR, f"ref_{algo}")
    own = workdir is None
    wd = workdir or tempfile.mkdtemp(prefix="gga_ref_")
    prefix = os.path.join(wd, "out")
    p = subprocess.run([exe, gr_path, str(level), str(buckets), str(src), prefix], capture_output=True, text=True)
    res = {"returncode": p.returncode, "stdout": p.stdout}
    if p.returncode == 0:
        for k in ("dist", "psrc", "noutgoing", "edgessrcdst", "childCount", "IsParent", "parentNode"):
            res[k] = np.fromfile(f"{prefix}.{k}.u32", dtype="<u4")
        with open(f"{prefix}.ary.txt") as f:
            res["ary_txt"] = f.read()
        for line in open(f"{prefix}.meta"):
            k, v = line.strip().split("=", 1)
            res[k] = v if k == "algo" else int(v)
        for line in p.stdout.splitlines():
            if "no of errors" in line:
                res["nerr"] = int(line.split("=")[1].strip().rstrip("."))
    if own:
        subprocess.run(["rm", "-rf", wd])
    return res
