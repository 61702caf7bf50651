"""GB300-native static-graph BFS/SSSP (GPUGraphAlgo's traversal hot path).

Python side of the C ABI in ``include/gga.h``: thin ctypes wrappers used by the
tests and the benchmark.  All computation happens in ``libgga.so`` (host C and
sm_103a CUDA kernels).  Method names follow the reference's ``struct Graph``
(Programs/CUDA_src/Kepler_BFS_SSSP/graph.h:23-64) where one exists:
``readFromGR``, ``getMaxdeg``, ``getMaxAllowedOutDegree``,
``getSizeafterLoadBalance``, ``NodeSplit``, ``cudaCopy``; ``verifysolution``,
``Ary2File`` and ``writeResult`` mirror myutils.h.  Errors raise
:class:`GGAError` carrying the C status code instead of exiting the process
(the reference calls ``exit(-1)`` in ``CudaTest``, graph.h:523-533).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _native as N

INFINITY = 1000000000  # MYINFINITY, bfs_sssp.cu:53
MAX_WEIGHT = 0xFFFFFFFF - INFINITY

BFS, SSSP = 0, 1
ALGOS = {"bfs": BFS, "sssp": SSSP}

VARIANTS = {
    "auto": 0,
    "frontier": 1,
    "topo_atomic": 2,  # "na_" build
    "topo_plain": 3,  # "n_" build
    "cdp_atomic": 4,  # "da_" build
    "cdp_plain": 5,  # "d_" build
}

OK, ERR_INVALID_ARG, ERR_IO, ERR_FORMAT, ERR_SPLIT_RULE = 0, 1, 2, 3, 4
ERR_NO_MEMORY, ERR_CUDA, ERR_NO_DEVICE, ERR_TIMEOUT, ERR_ADMISSION = 5, 6, 7, 8, 9
ERR_TOO_LARGE, ERR_NOT_READY, ERR_UNSUPPORTED, ERR_NO_PROGRESS = 10, 11, 12, 13
MESH_NONE = 0xFFFFFFFF  # no neighbour: a domain boundary edge
DMR_MIN_ANGLE = 25.0  # MINANGLE, Kepler_DMR/dmr.cu:34


class GGAError(RuntimeError):
    def __init__(self, status: int, where: str):
        lib = N.load()
        self.status = status
        msg = lib.gga_last_error().decode(errors="replace")
        super().__init__(f"{where}: {lib.gga_status_string(status).decode()} ({status}): {msg}")


def _check(status: int, where: str):
    if status != OK:
        raise GGAError(status, where)


def lib():
    return N.load()


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def _out_ptr(out):
    """Address of an output buffer: a numpy array or an object with data_ptr()."""
    return C.c_void_p(out.data_ptr()) if hasattr(out, "data_ptr") else _ptr(out)


class _HostBlock:
    """Page-locked host memory from gga_host_alloc, freed with its last array."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        _check(N.load().gga_host_alloc(nbytes, C.byref(p)), "host_alloc")
        self.ptr = p.value

    def __del__(self):
        if getattr(self, "ptr", None):
            N.load().gga_host_free(C.c_void_p(self.ptr))
            self.ptr = None


def pinned_empty(shape, dtype=np.uint32) -> np.ndarray:
    """An uninitialised numpy array in page-locked host memory, so copies to
    and from the GPU run asynchronously at full bandwidth."""
    dt = np.dtype(dtype)
    count = int(np.prod(shape))
    nbytes = max(1, count * dt.itemsize)
    blk = _HostBlock(nbytes)
    raw = (C.c_char * nbytes).from_address(blk.ptr)
    raw._gga_block = blk  # the array's base keeps the block alive
    return np.frombuffer(raw, dt, count).reshape(shape)


def _algo(a) -> int:
    return ALGOS[a] if isinstance(a, str) else int(a)


def _variant(v) -> int:
    return VARIANTS[v] if isinstance(v, str) else int(v)


class Graph:
    """A host CSR graph (struct Graph); device residency is cached per graph."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    # ---- construction
    @classmethod
    def readFromGR(cls, path: str) -> "Graph":
        h = C.c_void_p()
        _check(N.load().gga_graph_load_gr(path.encode(), C.byref(h)), f"readFromGR({path})")
        return cls(h.value)

    load_gr = readFromGR

    @classmethod
    def from_csr(cls, offsets, cols, weights=None) -> "Graph":
        off = np.ascontiguousarray(offsets, dtype=np.uint32)
        col = np.ascontiguousarray(cols, dtype=np.uint32)
        n, m = len(off) - 1, len(col)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.uint32)
        h = C.c_void_p()
        _check(
            N.load().gga_graph_from_csr(n, m, _ptr(off), _ptr(col) if m else None, None if w is None else _ptr(w), C.byref(h)),
            "from_csr",
        )
        return cls(h.value)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a=0.57, b=0.19, c=0.19, seed: int = 1, wmin: int = 1, wmax: int = 255):
        h = C.c_void_p()
        _check(N.load().gga_graph_gen_rmat(scale, edge_factor, a, b, c, seed, wmin, wmax, C.byref(h)), "gen_rmat")
        return cls(h.value)

    @classmethod
    def grid(cls, width: int, height: Optional[int] = None, del_prob=0.05, longrange_frac=0.001, seed: int = 3, wmin: int = 1, wmax: int = 1000):
        h = C.c_void_p()
        _check(
            N.load().gga_graph_gen_grid(width, height or width, del_prob, longrange_frac, seed, wmin, wmax, C.byref(h)),
            "gen_grid",
        )
        return cls(h.value)

    def save_gr(self, path: str):
        _check(N.load().gga_graph_save_gr(self._h, path.encode()), f"save_gr({path})")

    def free(self):
        if self._h and self._h.value:
            N.load().gga_graph_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ---- description
    def info(self) -> dict:
        i = N.GraphInfo()
        _check(N.load().gga_graph_get_info(self._h, C.byref(i)), "info")
        return {k: getattr(i, k) for k, _ in i._fields_}

    @property
    def n(self) -> int:
        return self.info()["nodes_orig"]

    @property
    def m(self) -> int:
        return self.info()["nedges"]

    def csr(self):
        """Copies of the unsplit 0-based CSR (offsets, cols, weights)."""
        o, c, w = N.PU32(), N.PU32(), N.PU32()
        _check(N.load().gga_graph_csr(self._h, C.byref(o), C.byref(c), C.byref(w)), "csr")
        n, m = self.n, self.m
        off = np.ctypeslib.as_array(o, shape=(n + 1,)).copy()
        col = np.ctypeslib.as_array(c, shape=(m,)).copy() if m else np.zeros(0, np.uint32)
        wt = np.ctypeslib.as_array(w, shape=(m,)).copy() if m else np.zeros(0, np.uint32)
        return off, col, wt

    def degrees(self) -> np.ndarray:
        off = self.csr()[0]
        return np.diff(off.astype(np.int64)).astype(np.uint32)

    # ---- split rules (graph.h:338-414)
    def getMaxdeg(self) -> int:
        v = C.c_uint32()
        _check(N.load().gga_max_degree(self._h, C.byref(v)), "getMaxdeg")
        return v.value

    def getMaxAllowedOutDegree(self, buckets: int = 10) -> int:
        v = C.c_uint32()
        _check(N.load().gga_max_allowed_out_degree(self._h, buckets, C.byref(v)), "getMaxAllowedOutDegree")
        return v.value

    def getSizeafterLoadBalance(self, level: int, buckets: int = 10):
        """Returns (MAX_EDGES_ALLOWED, split vertex count)."""
        mda, nn = C.c_uint32(), C.c_uint32()
        _check(N.load().gga_size_after_split(self._h, level, buckets, C.byref(mda), C.byref(nn)), "getSizeafterLoadBalance")
        return mda.value, nn.value

    def NodeSplit(self, ctx: "Context", level: int, buckets: int = 10):
        """Device-side node split (graph.h:415-522); level 0 removes it."""
        _check(N.load().gga_node_split(ctx.handle, self._h, level, buckets), f"NodeSplit({level},{buckets})")

    node_split = NodeSplit

    def split_maps(self, ctx: "Context") -> dict:
        """The split graph in the reference's layout (1-based psrc, slot-0 edge)."""
        i = self.info()
        nn, m = i["nnodes"], i["nedges"]
        out = {
            "psrc": np.zeros(nn + 1, np.uint32),
            "noutgoing": np.zeros(nn, np.uint32),
            "edgessrcdst": np.zeros(m + 1, np.uint32),
            "childCount": np.zeros(nn, np.uint32),
            "IsParent": np.zeros(nn, np.uint32),
            "parentNode": np.zeros(nn, np.uint32),
        }
        _check(
            N.load().gga_graph_split_maps(
                ctx.handle, self._h, *[_ptr(out[k]) for k in ("psrc", "noutgoing", "edgessrcdst", "childCount", "IsParent", "parentNode")]
            ),
            "split_maps",
        )
        return out

    def child_index(self, ctx: "Context"):
        """(myChildIndex, myChildCount), bfs_sssp.cu:256-283."""
        cnt = C.c_uint32(0)
        st = N.load().gga_child_index(ctx.handle, self._h, C.byref(cnt), None, None)
        if st not in (OK, ERR_INVALID_ARG):
            _check(st, "child_index")
        idx = np.zeros(max(cnt.value, 1), np.uint32)
        cc = np.zeros(max(cnt.value, 1), np.uint32)
        _check(N.load().gga_child_index(ctx.handle, self._h, C.byref(cnt), _ptr(idx), _ptr(cc)), "child_index")
        return idx[: cnt.value], cc[: cnt.value]

    def pin(self, on: bool = True):
        _check(N.load().gga_graph_pin(self._h, 1 if on else 0), "pin")

    def release_device(self):
        _check(N.load().gga_graph_release_device(self._h), "release_device")

    def cudaCopy(self, ctx: "Context"):
        _check(N.load().gga_graph_upload(ctx.handle, self._h), "cudaCopy")

    upload = cudaCopy

    # ---- checks and output (myutils.h)
    def verifysolution(self, dist: np.ndarray, algo="bfs") -> int:
        d = np.ascontiguousarray(dist, dtype=np.uint32)
        v = C.c_uint64()
        _check(N.load().gga_verify(self._h, _algo(algo), _ptr(d), C.byref(v)), "verifysolution")
        return v.value

    verify = verifysolution

    def Ary2File(self, path: str, dist: np.ndarray):
        d = np.ascontiguousarray(dist, dtype=np.uint32)
        _check(N.load().gga_write_dist(path.encode(), self._h, _ptr(d)), "Ary2File")

    def reached(self, dist: np.ndarray):
        d = np.ascontiguousarray(dist, dtype=np.uint32)
        vr, er = C.c_uint64(), C.c_uint64()
        _check(N.load().gga_reached(self._h, _ptr(d), C.byref(vr), C.byref(er)), "reached")
        return vr.value, er.value



class Mesh:
    """A 2-D triangulation on the host (the reference DMR's mesh: nodex/nodey,
    tnodes and neighbours, Kepler_DMR/dmesh.h), refined on the GPU by
    :meth:`Context.refine`."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def _make(cls, fn, *args, where="mesh"):
        h = C.c_void_p()
        _check(fn(*args, C.byref(h)), where)
        return cls(h.value)

    @classmethod
    def load(cls, base: str) -> "Mesh":
        """Reads <base>.node and <base>.ele (readNodes / readTriangles, helpers.h:5-63)."""
        return cls._make(N.load().gga_mesh_load_triangle, base.encode(), where=f"load({base})")

    @classmethod
    def from_arrays(cls, x, y, tri) -> "Mesh":
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        t = np.ascontiguousarray(tri, np.uint32).reshape(-1)
        return cls._make(N.load().gga_mesh_from_arrays, len(x), _ptr(x), _ptr(y), len(t) // 3,
                         _ptr(t) if len(t) else None, where="from_arrays")

    @classmethod
    def jittered(cls, w: int, h: int, jitter: float = 0.3, seed: int = 1) -> "Mesh":
        return cls._make(N.load().gga_mesh_gen_jittered, w, h, jitter, seed, where="jittered")

    @classmethod
    def random(cls, npoints: int, seed: int = 1) -> "Mesh":
        return cls._make(N.load().gga_mesh_gen_random, npoints, seed, where="random")

    def save(self, base: str):
        _check(N.load().gga_mesh_save_triangle(self._h, base.encode()), f"save({base})")

    def free(self):
        if self._h and self._h.value:
            N.load().gga_mesh_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        i = N.MeshInfo()
        _check(N.load().gga_mesh_get_info(self._h, C.byref(i)), "info")
        return {"npoints": i.npoints, "ntriangles": i.ntriangles}

    def arrays(self) -> dict:
        """Copies of x, y (float64) and tri, nbr (uint32, 3 per triangle)."""
        inf = self.info()
        x, y, t, n = N.PD(), N.PD(), N.PU32(), N.PU32()
        _check(N.load().gga_mesh_arrays(self._h, C.byref(x), C.byref(y), C.byref(t), C.byref(n)), "arrays")
        P, T = inf["npoints"], inf["ntriangles"]

        def grab(ptr, cnt, dt):
            return np.ctypeslib.as_array(ptr, (cnt,)).astype(dt, copy=True) if cnt else np.zeros(0, dt)
        return {"x": grab(x, P, np.float64), "y": grab(y, P, np.float64), "tri": grab(t, 3 * T, np.uint32),
                "nbr": grab(n, 3 * T, np.uint32)}

    def check(self, min_angle_deg: float = DMR_MIN_ANGLE) -> dict:
        r = N.MeshCheck()
        _check(N.load().gga_mesh_check(self._h, min_angle_deg, C.byref(r)), "check")
        return {k: getattr(r, k) for k, _ in r._fields_}


def writeResult(path: str, **fields):
    """Appends one 17-column result.vi row (myutils.h:86-113)."""
    r = N.ResultRow()
    for k, v in fields.items():
        setattr(r, k, v.encode() if isinstance(v, str) else v)
    _check(N.load().gga_write_result_row(path.encode(), C.byref(r)), "writeResult")


def combine_clocks(block_cycles, sms: int = 14):
    """The reference's load-balance estimate of one launch (combineClocks,
    metrics.h:68-84, with getminIndex / getmaxIndex, metrics.h:1-24): blocks
    in launch order go to the least-loaded SM (lowest index on ties), and the
    estimate is the busiest SM's total.  Returns (estimate, SM of each block).
    The reference sums the estimates of every iteration (bfs_sssp.cu:527-536)
    with its 14 SMs; pass sms=152 for a GB300."""
    load = [0] * sms
    where = []
    for c in block_cycles:
        k = min(range(sms), key=lambda j: (load[j], j))
        where.append(k)
        load[k] += int(c)
    return max(load), where


class Context:
    """A device context: stream, events and scratch on one GPU."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        _check(N.load().gga_ctx_create(device, C.byref(self._h)), f"ctx_create({device})")

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h and self._h.value:
            N.load().gga_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def device_info(self):
        sms = C.c_int()
        name = C.create_string_buffer(256)
        _check(N.load().gga_ctx_device_info(self._h, C.byref(sms), name, 256), "device_info")
        return {"sms": sms.value, "name": name.value.decode()}

    def mark(self, slot: int):
        _check(N.load().gga_ctx_mark(self._h, slot), "mark")

    def elapsed(self, a: int, b: int) -> float:
        ms = C.c_double()
        _check(N.load().gga_ctx_elapsed(self._h, a, b, C.byref(ms)), "elapsed")
        return ms.value

    def synchronize(self):
        _check(N.load().gga_ctx_synchronize(self._h), "synchronize")

    def set_params(self, **kw):
        p = N.Params()
        _check(N.load().gga_get_params(self._h, C.byref(p)), "get_params")
        for k, v in kw.items():
            setattr(p, k, v)
        _check(N.load().gga_set_params(self._h, C.byref(p)), "set_params")

    def reset_params(self):
        """Back to the per-graph defaults derived from the degree profile."""
        _check(N.load().gga_set_params(self._h, None), "reset_params")

    def params(self) -> dict:
        p = N.Params()
        _check(N.load().gga_get_params(self._h, C.byref(p)), "get_params")
        return p.as_dict()

    def prepare(self, graph: Graph, algo):
        """Upload `graph` if needed and build its once-per-graph derived data
        for `algo` under the current parameters (gga_graph_prepare)."""
        _check(N.load().gga_graph_prepare(self._h, graph.handle, _algo(algo)), f"prepare({algo})")

    def autotune(self, graph: Graph, trials: int = 0) -> dict:
        """Per-graph parameters (gga_autotune): stored on `graph` and set on
        this context.  With trials > 0 the choice comes from timed trials;
        autotune_report() lists them."""
        p = N.Params()
        _check(N.load().gga_autotune(self._h, graph.handle, trials, C.byref(p)), "autotune")
        return p.as_dict()

    def autotune_report(self) -> dict:
        """The last autotune's candidates and their times (ms)."""
        import json

        buf = C.create_string_buffer(1 << 16)
        _check(N.load().gga_autotune_report(self._h, buf, len(buf)), "autotune_report")
        return json.loads(buf.value.decode())

    def solve(self, graph: Graph, algo, src: int, variant="auto", out=None, stats: bool = False,
              keep_on_device: bool = False):
        """Single-source BFS levels / SSSP distances in original vertex order.

        out: numpy array, or any object with a ``data_ptr()`` (device buffer);
        keep_on_device leaves the result in the context's device buffer."""
        if keep_on_device:
            ptr = None
        else:
            if out is None:
                out = np.empty(graph.n, np.uint32)
            ptr = C.c_void_p(out.data_ptr()) if hasattr(out, "data_ptr") else _ptr(out)
        s = N.Stats()
        _check(
            N.load().gga_solve(self._h, graph.handle, _algo(algo), src, _variant(variant), ptr, C.byref(s)),
            f"solve({algo}, src={src}, {variant})",
        )
        return (out, s.as_dict()) if stats else out

    def solve_many(self, graph: Graph, algo, srcs: Sequence[int], out=None, stats: bool = False):
        """One frontier-engine traversal per source, back to back, each
        result copied out while the next runs (gga_solve_many).  out: an
        (len(srcs), n) uint32 array — page-locked (pinned_empty) for the
        copies to overlap — or any object with a ``data_ptr()``; row i is
        srcs[i]'s distances.  stats: one dict per source."""
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        if out is None:
            out = np.empty((len(s), graph.n), np.uint32)
        ptr = C.c_void_p(out.data_ptr()) if hasattr(out, "data_ptr") else _ptr(out)
        st = (N.Stats * max(1, len(s)))()
        _check(N.load().gga_solve_many(self._h, graph.handle, _algo(algo), len(s), _ptr(s), ptr, st),
               f"solve_many({algo}, {len(s)} sources)")
        return (out, [st[i].as_dict() for i in range(len(s))]) if stats else out

    def bfs(self, graph: Graph, src: int, variant="auto", **kw):
        return self.solve(graph, BFS, src, variant, **kw)

    def sssp(self, graph: Graph, src: int, variant="auto", **kw):
        return self.solve(graph, SSSP, src, variant, **kw)

    def trace(self, enable: bool = True):
        """Record per-round frontier records and per-CTA busy kilocycles of the
        following frontier-engine solves (cudaKernels.h:1-70's clock64
        histogram and convergence.h's per-iteration log, on device counters)."""
        _check(N.load().gga_trace_enable(self._h, 1 if enable else 0), "trace_enable")

    def last_trace(self) -> dict:
        nr, nb = C.c_uint32(), C.c_uint32()
        _check(N.load().gga_trace_get(self._h, None, 0, C.byref(nr), None, 0, C.byref(nb)), "trace_get")
        rounds = (N.RoundTrace * max(1, nr.value))()
        cta = np.zeros(max(1, nb.value), np.uint32)
        _check(N.load().gga_trace_get(self._h, rounds, nr.value, C.byref(nr),
                                      cta.ctypes.data_as(C.POINTER(C.c_uint32)), nb.value, C.byref(nb)), "trace_get")
        kinds = ("near", "bottom_up", "far", "heavy", "pull_scan", "pull")
        busy = cta[: nb.value]
        return {"rounds": [{"kind": kinds[r.kind] if r.kind < len(kinds) else r.kind, "items": r.items,
                            "edges": r.edges, "far_items": r.far_items, "us": r.ns / 1e3} for r in rounds[: nr.value]],
                "cta_kcycles": busy,
                # busiest CTA over the mean: 1.0 is a perfectly balanced launch
                "imbalance": float(busy.max() / busy.mean()) if len(busy) and busy.mean() > 0 else None}

    def convergence(self, graph: Graph, algo, src: int, final, variant="topo_atomic"):
        """Per-iteration convergence of a topology-driven solve against
        `final` (printConv_rtime, convergence.h:100-159): one dict per relax
        launch with the vertices still differing and the norm the reference
        prints.  Returns (records, distances)."""
        fin = np.ascontiguousarray(final, dtype=np.uint32)
        if fin.shape != (graph.n,):
            raise ValueError(f"final: {graph.n} distances expected")
        out = np.empty(graph.n, np.uint32)
        cap = min(graph.n + 2, 1 << 20)
        recs = (N.ConvRecord * cap)()
        nrec = C.c_uint32()
        _check(N.load().gga_convergence(self._h, graph.handle, _algo(algo), src, _variant(variant), _ptr(fin), recs,
                                        cap, C.byref(nrec), _ptr(out)), f"convergence({algo}, src={src}, {variant})")
        return ([{"iteration": r.iteration, "diff_count": r.diff_count, "norm2": r.norm2}
                 for r in recs[: min(nrec.value, cap)]], out)

    def refine(self, mesh: "Mesh", min_angle_deg: float = DMR_MIN_ANGLE, max_triangles: int = 0,
               batch_cap: int = 0, tail_max: int = 0, prefetch_max: int = 0) -> dict:
        """Delaunay refinement of `mesh` in place on this context's GPU until no
        angle is below min_angle_deg (the reference's dmr <basefile> run);
        returns the refinement statistics (myresult's fields and timings).
        tail_max / prefetch_max move work between the engine's kernels
        (gga_mesh_refine_ex) without changing the result."""
        st = N.RefineStats()
        p = N.RefineParams(min_angle_deg, max_triangles, batch_cap, tail_max, prefetch_max)
        _check(N.load().gga_mesh_refine_ex(self._h, mesh.handle, C.byref(p), C.byref(st)), "refine")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def msbfs(self, graph: Graph, srcs: Sequence[int], stats: bool = False, out=None):
        """Up to 64 BFS sources in one bit-packed launch; out: optional
        (len(srcs), n) uint32 array (pinned_empty for the fastest copy) or an
        object with ``data_ptr()``."""
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        if out is None:
            out = np.empty((len(s), graph.n), np.uint32)
        st = N.Stats()
        _check(N.load().gga_msbfs(self._h, graph.handle, len(s), _ptr(s), _out_ptr(out), C.byref(st)), "msbfs")
        return (out, st.as_dict()) if stats else out

    def sssp_batch(self, graph: Graph, srcs: Sequence[int], stats: bool = False, out=None):
        """Up to 32 SSSP sources in one launch; out as for msbfs."""
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        if out is None:
            out = np.empty((len(s), graph.n), np.uint32)
        st = N.Stats()
        _check(N.load().gga_sssp_batch(self._h, graph.handle, len(s), _ptr(s), _out_ptr(out), C.byref(st)),
               "sssp_batch")
        return (out, st.as_dict()) if stats else out

    def multi_solve(self, queries, stats: bool = False, outs=None):
        """queries: list of (graph, algo, src) -> list of distance arrays.
        outs: optional list of one output array (or ``data_ptr()`` object)
        per query."""
        if outs is None:
            outs = [np.empty(g.n, np.uint32) for g, _, _ in queries]
        arr = (N.Query * len(queries))()
        for i, (g, a, s) in enumerate(queries):
            arr[i].graph = g.handle.value
            arr[i].algo = _algo(a)
            arr[i].src = s
            arr[i].dist_out = _out_ptr(outs[i]).value
        st = N.Stats()
        _check(N.load().gga_multi_solve(self._h, len(queries), arr, C.byref(st)), "multi_solve")
        return (outs, st.as_dict()) if stats else outs


class Server:
    """Continuous-batching query loop over HBM-resident graphs."""

    def __init__(self, ctx: Context, graphs: Sequence[Graph], mem_cap_bytes: int, max_slots: int = 64):
        self._graphs = list(graphs)
        arr = (C.c_void_p * len(graphs))(*[g.handle.value for g in graphs])
        self._h = C.c_void_p()
        _check(N.load().gga_server_create(ctx.handle, len(graphs), arr, mem_cap_bytes, max_slots, C.byref(self._h)), "server_create")
        self._outs = {}

    def submit(self, graph_index: int, algo, src: int, out=None) -> int:
        """Queues one query; `out` (numpy array or an object with data_ptr(),
        e.g. a CUDA tensor) receives the distances, else a new host array."""
        if out is None:
            out = np.empty(self._graphs[graph_index].n, np.uint32)
        ptr = C.c_void_p(out.data_ptr()) if hasattr(out, "data_ptr") else _ptr(out)
        t = C.c_uint64()
        _check(N.load().gga_server_submit(self._h, graph_index, _algo(algo), src, ptr, C.byref(t)), "server_submit")
        self._outs[t.value] = out
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000):
        lat = C.c_double()
        _check(N.load().gga_server_wait(self._h, ticket, timeout_ms, C.byref(lat)), "server_wait")
        return self._outs.pop(ticket), lat.value

    def poll(self, ticket: int):
        lat = C.c_double()
        st = N.load().gga_server_wait(self._h, ticket, 0, C.byref(lat))
        if st == ERR_NOT_READY:
            return None
        _check(st, "server_poll")
        return self._outs.pop(ticket), lat.value

    def stats(self) -> dict:
        s = N.ServerStats()
        _check(N.load().gga_server_get_stats(self._h, C.byref(s)), "server_stats")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if self._h and self._h.value:
            N.load().gga_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def version() -> str:
    return N.load().gga_version().decode()
