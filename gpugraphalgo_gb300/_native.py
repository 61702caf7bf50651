"""ctypes declarations of the C ABI in include/gga.h.

The shared library is built in place by ``gpugraphalgo_gb300.build`` (or
``__graft_entry__.build()``) as ``gpugraphalgo_gb300/libgga.so``.  Loading it
does not need a GPU; solving does, and fails with ``GGA_ERR_NO_DEVICE`` when
there is none.  There is no fallback path: without the library nothing here
works.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgga.so")

u32 = C.c_uint32
u64 = C.c_uint64
i32 = C.c_int32
P = C.c_void_p
PU32 = C.POINTER(C.c_uint32)
PU64 = C.POINTER(C.c_uint64)


class Stats(C.Structure):
    _fields_ = [
        ("iterations", u32),
        ("kernel_launches", u32),
        ("vertices_reached", u64),
        ("edges_reached", u64),
        ("edges_relaxed", u64),
        ("cdp_children", u32),
        ("cdp_fallbacks", u32),
        ("kernel_ms", C.c_double),
        ("aux_ms", C.c_double),
        ("total_ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GraphInfo(C.Structure):
    _fields_ = [
        ("nnodes", u32),
        ("nodes_orig", u32),
        ("nedges", u32),
        ("maxdeg", u32),
        ("split_level", i32),
        ("split_buckets", i32),
        ("mda", u32),
        ("parents_with_children", u32),
        ("max_weight", u32),
        ("symmetric", i32),
        ("wsymmetric", i32),
    ]


class RoundTrace(C.Structure):
    _fields_ = [("kind", u32), ("items", u32), ("edges", u32), ("far_items", u32), ("ns", u32)]


class ConvRecord(C.Structure):
    _fields_ = [("iteration", u32), ("pad", u32), ("diff_count", C.c_uint64), ("norm2", C.c_double)]


class Params(C.Structure):
    _fields_ = [
        ("block_threads", u32),
        ("unit_iters", u32),
        ("sssp_delta", u32),
        ("use_split", u32),
        ("blocks_per_sm", u32),
        ("cdp_level", i32),
        ("cdp_buckets", i32),
        ("cdp_mode", u32),
        ("cdp_pending_limit", u32),
        ("skip_reached", u32),
        ("bfs_direction", u32),
        ("bfs_alpha", u32),
        ("bfs_beta", u32),
        ("sssp_light_heavy", u32),
        ("sssp_pull", u32),
        ("sssp_tail", u32),
        ("expansion", u32),
        ("split_level", i32),
        ("split_buckets", i32),
        ("batch_delta", u32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ResultRow(C.Structure):
    _fields_ = [
        ("exename", C.c_char * 100),
        ("algo", C.c_char * 10),
        ("graphfile", C.c_char * 200),
        ("bucket_size", u32),
        ("nnode", u32),
        ("nedge", u32),
        ("ns_nnode", u32),
        ("ns_nedge", u32),
        ("extranode", u32),
        ("maxdeg", u32),
        ("splitlevel", u32),
        ("max_edges_allowed", u32),
        ("iterations", u32),
        ("runtime", u32),
        ("time", C.c_float),
        ("ktime", C.c_float),
        ("sktime", C.c_float),
    ]


class Query(C.Structure):
    _fields_ = [("graph", P), ("algo", u32), ("src", u32), ("dist_out", P)]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", u64),
        ("completed", u64),
        ("rejected", u64),
        ("max_inflight", u32),
        ("supersteps", u32),
        ("state_bytes_peak", u64),
    ]


class MeshInfo(C.Structure):
    _fields_ = [("npoints", u32), ("ntriangles", u32)]


class MeshCheck(C.Structure):
    _fields_ = [
        ("bad_triangles", u64),
        ("bad_orientation", u64),
        ("bad_neighbors", u64),
        ("non_delaunay_edges", u64),
        ("boundary_edges", u64),
        ("area", C.c_double),
    ]


class RefineStats(C.Structure):
    _fields_ = [
        ("triangles_in", u32),
        ("bad_in", u32),
        ("triangles_out", u32),
        ("bad_out", u32),
        ("points_out", u32),
        ("rounds", u32),
        ("insertions", u64),
        ("boundary_splits", u64),
        ("failed_plans", u64),
        ("total_ms", C.c_double),
        ("device_ms", C.c_double),
        ("alloc_ms", C.c_double),
        ("upload_ms", C.c_double),
        ("download_ms", C.c_double),
    ]


class RefineParams(C.Structure):
    _fields_ = [("min_angle_deg", C.c_double), ("max_triangles", u32), ("batch_cap", u32), ("tail_max", u32),
                ("prefetch_max", u32)]


PD = C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol declared in include/gga.h
SIGNATURES = {
    "gga_status_string": (C.c_char_p, [C.c_int]),
    "gga_last_error": (C.c_char_p, []),
    "gga_version": (C.c_char_p, []),
    "gga_graph_load_gr": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "gga_graph_save_gr": (C.c_int, [P, C.c_char_p]),
    "gga_graph_from_csr": (C.c_int, [u32, u32, P, P, P, C.POINTER(P)]),
    "gga_graph_gen_rmat": (C.c_int, [u32, u32, C.c_double, C.c_double, C.c_double, u64, u32, u32, C.POINTER(P)]),
    "gga_graph_gen_grid": (C.c_int, [u32, u32, C.c_double, C.c_double, u64, u32, u32, C.POINTER(P)]),
    "gga_graph_free": (None, [P]),
    "gga_graph_get_info": (C.c_int, [P, C.POINTER(GraphInfo)]),
    "gga_graph_csr": (C.c_int, [P, C.POINTER(PU32), C.POINTER(PU32), C.POINTER(PU32)]),
    "gga_max_degree": (C.c_int, [P, PU32]),
    "gga_max_allowed_out_degree": (C.c_int, [P, i32, PU32]),
    "gga_size_after_split": (C.c_int, [P, i32, i32, PU32, PU32]),
    "gga_node_split": (C.c_int, [P, P, i32, i32]),
    "gga_graph_split_maps": (C.c_int, [P, P, P, P, P, P, P, P]),
    "gga_child_index": (C.c_int, [P, P, PU32, P, P]),
    "gga_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "gga_ctx_destroy": (None, [P]),
    "gga_graph_upload": (C.c_int, [P, P]),
    "gga_ctx_device_info": (C.c_int, [P, C.POINTER(C.c_int), C.c_char_p, C.c_size_t]),
    "gga_ctx_mark": (C.c_int, [P, C.c_int]),
    "gga_ctx_elapsed": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "gga_ctx_synchronize": (C.c_int, [P]),
    "gga_graph_pin": (C.c_int, [P, C.c_int]),
    "gga_graph_release_device": (C.c_int, [P]),
    "gga_graph_prepare": (C.c_int, [P, P, C.c_int]),
    "gga_bfs": (C.c_int, [P, P, u32, C.c_int, P, C.POINTER(Stats)]),
    "gga_sssp": (C.c_int, [P, P, u32, C.c_int, P, C.POINTER(Stats)]),
    "gga_solve": (C.c_int, [P, P, C.c_int, u32, C.c_int, P, C.POINTER(Stats)]),
    "gga_solve_many": (C.c_int, [P, P, C.c_int, u32, P, P, C.POINTER(Stats)]),
    "gga_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
    "gga_host_free": (None, [P]),
    "gga_set_params": (C.c_int, [P, C.POINTER(Params)]),
    "gga_get_params": (C.c_int, [P, C.POINTER(Params)]),
    "gga_autotune": (C.c_int, [P, P, u32, C.POINTER(Params)]),
    "gga_autotune_report": (C.c_int, [P, C.c_char_p, C.c_size_t]),
    "gga_verify": (C.c_int, [P, C.c_int, P, PU64]),
    "gga_write_dist": (C.c_int, [C.c_char_p, P, P]),
    "gga_reached": (C.c_int, [P, P, PU64, PU64]),
    "gga_write_result_row": (C.c_int, [C.c_char_p, C.POINTER(ResultRow)]),
    "gga_bfs_noalloc": (C.c_int, [P, P, u32, u32, u32, P, P]),
    "gga_msbfs": (C.c_int, [P, P, u32, P, P, C.POINTER(Stats)]),
    "gga_sssp_batch": (C.c_int, [P, P, u32, P, P, C.POINTER(Stats)]),
    "gga_multi_solve": (C.c_int, [P, u32, C.POINTER(Query), C.POINTER(Stats)]),
    "gga_server_create": (C.c_int, [P, u32, C.POINTER(P), u64, u32, C.POINTER(P)]),
    "gga_server_submit": (C.c_int, [P, u32, C.c_int, u32, P, PU64]),
    "gga_server_wait": (C.c_int, [P, u64, u32, C.POINTER(C.c_double)]),
    "gga_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
    "gga_server_destroy": (None, [P]),
    "gga_trace_enable": (C.c_int, [P, C.c_int]),
    "gga_convergence": (C.c_int, [P, P, C.c_int, u32, C.c_int, P, C.POINTER(ConvRecord), u32, C.POINTER(u32), P]),
    "gga_trace_get": (C.c_int, [P, C.POINTER(RoundTrace), u32, C.POINTER(u32), C.POINTER(u32), u32, C.POINTER(u32)]),
    "gga_mesh_load_triangle": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "gga_mesh_save_triangle": (C.c_int, [P, C.c_char_p]),
    "gga_mesh_from_arrays": (C.c_int, [u32, P, P, u32, P, C.POINTER(P)]),
    "gga_mesh_gen_jittered": (C.c_int, [u32, u32, C.c_double, u64, C.POINTER(P)]),
    "gga_mesh_gen_random": (C.c_int, [u32, u64, C.POINTER(P)]),
    "gga_mesh_free": (None, [P]),
    "gga_mesh_get_info": (C.c_int, [P, C.POINTER(MeshInfo)]),
    "gga_mesh_arrays": (C.c_int, [P, C.POINTER(PD), C.POINTER(PD), C.POINTER(PU32), C.POINTER(PU32)]),
    "gga_mesh_check": (C.c_int, [P, C.c_double, C.POINTER(MeshCheck)]),
    "gga_mesh_refine": (C.c_int, [P, P, C.c_double, u32, u32, C.POINTER(RefineStats)]),
    "gga_mesh_refine_ex": (C.c_int, [P, P, C.POINTER(RefineParams), C.POINTER(RefineStats)]),
}

_lib = None


def load():
    """Loads libgga.so once; raises RuntimeError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
