#!/usr/bin/env python3
"""Benchmark of the BFS/SSSP hot path on one GB300 (replicas across GPUs).

Workload (the single-GPU configuration the metric is quoted on): R-MAT scale
22, edge factor 16 (a/b/c/d = .57/.19/.19/.05, seed 2), symmetrised, self
loops and duplicates removed, vertex ids permuted, int32 CSR, uint32 weights
U[1,255]; 64 random sources (degree > 0) run one after another, each a
single-source BFS and a single-source SSSP.  One step = all 128 traversals.
The graph (1 GB of CSR) is larger than the 129 MB L2, so no flush is needed
between steps.

value    GTEPS = sum of E_r over the step's traversals / device time of the
         step (CUDA events on the library's stream around K steps); E_r is
         the out-degree sum of reached vertices, directed edges counted once.
e2e      the same metric through the C ABI with HOST buffers: every step
         re-uploads the pinned CSR and copies each distance vector back.
roofline the dominant persistent kernel: algorithmic bytes per launch
         (BFS 8*E_r + 20*V_r, SSSP 12*E_r + 20*V_r) / its mean launch time
         against the measured HBM copy bandwidth.
cpu_baseline  the oracle (C restatement of the reference's serial
         findSerialBFS/SSSP, graph.h:115-184) on the host cores, one source
         per thread, on a bounded sample of the same workload.

--impl reference times that CPU path alone (the reference's implementation of
the path; it has no other runnable form on this machine) on the same metric.
Multi-GPU: launched with torchrun, every rank runs an independent replica of
the workload on its own GPU with its own sources ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SSSP/BFS GTEPS at RMAT-22; batched queries/s + p99 vs one-at-a-time, 1 GB300"
UNIT = "GTEPS"


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gga", choices=["gga", "reference"])
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--sources", type=int, default=64)
    ap.add_argument("--variant", default="frontier")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--autotune-trials", type=int, default=1)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-query and serving sections")
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="offered-load duration per Poisson rate")
    return ap.parse_args()


# ------------------------------------------------------------ distributed

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


# ------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()) if rows else None}


# ------------------------------------------------------------ workload

def make_workload(args, rank: int):
    import gpugraphalgo_gb300 as gga

    g = gga.Graph.rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=2, wmin=1, wmax=255)
    deg = g.degrees()
    rng = np.random.default_rng(2 + 1000 * rank)
    cand = np.nonzero(deg > 0)[0]
    srcs = [int(x) for x in rng.choice(cand, size=args.sources, replace=False)]
    return g, srcs


def algorithmic_bytes(algo: str, er: int, vr: int) -> int:
    return (8 if algo == "bfs" else 12) * er + 20 * vr


def read_traffic(kind: str):
    """dram bytes per launch from the committed ncu summary, scaled per edge."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        f = line.split()
        if len(f) >= 3 and f[0] == "bytes_per_edge_reached" and f[1] == kind:
            return float(f[2])
    return None


def cpu_baseline(g, srcs, threads: int, budget_sources: int):
    """Oracle serial BFS/SSSP (the reference's algorithm) on host threads."""
    import oracle

    off, col, wt = g.csr()
    og = oracle.OracleGraph.from_csr(off, col, wt)
    lib = oracle.load()
    deg = np.diff(off.astype(np.int64))
    sample = srcs[:budget_sources]
    results = {}

    def work(i, s):
        for algo in ("bfs", "sssp"):
            d = np.empty(len(off) - 1, np.uint32)
            lib.oracle_serial(og._h, 1 if algo == "sssp" else 0, s, oracle._p(d))
            reach = d < oracle.INF
            results[(i, algo)] = int(deg[reach].sum())

    t0 = time.perf_counter()
    ths = []
    for i, s in enumerate(sample):
        th = threading.Thread(target=work, args=(i, s))
        th.start()
        ths.append(th)
        if len(ths) >= threads:
            ths.pop(0).join()
    for th in ths:
        th.join()
    dt = time.perf_counter() - t0
    er = sum(results.values())
    return er / dt / 1e9, dt, len(sample)


def run_reference(args, dist: Dist):
    """--impl reference: the reference's CPU path (oracle port) on host cores."""
    if dist.rank != 0:
        return None
    g, srcs = make_workload(args, 0)
    threads = os.cpu_count() or 1
    per_step = max(2, min(threads, (threads * 6) // max(1, args.steps + args.warmup)))
    for w in range(args.warmup):
        cpu_baseline(g, srcs[w * per_step % len(srcs):][:per_step] or srcs[:per_step], threads, per_step)
    vals, secs = [], 0.0
    for k in range(args.steps):
        start = (k * per_step) % len(srcs)
        v, dt, _ = cpu_baseline(g, (srcs[start:] + srcs[:start])[:per_step], threads, per_step)
        vals.append(v)
        secs += dt
    value = statistics.mean(vals)
    sample = f"{per_step} sources x (BFS+SSSP) per step, one source per thread, R-MAT-{args.scale}"
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"rmat{args.scale}_ef{args.edge_factor}_seed2_{args.sources}src_bfs+sssp",
                   "sources": args.sources,
                   "implementation": "serial in-order Bellman-Ford sweeps (graph.h:115-184), oracle C port",
                   "parallelism": f"{threads} host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ------------------------------------------------------------ batching / serving

def _timed(fn, reps):
    best = []
    for _ in range(reps):
        t0 = time.perf_counter()
        r = fn()
        best.append(time.perf_counter() - t0)
    return r, statistics.median(best)


def batch_section(gga, ctx):
    """Batched queries in one launch against the same queries one at a time.

    Both sides copy every distance vector to page-locked host memory (the
    user-facing call); kernel-only rates come from the library's CUDA
    events."""
    res = {}
    g = gga.Graph.rmat(20, 16, 0.57, 0.19, 0.19, seed=4, wmin=1, wmax=255)
    g.cudaCopy(ctx)
    rng = np.random.default_rng(4)
    cand = np.nonzero(g.degrees() > 0)[0]
    s64 = [int(x) for x in rng.choice(cand, 64, replace=False)]
    s32 = s64[:32]

    # every output (batched and one-at-a-time) lands in page-locked host
    # rows allocated here, outside the timed calls
    def rows(sizes):
        block = gga.pinned_empty(int(sum(sizes)))
        out, at = [], 0
        for n in sizes:
            out.append(block[at:at + n])
            at += n
        return out

    def singles(qs, outs):
        kms = 0.0
        t0 = time.perf_counter()
        for (gg, algo, s), o in zip(qs, outs):
            _, st = ctx.solve(gg, algo, s, out=o, stats=True)
            kms += st["kernel_ms"]
        return outs, time.perf_counter() - t0, kms

    def record(name, nq, batch_out, bst, bwall, single_outs, swall, skms, er):
        same = all(np.array_equal(a, b) for a, b in zip(batch_out, single_outs))
        res[name] = {"queries": nq, "identical_to_single": bool(same),
                     "batch_qps": nq / bwall, "one_at_a_time_qps": nq / swall, "speedup": swall / bwall,
                     "batch_kernel_ms": bst["kernel_ms"], "one_at_a_time_kernel_ms": skms,
                     "kernel_speedup": skms / bst["kernel_ms"] if bst["kernel_ms"] else None,
                     "batch_ms": bwall * 1e3, "gteps_kernel": er / (bst["kernel_ms"] * 1e-3) / 1e9 if bst["kernel_ms"] else None,
                     "rounds": bst["iterations"], "edges_relaxed": bst["edges_relaxed"], "edges_reached": er}

    def reference_kernel(name, algo, srcs, batch_out, k=3):
        """The same queries through the reference's own kernel (topology-driven
        Bellman-Ford with atomicMin, the "na_" build), one launch sequence per
        query with the result copied to host: a sample of k queries."""
        t0 = time.perf_counter()
        outs = [ctx.solve(g, algo, s, "topo_atomic", out=o64[i]) for i, s in enumerate(srcs[:k])]
        dt = time.perf_counter() - t0
        res[name]["reference_kernel_one_at_a_time"] = {
            "qps": k / dt, "sample_queries": k, "batch_speedup": res[name]["batch_qps"] / (k / dt),
            "identical": bool(all(np.array_equal(a, b) for a, b in zip(outs, batch_out)))}

    b64, o64 = gga.pinned_empty((64, g.n)), rows([g.n] * 64)
    ctx.msbfs(g, s64, out=b64)
    (bo, bst), bw = _timed(lambda: ctx.msbfs(g, s64, stats=True, out=b64), 3)
    so, sw, sk = singles([(g, "bfs", s) for s in s64], o64)
    record("msbfs64_rmat20", 64, list(bo), bst, bw, so, sw, sk, bst["edges_reached"])
    reference_kernel("msbfs64_rmat20", "bfs", s64, bo)

    b32 = b64[:32]
    ctx.sssp_batch(g, s32, out=b32)
    (bo, bst), bw = _timed(lambda: ctx.sssp_batch(g, s32, stats=True, out=b32), 3)
    so, sw, sk = singles([(g, "sssp", s) for s in s32], o64[:32])
    record("sssp32_rmat20", 32, list(bo), bst, bw, so, sw, sk, bst["edges_reached"])
    reference_kernel("sssp32_rmat20", "sssp", s32, bo)

    gs = [gga.Graph.rmat(sc, 16, 0.57, 0.19, 0.19, seed=10 + i, wmin=1, wmax=255) for i, sc in enumerate(range(12, 21))]
    gs += [gga.Graph.grid(w, w, 0.05, 0.001, seed=19 + i, wmin=1, wmax=1000)
           for i, w in enumerate((256, 512, 768, 1024, 1280, 1536, 2048))]
    qs = []
    for j, gg in enumerate(gs):
        gg.cudaCopy(ctx)
        r = np.random.default_rng(100 + j)
        for s in r.choice(np.nonzero(gg.degrees() > 0)[0], 8, replace=False):
            qs += [(gg, "bfs", int(s)), (gg, "sssp", int(s))]
    mb, mo = rows([gg.n for gg, _, _ in qs]), rows([gg.n for gg, _, _ in qs])
    ctx.multi_solve(qs, outs=mb)
    (bo, bst), bw = _timed(lambda: ctx.multi_solve(qs, stats=True, outs=mb), 3)
    so, sw, sk = singles(qs, mo)
    record("mixed16x8_bfs+sssp", len(qs), bo, bst, bw, so, sw, sk, bst["edges_reached"])
    res["mixed16x8_bfs+sssp"]["graphs"] = "R-MAT 12..20 ef16 seeds 10-18, grids 256..2048 seeds 19-25"
    return res


def serving_section(gga, ctx, seconds: float, device: int):
    """Open-loop Poisson query streams against the continuous-batching server."""
    import torch

    specs = [("rmat", 16, 30), ("rmat", 18, 31), ("rmat", 20, 32), ("rmat", 21, 33),
             ("grid", 512, 34), ("grid", 1024, 35), ("grid", 1536, 36), ("grid", 2048, 37)]
    graphs = []
    for kind, size, seed in specs:
        if kind == "rmat":
            gg = gga.Graph.rmat(size, 16, 0.57, 0.19, 0.19, seed=seed, wmin=1, wmax=255)
        else:
            gg = gga.Graph.grid(size, size, 0.05, 0.001, seed=seed, wmin=1, wmax=1000)
        gg.cudaCopy(ctx)
        graphs.append(gg)
    ns = [gg.n for gg in graphs]
    W = 512
    ring = torch.empty((W, max(ns)), dtype=torch.int32, device=f"cuda:{device}")
    rng = np.random.default_rng(77)

    def draw(k):
        gi = rng.integers(0, len(graphs), k)
        al = np.where(rng.random(k) < 0.7, "bfs", "sssp")
        src = [int(rng.integers(0, ns[i])) for i in gi]
        return list(zip(gi.tolist(), al.tolist(), src))

    # sequential plain launches, one query at a time, same mix, device outputs
    seq = draw(300)
    for gi, al, s in seq[:20]:
        ctx.solve(graphs[gi], al, s, out=ring[0][: ns[gi]])
    ctx.synchronize()
    t0 = time.perf_counter()
    for k, (gi, al, s) in enumerate(seq):
        ctx.solve(graphs[gi], al, s, out=ring[k % W][: ns[gi]])
    ctx.synchronize()
    seq_qps = len(seq) / (time.perf_counter() - t0)
    # the reference's own kernel (topology-driven Bellman-Ford, "na_"), one
    # query at a time, on the first queries of the same mix (at most ~5 s)
    t0, nref = time.perf_counter(), 0
    for gi, al, s in seq[:8]:
        ctx.solve(graphs[gi], al, s, "topo_atomic", out=ring[nref % W][: ns[gi]])
        nref += 1
        if time.perf_counter() - t0 > 5.0:
            break
    ctx.synchronize()
    ref_qps = nref / (time.perf_counter() - t0)

    srv = gga.Server(ctx, graphs, mem_cap_bytes=60 << 30, max_slots=256)
    old_switch = sys.getswitchinterval()
    sys.setswitchinterval(0.0002)  # the submitting and the waiting thread share the GIL
    out = {"graphs": "R-MAT 16/18/20/21 ef16 seeds 30-33, grids 512/1024/1536/2048 seeds 34-37 (5% deleted, w 1..1000)",
           "mix": "70% BFS / 30% SSSP, uniform graph and source", "mem_cap_bytes": 60 << 30, "max_slots": 256,
           "superstep_rounds": 8, "sequential_qps": seq_qps,
           "reference_kernel_sequential": {"qps": ref_qps, "sample_queries": nref}, "rates": []}
    try:
        # exactness: served answers equal single-query answers
        chk = draw(24)
        tk = [srv.submit(gi, al, s) for gi, al, s in chk]
        mism = 0
        for (gi, al, s), t in zip(chk, tk):
            got, _ = srv.wait(t)
            mism += int(not np.array_equal(got, ctx.solve(graphs[gi], al, s)))
        out["identical_to_single"] = mism == 0
        for rate in (1000, 5000, 20000, 50000):
            nq = max(50, int(rate * seconds))
            qs = draw(nq)
            arrivals = np.cumsum(rng.exponential(1.0 / rate, nq))
            free = list(range(W))
            lock = threading.Condition()
            pending = []  # (ticket, slot, scheduled arrival, submit time)
            lat = []
            done_t = [0.0]

            def consumer():
                k = 0
                while k < nq:
                    with lock:
                        while not pending:
                            lock.wait()
                        t, slot, arr, sub = pending.pop(0)
                    _, l_us = srv.wait(t, 120000)
                    fin = sub + l_us * 1e-6
                    lat.append(fin - arr)
                    done_t[0] = max(done_t[0], fin)
                    with lock:
                        free.append(slot)
                        lock.notify_all()
                    k += 1

            th = threading.Thread(target=consumer)
            th.start()
            throttled = 0
            base = time.perf_counter()
            for (gi, al, s), a in zip(qs, arrivals):
                when = base + a
                while time.perf_counter() < when:
                    pass
                with lock:
                    if not free:
                        throttled += 1
                        while not free:
                            lock.wait()
                    slot = free.pop()
                sub = time.perf_counter()
                t = srv.submit(gi, al, s, out=ring[slot][: ns[gi]])
                with lock:
                    pending.append((t, slot, when, sub))
                    lock.notify_all()
            th.join()
            span = done_t[0] - base
            lat_ms = np.array(lat) * 1e3
            out["rates"].append({"offered_qps": rate, "queries": nq, "achieved_qps": nq / span,
                                 "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
                                 "throttled_submits": throttled, "window": W})
        out["stats"] = srv.stats()
        out["peak_qps_vs_sequential"] = max(r["achieved_qps"] for r in out["rates"]) / seq_qps
        out["peak_qps_vs_reference_kernel_sequential"] = max(r["achieved_qps"] for r in out["rates"]) / ref_qps
    finally:
        sys.setswitchinterval(old_switch)
        srv.close()
    return out


def run_gga(args, dist: Dist):
    import gpugraphalgo_gb300 as gga

    ctx = gga.Context(dist.local_rank)
    dev = ctx.device_info()
    g, srcs = make_workload(args, dist.rank)
    info = g.info()
    g.cudaCopy(ctx)
    params = ctx.autotune(g, args.autotune_trials)
    ctx.set_params(skip_reached=1)
    variant = args.variant

    # E_r / V_r per traversal (fixed by graph and source), outside the timing
    ctx.set_params(skip_reached=0)
    reach = {}
    for s in srcs:
        for algo in ("bfs", "sssp"):
            _, st = ctx.solve(g, algo, s, variant, stats=True, keep_on_device=True)
            reach[(algo, s)] = (st["edges_reached"], st["vertices_reached"])
    ctx.set_params(skip_reached=1)

    def step(record=None):
        launches = 0
        for s in srcs:
            for algo in ("bfs", "sssp"):
                _, st = ctx.solve(g, algo, s, variant, stats=True, keep_on_device=True)
                launches += st["kernel_launches"]
                if record is not None:
                    record[algo].append(st["kernel_ms"])
        return launches

    for _ in range(args.warmup):
        step()
    dist.barrier()
    ctx.synchronize()
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    rec = {"bfs": [], "sssp": []}
    launches = 0
    ctx.mark(0)
    for _ in range(args.steps):
        launches += step(rec)
    ctx.mark(1)
    ctx.synchronize()
    ms = ctx.elapsed(0, 1)
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)

    er_step = sum(e for e, _ in reach.values())
    er_total = dist.sum(er_step * args.steps)
    value = er_total / (ms_max * 1e-3) / 1e9

    bfs_er = sum(reach[("bfs", s)][0] for s in srcs)
    sssp_er = sum(reach[("sssp", s)][0] for s in srcs)
    bfs_ms = sum(rec["bfs"]) / args.steps
    sssp_ms = sum(rec["sssp"]) / args.steps
    kinds = {}
    for algo, tot_ms in (("bfs", bfs_ms), ("sssp", sssp_ms)):
        byts = sum(algorithmic_bytes(algo, *reach[(algo, s)]) for s in srcs) / len(srcs)
        per_launch_ms = tot_ms / len(srcs)
        kinds[algo] = {"bytes_per_launch": byts, "ms_per_launch": per_launch_ms,
                       "achieved_gbs": byts / (per_launch_ms * 1e-3) / 1e9}
    dom = "sssp" if sssp_ms >= bfs_ms else "bfs"
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    tpe = read_traffic(dom)
    er_mean = (sssp_er if dom == "sssp" else bfs_er) / len(srcs)
    roofline = {"bound": "hbm", "kernel": f"k_frontier<{params['block_threads']},{'true' if dom == 'sssp' else 'false'}>",
                "achieved": kinds[dom]["achieved_gbs"], "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                "frac": kinds[dom]["achieved_gbs"] / peak,
                "traffic": tpe * er_mean if tpe else None,
                "algorithmic_bytes": kinds[dom]["bytes_per_launch"],
                "per_kind": kinds}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"rmat{args.scale}_ef{args.edge_factor}_seed2_{args.sources}src_bfs+sssp",
                   "graph": f"R-MAT scale {args.scale} ef {args.edge_factor} a/b/c=.57/.19/.19 seed 2, symmetrised, "
                            "dedup, ids permuted, weights U[1,255]",
                   "vertices": info["nodes_orig"], "edges": info["nedges"], "maxdeg": info["maxdeg"],
                   "sources": args.sources, "parallelism": "replicas" if dist.world > 1 else "single",
                   "l2": "inputs larger than L2 (CSR %.2f GB vs 129 MB L2); no flush" % ((4 * (info["nodes_orig"] + 1) + 8 * info["nedges"]) / 1e9),
                   "variant": variant, "params": params, "device": dev["name"], "sms": dev["sms"]},
        "bfs_gteps": bfs_er / (bfs_ms * 1e-3) / 1e9,
        "sssp_gteps": sssp_er / (sssp_ms * 1e-3) / 1e9,
        "roofline": roofline,
        "gpu_launches": launches,
        "clocks": clk,
    }

    # reference algorithm (topology-driven Bellman-Ford, "na_") on the same GPU
    try:
        ta = {}
        for algo in ("bfs", "sssp"):
            _, st = ctx.solve(g, algo, srcs[0], "topo_atomic", stats=True, keep_on_device=True)
            ta[algo] = {"ms": st["kernel_ms"], "iterations": st["iterations"],
                        "gteps": reach[(algo, srcs[0])][0] / (st["kernel_ms"] * 1e-3) / 1e9}
        out["reference_algorithm_same_gpu"] = ta
    except Exception as e:  # reported, not fatal
        out["reference_algorithm_same_gpu"] = {"error": str(e)}

    # end to end through the C ABI with host buffers: every step uploads the
    # CSR again and copies every distance vector to page-locked host rows
    # (gga_solve_many overlaps each copy with the next traversal)
    if not args.no_e2e:
        g.pin(True)
        hout = {algo: gga.pinned_empty((len(srcs), info["nodes_orig"])) for algo in ("bfs", "sssp")}
        src_list = [int(s) for s in srcs]
        dist.barrier()
        e2e_steps = max(1, min(args.steps, 2))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            g.release_device()
            for algo in ("bfs", "sssp"):
                if variant in ("frontier", "auto"):
                    ctx.solve_many(g, algo, src_list, out=hout[algo])
                else:
                    for i, s in enumerate(src_list):
                        ctx.solve(g, algo, s, variant, out=hout[algo][i])
        ctx.synchronize()
        dt = time.perf_counter() - t0
        dt_max = dist.max(dt)
        out["e2e"] = {"value": dist.sum(er_step * e2e_steps) / dt_max / 1e9, "unit": UNIT,
                      "h2d_bytes_per_step": 4 * (info["nodes_orig"] + 1) + 8 * info["nedges"],
                      "d2h_bytes_per_step": 4 * info["nodes_orig"] * 2 * len(srcs),
                      "steps": e2e_steps}
        g.cudaCopy(ctx)

    if not args.no_batch and dist.rank == 0:
        # both sides of the batched comparisons use each graph's own defaults,
        # not the parameters tuned for the R-MAT-22 step above
        ctx.reset_params()
        try:
            out["batched"] = batch_section(gga, ctx)
        except Exception as e:  # reported, not fatal
            out["batched"] = {"error": repr(e)}
        try:
            out["serving"] = serving_section(gga, ctx, args.serve_seconds, dist.local_rank)
        except Exception as e:
            out["serving"] = {"error": repr(e)}

    if dist.rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, dt, ns = cpu_baseline(g, srcs, threads, min(threads, len(srcs)))
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": min(threads, ns), "kind": "port",
                               "sample": f"{ns} sources x (BFS+SSSP), one source per thread, {dt:.1f} s wall"}
    ctx.close()
    return out


def main():
    args = parse_args()
    dist = Dist()
    try:
        res = run_reference(args, dist) if args.impl == "reference" else run_gga(args, dist)
        if dist.rank == 0 and res is not None:
            print(json.dumps(res))
    finally:
        dist.close()


if __name__ == "__main__":
    main()
