"""Turns a kernel source file into host-compilable text for the emulator
(prelude.h): each kernel becomes a template on its block index, so its
__shared__ statics are per-block, and dynamic shared memory comes from a
per-block host array.  Usage: gen_kernels.py {frontier|sssp32|msbfs|mq|dmr} OUT"""
import os
import re
import sys

CS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "gpugraphalgo_gb300", "csrc")


def _read(name):
    return open(os.path.join(CS, name)).read()


def helpers():
    dev = _read("gga_device.cuh")
    dev = dev[dev.index("__device__ __forceinline__ bool grid_barrier("):dev.index("/* ---- host-side entry points")]
    return '#include "prelude.h"\n' + dev.replace("__device__ __forceinline__ bool grid_barrier(",
                                                   "template <int BLK> __device__ __forceinline__ bool grid_barrier(")


def transform(name, start, end, kernels, dyn):
    s = _read(name)
    s = s[s.index(start):s.index(end)]
    for k in kernels:
        s = re.sub(r"__global__ void (__launch_bounds__\([^)]*\) )?" + k + r"\(", "template <int BLK> void " + k + "(", s)
    for decl, var in dyn:
        s = s.replace(decl, f'{var} = ({var.split("*")[0].strip()} *)g_dyn[BLK];')
    return s.replace("grid_barrier(", "grid_barrier<BLK>(").replace("__global__ ", "")


def generate(which):
    if which == "frontier":
        hdr = _read("frontier.cuh")
        hdr = hdr[hdr.index("/* Control block"):hdr.index("gga_status frontier_scratch_ensure")]
        body = transform("frontier.cu", "constexpr uint32_t NONE", "template <int BS, bool SSSP>\nsize_t dyn_smem", [],
                         [("extern __shared__ uint32_t dyn[];", "uint32_t *dyn")])
        body = re.sub(r"template <int BS, bool SSSP>\nvoid __launch_bounds__\([^\n]*\) k_frontier\(Args a\)",
                      "template <int BS, bool SSSP, int BLK>\nvoid k_frontier(Args a)", body)
        body = hdr + body
    elif which == "sssp32":
        body = transform("sssp32.cu", "constexpr uint32_t SU_BS", "/* Source-major output", ["k_sssp32"],
                         [("extern __shared__ uint32_t dyn[];", "uint32_t *dyn")])
    elif which == "msbfs":
        body = transform("msbfs.cu", "constexpr uint32_t MB_BS", "/* Source-major output: out[s * n + v]", ["k_msbfs"],
                         [("extern __shared__ unsigned long long dyn64[];", "unsigned long long *dyn64")])
    elif which == "mq":
        hdr = _read("batch.cuh")
        start = "/* Queries per launch" if "/* Queries per launch" in hdr else "/* One query as"
        hdr = hdr[hdr.index(start):hdr.index("/* Device buffers")]
        src = _read("batch.cu")
        first = "constexpr uint32_t NONE" if "constexpr uint32_t NONE" in src else "constexpr uint32_t MQ_BS"
        body = hdr + transform("batch.cu", first, "/* Reached vertices", ["k_mq"],
                               [("extern __shared__ uint32_t dyn[];", "uint32_t *dyn")])
    elif which == "dmr":
        body = transform("dmr.cu", "constexpr uint32_t NONE", "struct DmrBufs",
                         ["k_shadow", "k_mark_all", "k_bad_count", "k_bad_gather", "k_decide", "k_resolve0", "k_reclaim", "k_resolve1",
                          "k_compact", "k_commit", "k_finish", "k_tail"], [])
        body = re.sub(r"template <bool PF>\nvoid __launch_bounds__\(PLAN_BS\) k_plan\(DmrArgs a\)",
                      "template <bool PF, int BLK>\nvoid k_plan(DmrArgs a)", body)
    else:
        raise SystemExit("unknown kernel " + which)
    return helpers() + "\n" + body


if __name__ == "__main__":
    open(sys.argv[2], "w").write(generate(sys.argv[1]))
