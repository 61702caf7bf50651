"""The C ABI library: loads without a GPU and exports every declared symbol."""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import pytest

import gpugraphalgo_gb300 as gga
from gpugraphalgo_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(gga_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_native.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert sorted(_native.SIGNATURES) == declared_functions()


def test_nm_shows_extern_c_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH], capture_output=True, text=True).stdout
    for n in declared_functions():
        assert re.search(rf"\bT {n}$", out, flags=re.M), n


def test_version_and_status_strings():
    assert "sm_103a" in gga.version()
    lib = _native.load()
    assert lib.gga_status_string(gga.ERR_SPLIT_RULE).decode().startswith("split rule")


def test_context_without_gpu_fails_cleanly():
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = os.path.exists("/dev/nvidia0")
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(gga.GGAError) as e:
        gga.Context(0)
    assert e.value.status in (gga.ERR_NO_DEVICE, gga.ERR_CUDA)


def test_noalloc_host_checks_run_before_any_device_call():
    """gga_bfs_noalloc's argument checks are host-side: NULL pointers and
    graphs beyond its fixed working memory are rejected before any CUDA call,
    with the status a caller maps (no GPU needed)."""
    lib = _native.load()
    buf = (ctypes.c_uint32 * 8)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    assert lib.gga_bfs_noalloc(None, p, 4, 4, 0, p, None) == gga.ERR_INVALID_ARG
    assert lib.gga_bfs_noalloc(p, p, 4, 4, 0, None, None) == gga.ERR_INVALID_ARG
    assert lib.gga_bfs_noalloc(p, p, 4, 4, 4, p, None) == gga.ERR_INVALID_ARG  # source >= n
    assert lib.gga_bfs_noalloc(p, p, (1 << 18) + 1, 4, 0, p, None) == gga.ERR_TOO_LARGE
    assert "fixed working memory" in lib.gga_last_error().decode()
    assert lib.gga_bfs_noalloc(p, p, 4, (1 << 23) + 1, 0, p, None) == gga.ERR_TOO_LARGE
