"""The C-ABI library loads and exports every entry point declared in
include/mulskips_gpu.h (no compute call: runs without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "mulskips_gpu.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mks_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared()
    assert "mks_run" in names and "mks_replay" in names and len(names) >= 20


def test_library_exports_every_symbol(engine_lib):
    from mulskips_gb300 import _native
    for name in declared():
        assert hasattr(engine_lib, name), f"{name} missing from libmulskips_gpu.so"
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"


def test_version_string(engine_lib):
    assert b"sm_103a" in engine_lib.mks_version()


def test_library_is_sm103a_cuda():
    # the library links the CUDA runtime; no host-only build exists
    lib = os.path.join(ROOT, "mulskips_gb300", "_lib", "libmulskips_gpu.so")
    assert os.path.exists(lib)
    data = open(lib, "rb").read()
    assert b"cudaLaunchKernel" in data or b"cudaGraphLaunch" in data
