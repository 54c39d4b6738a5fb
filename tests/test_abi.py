"""The C ABI library: builds, loads and exports what include/vsr.h declares.

No compute calls: these run without a GPU.
"""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vsr.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"VSR_API\s+[^;(]*?\b(vsr\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path(pkg):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "vsr_build", os.path.join(ROOT, "anari-visionaray_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "vsrNewDevice" in syms and "vsrRenderFrame" in syms and "vsrMapFrame" in syms
    assert len(syms) >= 28


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    for s in declared_symbols():
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(vsr\w+)", out))
    assert set(declared_symbols()) <= exported


def test_python_binding_covers_the_header(pkg):
    assert sorted(pkg.vsr.EXPORTED_SYMBOLS) == declared_symbols()


def test_no_gpu_means_no_device(pkg):
    """Without a CUDA device the library refuses to create a device (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="no CUDA device"):
        pkg.vsr.Device()
