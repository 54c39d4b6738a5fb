"""ctypes binding of _ref/libref.so: a few of the reference's own functions
compiled from its sources (ref_probe.cpp, built by `make ref`).

TEST INFRASTRUCTURE ONLY: used to generate the golden fixtures under
tests/golden/ and, where the reference sources are present, to check the
oracle against reference code directly. load() returns None where the
library was not built (no reference sources).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libref.so")
REF_DIR = os.environ.get("VSR_REFERENCE_DIR", "/root/reference")

FP = ctypes.POINTER(ctypes.c_float)
UP = ctypes.POINTER(ctypes.c_uint32)
IP = ctypes.POINTER(ctypes.c_int32)

_lib = None


def build():
    """Compile _ref/libref.so when the reference sources are present;
    returns its path, or None."""
    if not os.path.isdir(REF_DIR):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_DIR}"], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is None and os.path.exists(LIB_PATH):
        lib = ctypes.CDLL(LIB_PATH)
        lib.ref_lcg.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, FP, UP]
        lib.ref_dda.restype = ctypes.c_int
        lib.ref_dda.argtypes = [FP, FP, ctypes.c_float, ctypes.c_float, IP, FP, FP, IP, FP,
                                ctypes.c_int]
        lib.ref_cvt.argtypes = [FP, ctypes.c_int, ctypes.c_int, UP]
        _lib = lib
    return _lib


def _f(a):
    return np.ascontiguousarray(a, np.float32)


def lcg(seed0, seed1, n):
    """(values float32[n], states uint32[n]) of LCG<4> seeded (seed0, seed1)."""
    v = np.zeros(n, np.float32)
    s = np.zeros(n, np.uint32)
    load().ref_lcg(seed0 & 0xFFFFFFFF, seed1 & 0xFFFFFFFF, n, v.ctypes.data_as(FP),
                   s.ctypes.data_as(UP))
    return v, s


def dda(ori, dirv, tmin, tmax, dims, lo, hi, max_cells=4096):
    """(cell ids int32[k], t0/t1 float32[k, 2]) visited by dda3."""
    cells = np.zeros(max_cells, np.int32)
    t01 = np.zeros((max_cells, 2), np.float32)
    o, d, l, h = _f(ori), _f(dirv), _f(lo), _f(hi)
    dm = np.ascontiguousarray(dims, np.int32)
    n = load().ref_dda(o.ctypes.data_as(FP), d.ctypes.data_as(FP), float(tmin), float(tmax),
                       dm.ctypes.data_as(IP), l.ctypes.data_as(FP), h.ctypes.data_as(FP),
                       cells.ctypes.data_as(IP), t01.ctypes.data_as(FP), max_cells)
    n = min(n, max_cells)
    return cells[:n].copy(), t01[:n].copy()


def cvt(rgba, srgb):
    """uint32[n] packed RGBA8 of float rgba[n, 4] (cvt_uint32 / cvt_uint32_srgb)."""
    c = _f(rgba).reshape(-1, 4)
    out = np.zeros(len(c), np.uint32)
    load().ref_cvt(c.ctypes.data_as(FP), len(c), int(bool(srgb)), out.ctypes.data_as(UP))
    return out
