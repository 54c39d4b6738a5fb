"""Device functions of the renderer core against fixtures made from the
reference's own code (tests/golden/, see make_golden.py): the LCG<4> stream,
the dda3 cell walk and the RGBA8 colour conversion, run on the GPU through
libvsr_probe.so, which calls the same inline device functions the render
kernels use (Rng, ddaWalk, packRGBA8).

Bars: the LCG and the UFIXED8 conversion bit for bit; the DDA's cells and
[t0, t1] bit for bit (the walk rounds the two products a compiler would
fuse, as the reference does); sRGB8 within one step of 255 (CUDA's powf and
the host's pow may differ by an ulp before truncation).
"""
import ctypes
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FP = ctypes.POINTER(ctypes.c_float)
UP = ctypes.POINTER(ctypes.c_uint32)
IP = ctypes.POINTER(ctypes.c_int32)


def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def probe(pkg, device):
    path = os.path.join(os.path.dirname(pkg.__file__), "libvsr_probe.so")
    lib = ctypes.CDLL(path)
    lib.vsrProbeLcg.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, FP, UP]
    lib.vsrProbeDda.argtypes = [FP, ctypes.c_int, IP, FP, FP, ctypes.c_int, IP, IP, FP, UP]
    lib.vsrProbeCvt.argtypes = [FP, ctypes.c_int, ctypes.c_int, UP]
    return lib


def test_device_lcg_equals_reference(probe):
    for c in golden("lcg.json"):
        n = len(c["values"])
        v = np.zeros(n, np.float32)
        s = np.zeros(n, np.uint32)
        assert probe.vsrProbeLcg(c["seed"][0], c["seed"][1], n, v.ctypes.data_as(FP),
                                 s.ctypes.data_as(UP)) == 0
        assert np.array_equal(v, np.asarray(c["values"], np.float32)), c["seed"]
        assert np.array_equal(s, np.asarray(c["states"], np.uint32)), c["seed"]


def test_device_dda_equals_reference(probe):
    cases = golden("dda.json")
    max_cells = 256
    for grid in ("voxel32", "world16", "ragged"):
        cs = [c for c in cases if c["grid"] == grid]
        rays = np.array([c["ori"] + c["dir"] + [c["tmin"], c["tmax"]] for c in cs], np.float32)
        n = len(cs)
        counts = np.zeros(n, np.int32)
        cells = np.zeros((n, max_cells), np.int32)
        t01 = np.zeros((n, max_cells, 2), np.float32)
        errs = np.zeros(n, np.uint32)
        dims = np.asarray(cs[0]["dims"], np.int32)
        lo, hi = np.asarray(cs[0]["lo"], np.float32), np.asarray(cs[0]["hi"], np.float32)
        assert probe.vsrProbeDda(rays.ctypes.data_as(FP), n, dims.ctypes.data_as(IP),
                                 lo.ctypes.data_as(FP), hi.ctypes.data_as(FP), max_cells,
                                 counts.ctypes.data_as(IP), cells.ctypes.data_as(IP),
                                 t01.ctypes.data_as(FP), errs.ctypes.data_as(UP)) == 0
        assert not errs.any()
        for i, c in enumerate(cs):
            k = len(c["cells"])
            assert counts[i] == k, (grid, i)
            assert cells[i, :k].tolist() == c["cells"], (grid, i)
            assert np.array_equal(t01[i, :k], np.asarray(c["t01"], np.float32).reshape(-1, 2)), \
                (grid, i)


def test_device_color_conversion_equals_reference(probe):
    g = golden("cvt.json")
    rgba = np.ascontiguousarray(g["rgba"], np.float32)
    n = len(rgba)
    for fmt, srgb in (("ufixed8", 0), ("srgb8", 1)):
        out = np.zeros(n, np.uint32)
        assert probe.vsrProbeCvt(rgba.ctypes.data_as(FP), n, srgb, out.ctypes.data_as(UP)) == 0
        ref = np.asarray(g[fmt], np.uint32)
        if not srgb:
            assert np.array_equal(out, ref)
        else:
            diff = np.abs(np.stack([(out >> (8 * k)) & 255 for k in range(4)], -1).astype(np.int64)
                          - np.stack([(ref >> (8 * k)) & 255 for k in range(4)], -1))
            print("sRGB8 words differing:", int((diff.max(-1) > 0).sum()), "of", n)
            assert diff.max() <= 1
