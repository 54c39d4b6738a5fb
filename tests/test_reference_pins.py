"""The oracle pinned against the reference's own code (no GPU).

tests/golden/{lcg,dda,cvt}.json were produced by tests/golden/make_golden.py
from the reference's LCG<4> (common.h:55-102), dda3 (renderer/DDA.h:12-113)
and cvt_uint32 / cvt_uint32_srgb (frame/common.h:31-48), compiled from the
reference sources (oracle/ref_probe.cpp). The oracle must reproduce them bit
for bit. Where the reference sources are present, the oracle is also run
against the compiled reference functions on fresh seeded inputs.
"""
import ctypes
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def oracle_dda(oracle, c, max_cells=4096):
    lib = oracle.load()
    cells = np.zeros(max_cells, np.int32)
    t01 = np.zeros((max_cells, 2), np.float32)
    dims = (ctypes.c_int32 * 3)(*c["dims"])
    n = lib.or_dda(oracle.farr(3, c["ori"]), oracle.farr(3, c["dir"]), c["tmin"], c["tmax"], dims,
                   oracle.farr(3, c["lo"]), oracle.farr(3, c["hi"]),
                   cells.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                   t01.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), max_cells)
    return cells[:n], t01[:n]


def oracle_cvt(oracle, rgba, srgb):
    c = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(len(c), np.uint32)
    oracle.load().or_cvt(c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(c), int(srgb),
                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out


def test_lcg_values_from_reference_code(oracle):
    lib = oracle.load()
    for c in golden("lcg.json"):
        out = np.zeros(len(c["values"]), np.float32)
        lib.or_lcg_sequence(c["seed"][0], c["seed"][1], len(out), oracle.fptr(out))
        assert np.array_equal(out, np.asarray(c["values"], np.float32)), c["seed"]


def test_dda_cells_from_reference_code(oracle):
    cases = golden("dda.json")
    assert len(cases) >= 100
    assert {c["grid"] for c in cases} == {"voxel32", "world16", "ragged"}
    assert any(0.0 in c["dir"] for c in cases)  # axis-parallel rays are covered
    for c in cases:
        cells, t01 = oracle_dda(oracle, c)
        assert cells.tolist() == c["cells"], (c["grid"], c["ori"], c["dir"])
        assert np.array_equal(t01, np.asarray(c["t01"], np.float32).reshape(-1, 2))


@pytest.mark.parametrize("fmt", ["ufixed8", "srgb8"])
def test_color_conversion_from_reference_code(oracle, fmt):
    g = golden("cvt.json")
    got = oracle_cvt(oracle, g["rgba"], fmt == "srgb8")
    assert np.array_equal(got, np.asarray(g[fmt], np.uint32))


@pytest.fixture(scope="module")
def ref():
    import refprobe

    if not os.path.isdir(refprobe.REF_DIR):
        pytest.skip("reference sources not present")
    refprobe.build()
    if refprobe.load() is None:
        pytest.skip("reference functions not built")
    return refprobe


def test_lcg_live_against_reference(oracle, ref):
    rng = np.random.default_rng(11)
    lib = oracle.load()
    for _ in range(200):
        s0, s1 = (int(x) for x in rng.integers(0, 2 ** 32, 2))
        v, _ = ref.lcg(s0, s1, 8)
        out = np.zeros(8, np.float32)
        lib.or_lcg_sequence(s0, s1, 8, oracle.fptr(out))
        assert np.array_equal(out, v)


def test_dda_live_against_reference(oracle, ref):
    rng = np.random.default_rng(12)
    for k in range(400):
        dims = [int(x) for x in rng.integers(1, 40, 3)]
        lo = rng.uniform(-5, 5, 3).astype(np.float32)
        hi = (lo + rng.uniform(0.5, 8, 3)).astype(np.float32)
        o = (lo + rng.uniform(-0.5, 1.5, 3) * (hi - lo)).astype(np.float32)
        d = rng.normal(size=3)
        if k % 5 == 0:
            d[rng.integers(0, 3)] = 0.0
        d = (d / np.linalg.norm(d)).astype(np.float32)
        tmin = np.float32(rng.uniform(0, 2))
        tmax = np.float32(tmin + rng.uniform(0.1, 20))
        c = {"dims": dims, "lo": lo.tolist(), "hi": hi.tolist(), "ori": o.tolist(),
             "dir": d.tolist(), "tmin": float(tmin), "tmax": float(tmax)}
        cells, t01 = oracle_dda(oracle, c)
        rc, rt = ref.dda(o, d, tmin, tmax, dims, lo, hi)
        assert cells.tolist() == rc.tolist()
        assert np.array_equal(t01, rt)


def test_color_conversion_live_against_reference(oracle, ref):
    rng = np.random.default_rng(13)
    rgba = rng.uniform(-0.2, 1.2, (20000, 4)).astype(np.float32)
    for srgb in (False, True):
        assert np.array_equal(oracle_cvt(oracle, rgba, srgb), ref.cvt(rgba, srgb))
