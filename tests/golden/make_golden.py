"""Generate the known-answer fixtures under tests/golden/ from the
reference's own code.

The reference's LCG<4> (common.h:55-102), dda3 (renderer/DDA.h:12-113 with
GridAccel-common.h:9-25) and cvt_uint32 / cvt_uint32_srgb
(frame/common.h:31-48) are compiled from the reference sources by
`make -C oracle ref` (oracle/ref_probe.cpp; Visionaray's vector types and
linear_to_srgb come from the stand-in in oracle/ref_shim/) and called here
through oracle/refprobe.py:

  lcg.json : values and generator states for fixed seeds (the values are
             also cross-checked against an independent pure-Python
             restatement of the integer arithmetic below);
  dda.json : cells and [t0, t1] visited by dda3 for seeded rays over a
             32^3 grid on [0,1]^3 (the voxel-space brick grid the renderer
             walks), a 16^3 grid over world bounds (the reference CPU
             device's grid) and a ragged 5 x 7 x 3 grid, including rays
             parallel to an axis, rays starting inside, and rays clipped to
             the box first as delta tracking does;
  cvt.json : packed RGBA8 words of seeded colours in [-0.5, 1.5] and of
             edge values (0, 1, k/255 and their neighbours, the sRGB knee).

Needs the reference sources (VSR_REFERENCE_DIR, default /root/reference).
Run: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import refprobe  # noqa: E402

M = 0xFFFFFFFF


def lcg_init(v0, v1):
    s0 = 0
    for _ in range(4):
        s0 = (s0 + 0x9E3779B9) & M
        v0 = (v0 + ((((v1 << 4) & M) + 0xA341316C) & M ^ ((v1 + s0) & M) ^ (((v1 >> 5) + 0xC8013EA4) & M))) & M
        v1 = (v1 + ((((v0 << 4) & M) + 0xAD90777D) & M ^ ((v0 + s0) & M) ^ (((v0 >> 5) + 0x7E95761E) & M))) & M
    return v0


def lcg_sequence(v0, v1, n):
    st = lcg_init(v0, v1)
    out = []
    for _ in range(n):
        st = (1664525 * st + 1013904223) & M
        out.append((st & 0x00FFFFFF) / float(0x01000000))
    return out


LCG_SEEDS = [(0, 0), (1, 0), (0, 1), (12345, 7), (1048575, 1023), (0xFFFFFFFF, 0xFFFFFFFF),
             (511 + 1024 * 300, 0), (1920 * 1080 - 1, 1023), (77, 1000)]


def make_lcg():
    data = []
    for s in LCG_SEEDS:
        v, st = refprobe.lcg(s[0], s[1], 32)
        indep = np.array(lcg_sequence(s[0], s[1], 32), np.float32)
        assert np.array_equal(v, indep), s
        data.append({"seed": list(s), "values": [float(x) for x in v],
                     "states": [int(x) for x in st]})
    return data


def clip_to_box(o, d, lo, hi, tmin, tmax):
    """Box entry / exit in float32, as the renderer clips a ray before the
    walk (empty when the ray misses)."""
    o, d = np.float32(o), np.float32(d)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.float32(1.0) / d
        t1 = (np.float32(lo) - o) * inv
        t2 = (np.float32(hi) - o) * inv
    tn = np.float32(np.nanmax(np.fmin(t1, t2)))
    tf = np.float32(np.nanmin(np.fmax(t1, t2)))
    if not tn <= tf:
        return None
    return max(np.float32(tmin), tn), min(np.float32(tmax), tf)


def dda_cases():
    rng = np.random.default_rng(0x5EED0D0A)
    grids = [("voxel32", (32, 32, 32), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)),
             ("world16", (16, 16, 16), (-10.0, -10.0, -10.0), (10.0, 10.0, 10.0)),
             ("ragged", (5, 7, 3), (-1.0, 0.5, 2.0), (3.0, 2.0, 2.75))]
    cases = []
    for name, dims, lo, hi in grids:
        lo_a, hi_a = np.array(lo, np.float32), np.array(hi, np.float32)
        ext = hi_a - lo_a
        for k in range(40):
            kind = k % 4
            d = rng.normal(size=3)
            if kind == 3:  # parallel to one or two axes
                d[rng.integers(0, 3)] = 0.0
                if k % 8 == 7:
                    d[(rng.integers(0, 3))] = 0.0
                if not np.any(d):
                    d[0] = 1.0
            d = (d / np.linalg.norm(d)).astype(np.float32)
            if kind == 1:  # starts inside
                o = (lo_a + rng.uniform(0.05, 0.95, 3) * ext).astype(np.float32)
                tmin, tmax = np.float32(0.0), np.float32(rng.uniform(0.2, 3.0) * ext.max())
            else:  # from outside towards a point inside, clipped to the box
                target = lo_a + rng.uniform(0.1, 0.9, 3) * ext
                o = (target - d * rng.uniform(1.5, 3.0) * ext.max()).astype(np.float32)
                if kind == 3:
                    o = (target - d * 2.0 * ext.max()).astype(np.float32)
                clip = clip_to_box(o, d, lo_a, hi_a, 0.0, 1e30)
                if clip is None:
                    continue
                tmin, tmax = clip
                if kind == 2:  # stop inside the box
                    tmax = np.float32(tmin + np.float32(0.5) * (tmax - tmin))
            cells, t01 = refprobe.dda(o, d, tmin, tmax, dims, lo, hi)
            cases.append({"grid": name, "dims": list(dims), "lo": list(lo), "hi": list(hi),
                          "ori": [float(x) for x in o], "dir": [float(x) for x in d],
                          "tmin": float(tmin), "tmax": float(tmax),
                          "cells": [int(c) for c in cells],
                          "t01": [[float(a), float(b)] for a, b in t01]})
    return cases


def cvt_cases():
    rng = np.random.default_rng(0x5EED0C07)
    rnd = rng.uniform(-0.5, 1.5, (256, 4)).astype(np.float32)
    edges = [0.0, 1.0, -0.0, 0.0031308, 0.04045, 0.5, 2.0, -1.0]
    for k in (1, 2, 3, 64, 127, 128, 200, 254, 255):
        v = np.float32(k / 255.0)
        edges += [float(v), float(np.nextafter(v, np.float32(0))), float(np.nextafter(v, np.float32(2)))]
    e = np.array(edges, np.float32)
    pad = (-len(e)) % 4
    e = np.concatenate([e, np.zeros(pad, np.float32)])
    # each edge value in every channel position
    edge_rgba = np.stack([np.roll(e, s) for s in range(4)], axis=1)
    rgba = np.concatenate([rnd, edge_rgba]).astype(np.float32)
    return {"rgba": rgba.tolist(),
            "ufixed8": [int(x) for x in refprobe.cvt(rgba, False)],
            "srgb8": [int(x) for x in refprobe.cvt(rgba, True)]}


def main():
    if refprobe.build() is None or refprobe.load() is None:
        sys.exit("the reference sources are needed to generate the fixtures")
    out = {"lcg.json": make_lcg(), "dda.json": dda_cases(), "cvt.json": cvt_cases()}
    for name, data in out.items():
        path = os.path.join(HERE, name)
        with open(path, "w") as f:
            json.dump(data, f, indent=None if name != "lcg.json" else 1)
        print("wrote", path)


if __name__ == "__main__":
    main()
