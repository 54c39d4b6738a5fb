"""The CPU oracle pinned against known answers (no GPU).

The reference ships no tests, golden images or fixtures, so the oracle is
pinned by (a) golden vectors of the reference's LCG<4>, made by the
reference's own code compiled here (tests/golden/lcg.json; the DDA and
colour-conversion fixtures are checked in test_reference_pins.py), (b)
closed-form cases:
texel-centred trilinear sampling, a Lambertian plane under a directional
light, an emission-absorption slab, (c) brute-force cross-checks of the BVH
and of the majorant grid, and (d) invariants of the DDA and the BSDF
sampler.
"""
import ctypes
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_lcg_matches_golden(oracle):
    lib = oracle.load()
    with open(os.path.join(GOLDEN, "lcg.json")) as f:
        cases = json.load(f)
    for c in cases:
        out = np.zeros(len(c["values"]), np.float32)
        lib.or_lcg_sequence(c["seed"][0], c["seed"][1], len(out), oracle.fptr(out))
        assert np.array_equal(out, np.asarray(c["values"], np.float32)), c["seed"]


def _volume(oracle, data, tf):
    v = oracle.OrVolume()
    v._data = np.ascontiguousarray(data, np.float32)
    v._tf = np.ascontiguousarray(tf, np.float32)
    v.data = oracle.fptr(v._data)
    nz, ny, nx = v._data.shape
    v.dims = (ctypes.c_int32 * 3)(nx, ny, nz)
    v.origin = oracle.farr(3, [0, 0, 0])
    v.spacing = oracle.farr(3, [1, 1, 1])
    v.tf = oracle.fptr(v._tf)
    v.tfSize = len(v._tf)
    v.valueRange = oracle.farr(2, [0, 1])
    v.unitDistance = 1.0
    return v


def test_trilinear_texel_centres_and_clamp(oracle):
    lib = oracle.load()
    rng = np.random.default_rng(1)
    data = rng.uniform(0, 1, (5, 6, 7)).astype(np.float32)
    v = _volume(oracle, data, np.ones((4, 4)))
    nz, ny, nx = data.shape
    for (i, j, k) in [(0, 0, 0), (6, 5, 4), (3, 2, 1)]:
        p = ((i + 0.5) / nx, (j + 0.5) / ny, (k + 0.5) / nz)
        assert lib.or_sample_field(ctypes.byref(v), *p) == pytest.approx(data[k, j, i], abs=1e-6)
    # clamp addressing outside [0,1]
    assert lib.or_sample_field(ctypes.byref(v), -3.0, -3.0, -3.0) == pytest.approx(data[0, 0, 0])
    assert lib.or_sample_field(ctypes.byref(v), 4.0, 4.0, 4.0) == pytest.approx(data[-1, -1, -1])
    # linear along x between centres
    p = ((1 + 0.5 + 0.25) / nx, (2 + 0.5) / ny, (3 + 0.5) / nz)
    ref = 0.75 * data[3, 2, 1] + 0.25 * data[3, 2, 2]
    assert lib.or_sample_field(ctypes.byref(v), *p) == pytest.approx(ref, abs=1e-6)


def test_tf_lookup_bins(oracle):
    lib = oracle.load()
    tf = np.stack([np.linspace(0, 1, 8)] * 4, -1).astype(np.float32)
    v = _volume(oracle, np.zeros((2, 2, 2)), tf)
    out = np.zeros(4, np.float32)
    for i in range(8):
        lib.or_tf_lookup(ctypes.byref(v), (i + 0.5) / 8, oracle.fptr(out))
        assert np.allclose(out, tf[i])
    lib.or_tf_lookup(ctypes.byref(v), 2.0, oracle.fptr(out))
    assert np.allclose(out, tf[-1])


def test_tf_build_restatement(oracle):
    """TransferFunction1D::finalize resampling: 3 colours, 5 opacities -> 5 entries."""
    color = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    opacity = np.array([0, 0.25, 0.5, 0.75, 1.0], np.float32)
    tf = oracle.build_tf(color, opacity)
    assert tf.shape == (5, 4)
    assert np.allclose(tf[0], [1, 0, 0, 0])
    assert np.allclose(tf[2], [0, 1, 0, 0.5])
    assert np.allclose(tf[1], [0.5, 0.5, 0, 0.25])
    assert np.allclose(tf[4], [0, 0, 1, 1])


def plane_scene(color=(0.6, 0.5, 0.4), light_dir=(0.0, -0.6, -0.8), irradiance=2.0,
                renderer="raycast"):
    g = 50.0
    quad = np.array([[-g, -g, 0], [g, -g, 0], [g, g, 0], [-g, g, 0]], np.float32)
    return {
        "surfaces": [{"vertices": quad, "indices": np.array([[0, 1, 2], [0, 2, 3]], np.uint32),
                      "material": {"type": "matte", "color": list(color)}}],
        "volumes": [],
        "lights": [{"direction": list(light_dir), "irradiance": irradiance}],
        "camera": {"type": "perspective", "position": [0.0, 0.0, 10.0],
                   "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0],
                   "fovy": math.radians(30.0), "aspect": 1.0},
        "renderer": {"type": renderer, "ambientRadiance": 0.2, "background": [0, 0, 0, 1]},
        "frame": {"size": (16, 16)},
    }


def test_lambertian_plane_closed_form(oracle):
    """Raycast of a matte plane: c/pi * E * cos(theta) + c * ambient."""
    sc = plane_scene()
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16)
    oracle.render(S, F)
    c = np.array([0.6, 0.5, 0.4])
    L = -np.array([0.0, -0.6, -0.8])
    cos = max(0.0, float(np.dot([0, 0, 1], L / np.linalg.norm(L))))
    expect = c / math.pi * 2.0 * cos + c * 0.2
    assert np.allclose(F.color[..., :3], expect, atol=1e-5)
    assert np.allclose(F.color[..., 3], 1.0)
    assert np.allclose(F.depth[8, 8], 10.0, rtol=1e-3)
    assert np.allclose(F.normal, [0, 0, 1], atol=1e-6)
    assert np.allclose(F.albedo, c, atol=1e-6)


@pytest.mark.parametrize("kind", ["point", "spot"])
def test_point_and_spot_lights_closed_form(oracle, kind):
    """Raycast of a matte plane under a point or spot light (orthographic
    view from above): c/pi * color * intensity / d^2 * cos(theta) +
    c * ambient, times the spot's smoothstep between cos(openingAngle) and
    cos(openingAngle - 2 falloffAngle) of the angle to its axis."""
    pos = np.array([1.0, -0.5, 3.0])
    col, inten = np.array([1.0, 0.8, 0.6]), 5.0
    light = {"type": kind, "position": pos.tolist(), "intensity": inten, "color": col.tolist()}
    if kind == "spot":
        light.update(direction=[0.0, 0.0, -1.0], openingAngle=0.9, falloffAngle=0.2)
    sc = plane_scene()
    sc["lights"] = [light]
    sc["camera"] = {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                    "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 8.0,
                    "aspect": 1.0}
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16)
    oracle.render(S, F)
    xs = ((np.arange(16) + 0.5) / 16 - 0.5) * 8.0
    X, Y = np.meshgrid(xs, xs)  # rows are image y (up)
    L = pos[None, None, :] - np.stack([X, Y, np.zeros_like(X)], axis=-1)
    d2 = (L * L).sum(-1)
    cos = np.maximum(0.0, L[..., 2] / np.sqrt(d2))
    factor = np.ones_like(d2)
    if kind == "spot":
        spot = L[..., 2] / np.sqrt(d2)  # axis (0,0,-1) against the direction light -> point
        co, ci = math.cos(0.9), math.cos(0.9 - 0.4)
        u = np.clip((spot - co) / (ci - co), 0.0, 1.0)
        factor = np.where(spot < co, 0.0, np.where(spot > ci, 1.0, u * u * (3 - 2 * u)))
        assert (factor == 0).any() and (factor == 1).any() and ((factor > 0) & (factor < 1)).any()
    c = np.array([0.6, 0.5, 0.4])
    expect = (c / math.pi)[None, None, :] * (col * inten)[None, None, :] * \
        (cos * factor / d2)[..., None] + c * 0.2
    assert np.allclose(F.color[..., :3], expect, rtol=1e-4, atol=1e-5)


def test_sphere_closed_form(oracle):
    """Raycast of a matte sphere (centre (0.5, -0.25, 0), radius 2, placed
    through primitive.index with a per-sphere radius) seen from above by an
    orthographic camera under a directional light: each covered pixel is
    c/pi E max(0, n.L) + c ambient with n the analytic sphere normal at the
    pixel; the rest is background."""
    centre, r = np.array([0.5, -0.25, 0.0]), 2.0
    sc = plane_scene()
    sc["surfaces"] = [{"geometry": "sphere",
                       "vertices": np.array([[9.0, 9.0, 9.0], centre], np.float32),
                       "indices": np.array([1], np.uint32), "radii": np.array([r], np.float32),
                       "material": {"type": "matte", "color": [0.6, 0.5, 0.4]}}]
    sc["camera"] = {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                    "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 6.0,
                    "aspect": 1.0}
    S = oracle.Scene(sc)
    F = oracle.Frame(24, 24)
    oracle.render(S, F)
    xs = ((np.arange(24) + 0.5) / 24 - 0.5) * 6.0
    X, Y = np.meshgrid(xs, xs)
    dx, dy = X - centre[0], Y - centre[1]
    q = r * r - dx * dx - dy * dy
    inside, outside = q > 1e-3, q < -1e-3
    n = np.stack([dx, dy, np.sqrt(np.maximum(q, 0.0))], axis=-1) / r
    L = -np.array([0.0, -0.6, -0.8])
    L /= np.linalg.norm(L)
    c = np.array([0.6, 0.5, 0.4])
    expect = c / math.pi * 2.0 * np.maximum(0.0, n @ L)[..., None] + c * 0.2
    assert inside.sum() > 100 and outside.sum() > 50
    assert np.allclose(F.color[inside][:, :3], expect[inside], atol=2e-5)
    assert np.all(F.color[outside][:, :3] == 0.0)
    assert np.allclose(F.depth[inside], 10.0 - np.sqrt(q[inside]), rtol=1e-4)
    assert np.allclose(F.normal[inside], n[inside], atol=1e-4)


def _lit(n, c=np.array([0.6, 0.5, 0.4])):
    """Matte shading of plane_scene's light: c/pi E max(0, n.L) + c ambient."""
    L = -np.array([0.0, -0.6, -0.8])
    L /= np.linalg.norm(L)
    return c / math.pi * 2.0 * np.maximum(0.0, n @ L)[..., None] + c * 0.2


def _top_view(oracle, surface, size=32, height=6.0):
    sc = plane_scene()
    sc["surfaces"] = [dict(surface, material={"type": "matte", "color": [0.6, 0.5, 0.4]})]
    sc["camera"] = {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                    "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": height,
                    "aspect": 1.0}
    S = oracle.Scene(sc)
    F = oracle.Frame(size, size)
    oracle.render(S, F)
    xs = ((np.arange(size) + 0.5) / size - 0.5) * height
    X, Y = np.meshgrid(xs, xs)
    return F, X, Y


def test_cylinder_closed_form(oracle):
    """A cylinder along x (radius 1, from x = -2 to 2, placed through
    primitive.index) seen from above: the body's top half, normal
    (0, y, sqrt(1 - y^2)), shaded as a matte surface; nothing past the ends."""
    F, X, Y = _top_view(oracle, {"geometry": "cylinder",
                                 "vertices": np.array([[5, 5, 5], [-2, 0, 0], [2, 0, 0]],
                                                      np.float32),
                                 "indices": np.array([[1, 2]], np.uint32), "radius": 1.0})
    body = (np.abs(X) < 1.9) & (np.abs(Y) < 0.95)
    miss = (np.abs(X) > 2.1) | (np.abs(Y) > 1.05)
    z = np.sqrt(np.maximum(0.0, 1.0 - Y * Y))
    n = np.stack([np.zeros_like(Y), Y, z], axis=-1)
    assert body.sum() > 100 and miss.sum() > 100
    assert np.allclose(F.color[body][:, :3], _lit(n)[body], atol=2e-5)
    assert np.allclose(F.depth[body], 10.0 - z[body], rtol=1e-4)
    assert np.all(F.color[miss][:, :3] == 0.0)


def test_cone_closed_form(oracle):
    """A cone frustum along z (radius 2 at z = 0 to radius 1 at z = 3) seen
    from above: the top cap (normal +z) inside radius 1, the body between
    radius 1 and 2 at height 3 (2 - rho) with normal along (x/rho, y/rho, 1/3)."""
    F, X, Y = _top_view(oracle, {"geometry": "cone",
                                 "vertices": np.array([[0, 0, 0], [0, 0, 3]], np.float32),
                                 "radii": np.array([2.0, 1.0], np.float32)})
    rho = np.sqrt(X * X + Y * Y)
    cap, body, miss = rho < 0.95, (rho > 1.05) & (rho < 1.95), rho > 2.05
    nb = np.stack([X / rho, Y / rho, np.full_like(rho, 1.0 / 3.0)], axis=-1)
    nb /= np.linalg.norm(nb, axis=-1, keepdims=True)
    assert cap.sum() > 20 and body.sum() > 100 and miss.sum() > 50
    assert np.allclose(F.color[cap][:, :3], _lit(np.array([0.0, 0.0, 1.0]))[None, :], atol=2e-5)
    assert np.allclose(F.depth[cap], 7.0, rtol=1e-5)
    assert np.allclose(F.color[body][:, :3], _lit(nb)[body], atol=5e-5)
    assert np.allclose(F.depth[body], 10.0 - 3.0 * (2.0 - rho[body]), rtol=1e-4)
    assert np.all(F.color[miss][:, :3] == 0.0)


def test_quad_closed_form(oracle):
    """Two quads seen from above: a flat one at z = 0 and a tilted one
    (z = 0.5 x) beside it. Quad k is shaded with the normal of triangle k of
    the geometry's tessellated list (Quad.cpp tessellation, getNormals
    taking the geometry's primitive at the quad's index), so the tilted quad
    (k = 1) takes triangle 1, the second triangle of the flat quad: it is
    shaded as if flat, with depth from its own tilted plane."""
    v = np.array([[-3, -2, 0], [-1, -2, 0], [-1, 2, 0], [-3, 2, 0],
                  [1, -2, 0.5], [3, -2, 1.5], [3, 2, 1.5], [1, 2, 0.5]], np.float32)
    F, X, Y = _top_view(oracle, {"geometry": "quad", "vertices": v,
                                 "indices": np.array([[0, 1, 2, 3], [4, 5, 6, 7]], np.uint32)},
                        size=32, height=8.0)
    flat = (X > -2.9) & (X < -1.1) & (np.abs(Y) < 1.9)
    tilt = (X > 1.1) & (X < 2.9) & (np.abs(Y) < 1.9)
    up = _lit(np.array([0.0, 0.0, 1.0]))
    assert flat.sum() > 20 and tilt.sum() > 20
    assert np.allclose(F.color[flat][:, :3], up[None, :], atol=2e-5)
    assert np.allclose(F.color[tilt][:, :3], up[None, :], atol=2e-5)
    assert np.allclose(F.depth[tilt], 10.0 - 0.5 * X[tilt], rtol=1e-5)


def _entry_t(o, d, kind, q):
    """Float64 entry distance of the ray o + t d (t >= 0, o outside) into a
    sphere, or into the solid capped cone / cylinder (v1, r1, v2, r2): the
    nearest of the body's roots inside the slab and the cap discs; inf on a
    miss. Written from the geometry, independently of the intersectors."""
    p1, r1, p2, r2 = q[:3], q[3], q[4:7], q[7]
    if kind == "sphere":
        oc = o - p1
        b, c = oc @ d, oc @ oc - r1 * r1
        disc = b * b - c
        if disc < 0:
            return np.inf
        t = -b - np.sqrt(disc)
        return t if t >= 0 else np.inf
    axis = p2 - p1
    L = np.linalg.norm(axis)
    a = axis / L
    cands = []
    for centre, r in ((p1, r1), (p2, r2)):  # caps
        den = d @ a
        if abs(den) > 1e-12:
            t = ((centre - o) @ a) / den
            x = o + t * d - centre
            if t >= 0 and x @ x < r * r:
                cands.append(t)
    # body: |w - (w.a) a| = r1 + (r2 - r1) (w.a) / L with w = o + t d - p1
    k = (r2 - r1) / L
    w0 = o - p1
    da, wa = d @ a, w0 @ a
    dp, wp = d - da * a, w0 - wa * a
    A = dp @ dp - (k * da) ** 2
    B = 2 * (dp @ wp - k * da * (r1 + k * wa))
    C = wp @ wp - (r1 + k * wa) ** 2
    disc = B * B - 4 * A * C
    if abs(A) > 1e-12 and disc >= 0:
        for t in ((-B - np.sqrt(disc)) / (2 * A), (-B + np.sqrt(disc)) / (2 * A)):
            y = wa + t * da
            if t >= 0 and 0 < y < L and r1 + k * y >= 0:
                cands.append(t)
    return min(cands) if cands else np.inf


@pytest.mark.parametrize("kind", ["sphere", "cone", "cylinder"])
def test_analytic_intersectors_against_float64(oracle, kind):
    """The oracle's sphere, cone and cylinder tests (the reference's cone
    intersector, the capped-cylinder and sphere quadratics, with the origin
    moved next to cones and cylinders) against a float64 evaluation of the
    entry point, for rays from outside: the same hit or miss, and t within
    1e-4 relative, except for rays grazing a silhouette."""
    lib = oracle.load()
    rng = np.random.default_rng({"sphere": 1, "cone": 2, "cylinder": 3}[kind])
    n = 40
    a = rng.uniform(-8.0, 8.0, (n, 3)).astype(np.float32)
    b = (a + rng.uniform(-3.0, 3.0, (n, 3))).astype(np.float32)
    if kind == "sphere":
        surf = {"geometry": "sphere", "vertices": a, "radii": rng.uniform(0.3, 1.5, n).astype(np.float32)}
        q = np.zeros((n, 8))
        q[:, :3], q[:, 3] = a, surf["radii"]
    else:
        ends = np.stack([a, b], axis=1).reshape(-1, 3)
        radii = rng.uniform(0.2, 1.2, 2 * n).astype(np.float32)
        surf = {"geometry": kind, "vertices": ends}
        q = np.zeros((n, 8))
        q[:, :3], q[:, 4:7] = a, b
        if kind == "cone":
            surf["radii"] = radii
            q[:, 3], q[:, 7] = radii[0::2], radii[1::2]
        else:
            surf["radii"] = radii[:n]
            q[:, 3] = q[:, 7] = radii[:n]
    sc = plane_scene()
    sc["surfaces"] = [dict(surf, material={"type": "matte", "color": [0.5, 0.5, 0.5]})]
    S = oracle.Scene(sc)
    mismatch, checked = 0, 0
    for _ in range(400):
        o = rng.normal(size=3)
        o = o / np.linalg.norm(o) * 30.0
        target = q[rng.integers(n), :3] + rng.uniform(-1.5, 1.5, 3)
        d = target - o
        d /= np.linalg.norm(d)
        o32, d32 = o.astype(np.float32), d.astype(np.float32)
        of, df = (ctypes.c_float * 3)(*o32), (ctypes.c_float * 3)(*d32)
        tt = ctypes.c_float(0)
        ins, tri = ctypes.c_uint32(0), ctypes.c_uint32(0)
        uv = (ctypes.c_float * 2)()
        hit = lib.or_trace(S.handle, of, df, 0.0, 3.0e38, ctypes.byref(tt), ctypes.byref(ins),
                           ctypes.byref(tri), uv)
        ts = [_entry_t(o32.astype(np.float64), d32.astype(np.float64), kind, q[k]) for k in range(n)]
        t64 = min(ts)
        checked += 1
        if hit != np.isfinite(t64) or (hit and abs(tt.value - t64) > 1e-4 * t64):
            mismatch += 1
    print(kind, "mismatches", mismatch, "of", checked)
    assert checked == 400 and mismatch <= 2


def test_isosurface_plane_closed_form(oracle):
    """A field rising linearly along z (16^3 nodes over [0,15]^3) with iso
    value 0.5 seen from above: with texel centres at (i + 0.5) / N the level
    set is the mid plane z = 7.5 exactly, linear interpolation along the ray
    is exact there, and the normal is the gradient direction +z."""
    n = 16
    ramp = np.linspace(0.0, 1.0, n, dtype=np.float32)
    data = np.ascontiguousarray(np.broadcast_to(ramp[:, None, None], (n, n, n)))
    sc = plane_scene()
    sc["surfaces"] = [{"geometry": "isosurface", "data": data, "origin": [0.0, 0.0, 0.0],
                       "spacing": [1.0, 1.0, 1.0], "isovalues": [0.5],
                       "material": {"type": "matte", "color": [0.6, 0.5, 0.4]}}]
    sc["camera"] = {"type": "orthographic", "position": [7.5, 7.5, 40.0],
                    "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 12.0,
                    "aspect": 1.0}
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16)
    oracle.render(S, F)
    assert np.allclose(F.depth, 40.0 - 7.5, rtol=1e-5)
    assert np.allclose(F.normal, [0.0, 0.0, 1.0], atol=1e-5)
    assert np.allclose(F.color[..., :3], _lit(np.array([0.0, 0.0, 1.0]))[None, None, :], atol=2e-5)


def test_isosurface_sphere(oracle):
    """A distance field |p - c| (sampled at the texel centres of a 32^3 field
    over [0,31]^3) with two iso values 6 and 9: seen from above, the hits lie
    on the radius-9 sphere (the outer level set is met first) to trilinear
    accuracy, with radial normals; rays missing it hit nothing."""
    n, c = 32, np.array([15.5, 15.5, 15.5])
    w = (np.arange(n) + 0.5) / n * 31.0
    Z, Y, X = np.meshgrid(w, w, w, indexing="ij")
    data = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2).astype(np.float32)
    sc = plane_scene()
    sc["surfaces"] = [{"geometry": "isosurface", "data": data, "origin": [0.0, 0.0, 0.0],
                       "spacing": [1.0, 1.0, 1.0], "isovalues": [6.0, 9.0],
                       "material": {"type": "matte", "color": [0.6, 0.5, 0.4]}}]
    sc["camera"] = {"type": "orthographic", "position": [15.5, 15.5, 60.0],
                    "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 24.0,
                    "aspect": 1.0}
    S = oracle.Scene(sc)
    F = oracle.Frame(24, 24)
    oracle.render(S, F)
    xs = 15.5 + ((np.arange(24) + 0.5) / 24 - 0.5) * 24.0
    X2, Y2 = np.meshgrid(xs, xs)
    rho2 = (X2 - c[0]) ** 2 + (Y2 - c[1]) ** 2
    inside, outside = rho2 < 8.0 ** 2, rho2 > 9.6 ** 2
    P = np.stack([X2, Y2, 60.0 - F.depth], axis=-1)
    r = np.linalg.norm(P - c, axis=-1)
    assert inside.sum() > 100 and outside.sum() > 50
    assert np.all(np.abs(r[inside] - 9.0) < 0.05)
    radial = (P - c) / r[..., None]
    assert np.all(np.abs(F.normal[inside] - radial[inside]) < 0.02)
    assert np.all(F.depth[outside] > 1e30)


def test_instanced_lights_match_transformed_world_lights(oracle):
    """xfmLight (DeviceCopyableObjects.h:2398-2430): a point and a spot light
    inside an instance (rotation about z, scale 1.5, translation) light the
    scene as world-level lights at the transformed position and axis."""
    c, s_ = np.cos(0.7), np.sin(0.7)
    R = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]]) * 1.5
    t = np.array([0.5, -1.0, 0.25])
    xfm = list(R.T.reshape(-1)) + list(t)  # column-major 3x4
    lights = [{"type": "point", "position": [0.4, 0.2, 2.0], "intensity": 6.0},
              {"type": "spot", "position": [-0.3, 0.1, 2.5], "direction": [0.1, 0.0, -1.0],
               "openingAngle": 0.8, "falloffAngle": 0.2, "intensity": 9.0}]
    moved = []
    for L in lights:
        L2 = dict(L, position=list(R @ np.array(L["position"]) + t))
        if "direction" in L:
            L2["direction"] = list(R @ np.array(L["direction"]))
        moved.append(L2)
    images = []
    for world, inst in ((moved, []), ([], lights)):
        sc = plane_scene()
        sc["lights"] = world
        sc["instances"] = [{"transform": xfm, "lights": inst}] if inst else []
        S = oracle.Scene(sc)
        F = oracle.Frame(16, 16)
        oracle.render(S, F)
        images.append(F.color.copy())
    assert images[0][..., :3].max() > 0.2
    assert np.allclose(images[0], images[1], atol=1e-5)


def _quad_light(visible=False, intensity=3.0, color=(1.0, 0.9, 0.8)):
    """A unit square light 2 above the origin, facing the z = 0 plane."""
    return {"type": "quad", "position": [-0.5, -0.5, 2.0], "edge1": [1.0, 0.0, 0.0],
            "edge2": [0.0, 1.0, 0.0], "intensity": intensity, "color": list(color),
            "visible": visible}


def _ortho_down(height=0.01):
    return {"type": "orthographic", "position": [0.0, 0.0, 10.0], "direction": [0.0, 0.0, -1.0],
            "up": [0.0, 1.0, 0.0], "height": height, "aspect": 1.0}


def _lcg_zero_state_draws(n):
    """The first n draws of the reference's LCG<4> from state 0."""
    state, out = 0, []
    for _ in range(n):
        state = (1664525 * state + 1013904223) & 0xFFFFFFFF
        out.append(np.float32(state & 0xFFFFFF) / np.float32(1 << 24))
    return out


def test_quad_light_raycast_closed_form(oracle):
    """Raycast of the matte plane under an invisible quad light: the light is
    sampled once (zero-state stream: triangle pick r, then the point
    v1 + sqrt(u1)(1 - u2) a + sqrt(u1) u2 b of that triangle) and shades
    as c/pi * I * cos_s * A cos_l / d^2, plus the ambient term."""
    sc = plane_scene()
    sc["lights"] = [_quad_light()]
    sc["camera"] = _ortho_down(8.0)
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16)
    oracle.render(S, F)
    r, u1, u2 = (float(x) for x in _lcg_zero_state_draws(3))
    v1, e1, e2 = np.array([-0.5, -0.5, 2.0]), np.array([1.0, 0, 0]), np.array([0, 1.0, 0])
    a, b = (e1, e1 + e2) if 0.5 < r else (e1 + e2, e2)
    y = v1 + math.sqrt(u1) * (1 - u2) * a + math.sqrt(u1) * u2 * b
    xs = ((np.arange(16) + 0.5) / 16 - 0.5) * 8.0
    X, Y = np.meshgrid(xs, xs)
    L = y[None, None, :] - np.stack([X, Y, np.zeros_like(X)], axis=-1)
    d2 = (L * L).sum(-1)
    cos_s = np.maximum(0.0, L[..., 2] / np.sqrt(d2))
    cos_l = np.abs(L[..., 2]) / np.sqrt(d2)
    c = np.array([0.6, 0.5, 0.4])
    I = 3.0 * np.array([1.0, 0.9, 0.8])
    expect = (c / math.pi) * I * (cos_s * cos_l / d2)[..., None] + c * 0.2
    assert np.allclose(F.color[..., :3], expect, rtol=2e-4, atol=1e-5)


@pytest.mark.parametrize("renderer", ["raycast", "pathtrace"])
def test_quad_light_seen_by_the_camera(oracle, renderer):
    """A visible quad light in front of the camera shows its intensity with
    alpha 1 in both renderers; an invisible one is skipped by camera rays
    (the background shows)."""
    sc = plane_scene(renderer=renderer)
    sc["camera"] = {"type": "orthographic", "position": [0.0, 0.0, 1.0],
                    "direction": [0.0, 0.0, 1.0], "up": [0.0, 1.0, 0.0], "height": 0.5,
                    "aspect": 1.0}
    sc["renderer"]["background"] = [0.1, 0.2, 0.3, 0.5]
    for visible in (True, False):
        sc["lights"] = [_quad_light(visible=visible)]
        S = oracle.Scene(sc)
        F = oracle.Frame(8, 8)
        oracle.render(S, F)
        expect = [3.0, 2.7, 2.4, 1.0] if visible else [0.1, 0.2, 0.3, 0.5]
        assert np.allclose(F.color, np.array(expect, np.float32), atol=1e-6), visible


def test_quad_light_pathtrace_mis_closed_form(oracle):
    """Path-traced matte plane under an invisible quad light: next-event
    estimation weighted by power_heuristic(pdf_light / n, pdf_bsdf) plus
    emission of BSDF-sampled rays that hit the light weighted by
    power_heuristic(pdf_bsdf, pdf_solid_angle / n) (Pathtrace_impl.cpp:
    139-182, :365-375). The weights do not sum to 1, as the reference
    writes them: the light sample's weight takes the pdf of the BSDF sample
    drawn at the same hit (cos_r / pi of a cosine-distributed direction,
    whose expectation over cos_r^2 ~ U(0,1) is a^2 ln(1 + 1/a^2) with
    a = pi pdf_light), not of the light direction, and its pdf is
    1 / (A cos_l) against the hit's d^2 / (A cos_l). The expectation is
    c/pi * I * int cos_s cos_l / d^2 (w_nee + w_bsdf) dA, integrated here
    by the midpoint rule."""
    sc = plane_scene(renderer="pathtrace")
    sc["lights"] = [_quad_light()]
    sc["camera"] = _ortho_down()
    sc["renderer"].update(pixelSamples=16, maxBounce=3, ambientRadiance=0.0, ambientSamples=0)
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16, stats=True)
    frames = 4
    for _ in range(frames):
        oracle.render(S, F)
    n = 16 * 16 * 16 * frames
    mean = F.sum.reshape(-1, 3).sum(0) / n
    var = F.sumsq.reshape(-1, 3).sum(0) / n - mean * mean
    k = 400
    g = (np.arange(k) + 0.5) / k - 0.5
    U, V = np.meshgrid(g, g)
    d = np.sqrt(U * U + V * V + 4.0)
    cos_s = cos_l = 2.0 / d
    geo = cos_s * cos_l / (d * d)
    p_nee, p_bsdf, p_hit = 1.0 / cos_l, cos_s / math.pi, d * d / cos_l
    a2 = (math.pi * p_nee) ** 2
    w_nee = a2 * np.log1p(1.0 / a2)
    w_bsdf = p_bsdf ** 2 / (p_bsdf ** 2 + p_hit ** 2)
    c = np.array([0.6, 0.5, 0.4])
    I = 3.0 * np.array([1.0, 0.9, 0.8])
    expect = c / math.pi * I * float((geo * (w_nee + w_bsdf)).mean())
    unweighted = c / math.pi * I * float(geo.mean())
    assert np.all(np.abs(mean - expect) <= 5 * np.sqrt(var / n) + 1e-4 * expect), (mean, expect)
    assert np.all(np.abs(mean - unweighted) > 10 * np.sqrt(var / n))  # the quirk is visible


def _hdri(radiance, scale=1.0, visible=False):
    """An HDRI light whose image frame puts its v axis (the polar angle)
    on world z: up (0, 0, -1) and direction (1, 0, 0) give
    toWorld = [(0, 1, 0), (0, 0, 1), (1, 0, 0)] (columns)."""
    return {"type": "hdri", "radiance": np.asarray(radiance, np.float32), "scale": scale,
            "up": [0.0, 0.0, -1.0], "direction": [1.0, 0.0, 0.0], "visible": visible}


@pytest.mark.parametrize("renderer", ["raycast", "pathtrace"])
def test_hdri_seen_by_the_camera(oracle, renderer):
    """Camera rays that leave the scene show a visible HDRI light's radiance
    times its scale, alpha 1, in both renderers; an invisible one leaves the
    background."""
    sc = plane_scene(renderer=renderer)
    sc["camera"] = {"type": "orthographic", "position": [0.0, 0.0, 1.0],
                    "direction": [0.0, 0.0, 1.0], "up": [0.0, 1.0, 0.0], "height": 0.5,
                    "aspect": 1.0}
    sc["renderer"]["background"] = [0.1, 0.2, 0.3, 0.5]
    img = np.tile(np.array([0.5, 0.4, 0.3], np.float32), (8, 16, 1))
    for visible in (True, False):
        sc["lights"] = [_hdri(img, scale=2.0, visible=visible)]
        S = oracle.Scene(sc)
        F = oracle.Frame(8, 8)
        oracle.render(S, F)
        expect = [1.0, 0.8, 0.6, 1.0] if visible else [0.1, 0.2, 0.3, 0.5]
        assert np.allclose(F.color, np.array(expect, np.float32), atol=1e-6), visible


def test_hdri_pathtrace_closed_form(oracle):
    """Path-traced matte plane (normal +z) under an invisible HDRI whose
    only bright texels form row 2 of 8 (the polar band 45..67.5 degrees
    from the normal), an expectation the reference's sampling fixes:
    next-event estimation always picks row 2 (pdf_y 1) and a column
    (pdf_x 1/W), aims at the texel corner (polar angle 45 degrees) where
    the bilinear lookup reads half the band's radiance, with
    pdf = pdf_x pdf_y W H / (4 pi), weighted against the BSDF sample drawn
    at the same hit (expectation a^2 ln(1 + 1/a^2), a = pi pdf); BSDF
    samples that leave the plane read the bilinear band and are weighted
    against the hit density pdf_x pdf_y W H / (2 pi^2 sin theta), where
    the CDF lookup gives row 2 and column probability 1/W for every
    direction. The oracle's 16 384-sample mean lies within 5 sigma of
    E_nee + E_bsdf (the latter by quadrature over the polar angle)."""
    W, H, y0, V, s_ = 16, 8, 2, 4.0, 1.5
    img = np.zeros((H, W, 3), np.float32)
    img[y0] = V
    sc = plane_scene(renderer="pathtrace")
    sc["lights"] = [_hdri(img, scale=s_)]
    sc["camera"] = _ortho_down()
    sc["renderer"].update(pixelSamples=16, maxBounce=3, ambientRadiance=0.0, ambientSamples=0)
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16, stats=True)
    frames = 4
    for _ in range(frames):
        oracle.render(S, F)
    n = 16 * 16 * 16 * frames
    mean = F.sum.reshape(-1, 3).sum(0) / n
    var = F.sumsq.reshape(-1, 3).sum(0) / n - mean * mean
    rho = np.array([0.6, 0.5, 0.4])
    a2 = (math.pi * H / (4 * math.pi)) ** 2
    e_nee = 2 * rho * V * s_ * math.cos(math.pi * y0 / H) / H * a2 * math.log1p(1 / a2)
    k = 200000
    th = (np.arange(k) + 0.5) / k * (math.pi / 2)
    v = np.clip(th / math.pi, 0.001, 0.999)
    yy = v * H - 0.5
    f0 = np.floor(yy)
    fy = yy - f0
    band = np.where(f0 == y0, 1 - fy, np.where(f0 + 1 == y0, fy, 0.0))
    p_b = np.cos(th) / math.pi
    p_l = H / (2 * math.pi ** 2 * np.sin(th))
    w = p_b ** 2 / (p_b ** 2 + p_l ** 2)
    integral = float((band * w * np.cos(th) / math.pi * 2 * math.pi * np.sin(th)).sum() *
                     (math.pi / 2) / k)
    e_bsdf = rho * V * s_ * integral
    expect = e_nee + e_bsdf
    assert np.all(e_nee > 0.1 * expect) and np.all(e_bsdf > 0.1 * expect)  # both terms count
    assert np.all(np.abs(mean - expect) <= 5 * np.sqrt(var / n) + 1e-4 * expect), (mean, expect)


def _tri_scene(material, extra=None, light=(0.0, 0.0, -1.0), renderer="raycast"):
    """One large triangle in z = 0 seen from above by an orthographic
    camera, lit straight down (irradiance 2), ambient 0.2."""
    v = np.array([[-6.0, -6.0, 0.0], [6.0, -6.0, 0.0], [-6.0, 6.0, 0.0]], np.float32)
    surf = {"vertices": v, "indices": np.array([[0, 1, 2]], np.uint32), "material": material}
    surf.update(extra or {})
    return {
        "surfaces": [surf], "volumes": [],
        "lights": [{"direction": list(light), "irradiance": 2.0}],
        "camera": {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                   "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 8.0,
                   "aspect": 1.0},
        "renderer": {"type": renderer, "ambientRadiance": 0.2, "background": [0, 0, 0, 1]},
        "frame": {"size": (16, 16)},
    }


def _pixel_bary():
    """Pixel centres of the 16 x 16 view of _tri_scene and their
    barycentrics (u of vertex 1, v of vertex 2); mask: inside the triangle."""
    xs = ((np.arange(16) + 0.5) / 16 - 0.5) * 8.0
    X, Y = np.meshgrid(xs, xs)
    u = (X + 6.0) / 12.0
    v = (Y + 6.0) / 12.0
    return X, Y, u, v, (u + v) <= 1.0


def test_vertex_colors_closed_form(oracle):
    """A matte material whose color is the "color" attribute: the vertex
    colours interpolated with the hit's barycentrics,
    (1 - u - v) c0 + u c1 + v c2, shade as c/pi E + c ambient."""
    cols = np.array([[1.0, 0.0, 0.0, 1.0], [0.0, 1.0, 0.0, 1.0], [0.0, 0.0, 1.0, 1.0]], np.float32)
    sc = _tri_scene({"type": "matte", "color": "color"}, {"attributes": {"color": cols}})
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16)
    oracle.render(S, F)
    X, Y, u, v, inside = _pixel_bary()
    c = (1 - u - v)[..., None] * cols[0, :3] + u[..., None] * cols[1, :3] + v[..., None] * cols[2, :3]
    expect = c / math.pi * 2.0 + c * 0.2
    assert inside.sum() > 100
    assert np.allclose(F.color[inside][:, :3], expect[inside], atol=1e-5)
    assert np.allclose(F.albedo[inside], c[inside], atol=1e-6)


def test_vertex_normals_shade(oracle):
    """Vertex normals tilted towards +x at every corner: the shading normal
    is the interpolated, normalised vertex normal, so the light straight
    down gives cos = n.z / |n| while the geometric normal stays (0, 0, 1)."""
    n = np.array([[0.6, 0.0, 0.8]] * 3, np.float32)
    sc = _tri_scene({"type": "matte", "color": [0.5, 0.5, 0.5]}, {"normals": n})
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16)
    oracle.render(S, F)
    X, Y, u, v, inside = _pixel_bary()
    expect = 0.5 / math.pi * 2.0 * 0.8 + 0.5 * 0.2
    assert np.allclose(F.color[inside][:, :3], expect, atol=1e-5)
    assert np.allclose(F.normal[inside], [0.0, 0.0, 1.0], atol=1e-6)


@pytest.mark.parametrize("filt,wrap", [("nearest", "clampToEdge"), ("linear", "clampToEdge"),
                                       ("nearest", "repeat"), ("nearest", "mirrorRepeat")])
def test_image2d_sampler(oracle, filt, wrap):
    """An image2D sampler on attribute0 (per-vertex texture coordinates
    (0,0), (2,0), (0,2)), through inTransform (scale 0.5 in u: so the
    coordinates reach 1 in u and 2 in v) and outOffset: texels as RGBA8
    (float texels x 255, truncated), nearest or bilinear with texel centres
    at (i + 0.5) / n, the address mode on texel indices."""
    img = np.array([[[0.1, 0.2, 0.3], [0.9, 0.8, 0.7]],
                    [[0.5, 0.0, 1.0], [0.25, 0.75, 0.5]]], np.float32)  # [y][x]
    tc = np.array([[0.0, 0.0], [2.0, 0.0], [0.0, 2.0]], np.float32)
    inx = [0.5, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1]
    samp = {"type": "image2D", "image": img, "filter": filt, "wrapMode1": wrap, "wrapMode2": wrap,
            "inTransform": inx, "outOffset": [0.01, 0.0, 0.0, 0.0]}
    sc = _tri_scene({"type": "matte", "color": {"sampler": samp}}, {"attributes": {"attribute0": tc}})
    S = oracle.Scene(sc)
    F = oracle.Frame(16, 16)
    oracle.render(S, F)
    X, Y, u, v, inside = _pixel_bary()
    tu, tv = 0.5 * (2.0 * u), 2.0 * v
    q = (np.floor(255.0 * np.clip(img, 0, 1)) / 255.0).astype(np.float64)

    def wrapi(i, n):
        if wrap == "repeat":
            return np.mod(i, n)
        if wrap == "mirrorRepeat":
            m = np.mod(i, 2 * n)
            return np.where(m < n, m, 2 * n - 1 - m)
        return np.clip(i, 0, n - 1)

    if filt == "nearest":
        c = q[wrapi(np.floor(tv * 2).astype(int), 2), wrapi(np.floor(tu * 2).astype(int), 2)]
    else:
        x, y = tu * 2 - 0.5, tv * 2 - 0.5
        x0, y0 = np.floor(x), np.floor(y)
        fx, fy = (x - x0)[..., None], (y - y0)[..., None]
        i0, i1 = wrapi(x0.astype(int), 2), wrapi(x0.astype(int) + 1, 2)
        j0, j1 = wrapi(y0.astype(int), 2), wrapi(y0.astype(int) + 1, 2)
        r0 = q[j0, i0] + fx * (q[j0, i1] - q[j0, i0])
        r1 = q[j1, i0] + fx * (q[j1, i1] - q[j1, i0])
        c = r0 + fy * (r1 - r0)
    c = c + np.array([0.01, 0.0, 0.0])
    expect = c / math.pi * 2.0 + c * 0.2
    assert np.allclose(F.color[inside][:, :3], expect[inside], atol=2e-5)


def test_primitive_transform_and_instance_attributes(oracle):
    """Per-primitive colours (primitive.color), a transform sampler mapping
    attribute1 to the colour (outTransform halves it, outOffset adds 0.1),
    and an instance's uniform colour behind a geometry without colours."""
    X, Y, u, v, inside = _pixel_bary()
    # primitive colour of the only triangle
    sc = _tri_scene({"type": "matte", "color": "color"},
                    {"primitive": {"color": np.array([[0.2, 0.4, 0.6]], np.float32)}})
    F = oracle.Frame(16, 16)
    oracle.render(oracle.Scene(sc), F)
    c = np.array([0.2, 0.4, 0.6])
    assert np.allclose(F.color[inside][:, :3], c / math.pi * 2 + c * 0.2, atol=1e-5)
    # transform sampler on a per-vertex attribute1
    a1 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]], np.float32)
    xf = [0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1]
    samp = {"type": "transform", "inAttribute": "attribute1", "outTransform": xf,
            "outOffset": [0.1, 0.1, 0.1, 0.0]}
    sc = _tri_scene({"type": "matte", "color": {"sampler": samp}}, {"attributes": {"attribute1": a1}})
    F = oracle.Frame(16, 16)
    oracle.render(oracle.Scene(sc), F)
    c = 0.5 * np.stack([1 - u - v, u, v], -1) + 0.1
    assert np.allclose(F.color[inside][:, :3], (c / math.pi * 2 + c * 0.2)[inside], atol=1e-5)
    # instance uniform colour
    sc = _tri_scene({"type": "matte", "color": "color"})
    inst = {"transform": [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], "surfaces": sc.pop("surfaces"),
            "attributes": {"color": [0.7, 0.3, 0.1, 1.0]}}
    sc["surfaces"] = []
    sc["instances"] = [inst]
    F = oracle.Frame(16, 16)
    oracle.render(oracle.Scene(sc), F)
    c = np.array([0.7, 0.3, 0.1])
    assert np.allclose(F.color[inside][:, :3], c / math.pi * 2 + c * 0.2, atol=1e-5)


def test_opacity_from_attribute_blends(oracle):
    """alphaMode blend with the opacity from attribute0's x (0.25 at every
    vertex) and the colour's alpha (vertex colour alpha 0.8): the raycast
    composites 0.2 of the surface over the background."""
    a0 = np.full((3, 1), 0.25, np.float32)
    cols = np.tile(np.array([[0.5, 0.5, 0.5, 0.8]], np.float32), (3, 1))
    sc = _tri_scene({"type": "matte", "color": "color", "opacity": "attribute0",
                     "alphaMode": "blend"}, {"attributes": {"attribute0": a0, "color": cols}})
    sc["renderer"]["background"] = [0.0, 0.0, 1.0, 1.0]
    F = oracle.Frame(16, 16)
    oracle.render(oracle.Scene(sc), F)
    X, Y, u, v, inside = _pixel_bary()
    a = 0.25 * 0.8
    shaded = 0.5 / math.pi * 2 + 0.5 * 0.2
    expect = np.array([a * shaded, a * shaded, a * shaded + (1 - a) * 1.0])
    assert np.allclose(F.color[inside][:, :3], expect, atol=1e-5)


def _curve_scene(vertices, radius, light=(0.0, 0.0, -1.0)):
    return {
        "surfaces": [{"geometry": "bezierCurve", "vertices": np.asarray(vertices, np.float32),
                      "radius": radius, "material": {"type": "matte", "color": [0.6, 0.5, 0.4]}}],
        "volumes": [],
        "lights": [{"direction": list(light), "irradiance": 2.0}],
        "camera": {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                   "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 2.0,
                   "aspect": 1.0},
        "renderer": {"type": "raycast", "ambientRadiance": 0.2, "background": [0, 0, 0, 1]},
        "frame": {"size": (32, 32)},
    }


def test_straight_bezier_curve_closed_form(oracle):
    """A cubic with evenly spaced collinear control points along x (a tube
    of radius 0.5) seen from above: the Phantom intersector converges to the
    tube, depth 10 - sqrt(r^2 - y^2), normal (0, y, z) / r (the hit minus
    the curve point at the converged parameter), matte shading with the
    light straight down."""
    w = [[-2.0, 0.0, 0.0], [-2.0 / 3.0, 0.0, 0.0], [2.0 / 3.0, 0.0, 0.0], [2.0, 0.0, 0.0]]
    F = oracle.Frame(32, 32)
    oracle.render(oracle.Scene(_curve_scene(w, 0.5)), F)
    xs = ((np.arange(32) + 0.5) / 32 - 0.5) * 2.0
    X, Y = np.meshgrid(xs, xs)
    inner = (np.abs(Y) < 0.45) & (np.abs(X) < 0.9)
    outside = np.abs(Y) > 0.55
    z = np.sqrt(np.maximum(0.25 - Y * Y, 0.0))
    assert inner.sum() > 100
    assert np.all(F.depth[outside] > 1e30)
    assert np.allclose(F.depth[inner], (10.0 - z)[inner], atol=2e-4)
    n = np.stack([np.zeros_like(Y), Y, z], -1) / 0.5
    assert np.allclose(F.normal[inner], n[inner], atol=2e-3)
    c = np.array([0.6, 0.5, 0.4])
    expect = (c / math.pi * 2.0)[None, :] * (z[inner] / 0.5)[:, None] + c * 0.2
    assert np.allclose(F.color[inner][:, :3], expect, atol=2e-3)


def test_curved_bezier_hits_lie_on_the_tube(oracle):
    """A bent cubic (radius 0.15) seen from above: every hit point the oracle
    reports (from its depth) lies on the tube, i.e. at distance r from the
    curve (dense sampling of the cubic), and the hits cover the curve."""
    w = np.array([[-0.9, -0.6, 0.0], [-0.3, 0.9, 0.3], [0.3, -0.9, -0.3], [0.9, 0.6, 0.0]],
                 np.float32)
    r = 0.15
    F = oracle.Frame(32, 32)
    oracle.render(oracle.Scene(_curve_scene(w, r)), F)
    xs = ((np.arange(32) + 0.5) / 32 - 0.5) * 2.0
    X, Y = np.meshgrid(xs, xs)
    hit = F.depth < 1e30
    assert hit.sum() > 60
    P = np.stack([X[hit], Y[hit], 10.0 - F.depth[hit]], -1)
    t = np.linspace(0.0, 1.0, 20001)[:, None]
    ti = 1 - t
    curve = ti ** 3 * w[0] + 3 * ti ** 2 * t * w[1] + 3 * ti * t ** 2 * w[2] + t ** 3 * w[3]
    d = np.sqrt(((P[:, None, :] - curve[None, :, :]) ** 2).sum(-1)).min(axis=1)
    assert np.all(np.abs(d - r) < 2e-3), np.abs(d - r).max()
    # pixels whose ray passes within 0.6 r of the projection of the curve's
    # middle part (away from the open ends) are hit
    mid = curve[2000:18001, :2]
    d2 = np.sqrt(((np.stack([X, Y], -1)[..., None, :] - mid[None, None, :, :]) ** 2).sum(-1)).min(-1)
    d2all = np.sqrt(((np.stack([X, Y], -1)[..., None, :] - curve[None, None, :, :2]) ** 2).sum(-1))
    near_end = np.minimum(d2all[..., :2000].min(-1), d2all[..., 18001:].min(-1)) < r
    assert np.all(hit[(d2 < 0.6 * r) & ~near_end])


def test_emission_absorption_slab(oracle):
    """Constant field, TF alpha a: alpha after k steps is 1 - (1-a)^(k dt/ud)."""
    n = 16
    data = np.full((n, n, n), 0.5, np.float32)
    a = 0.02
    tf = np.array([[1, 1, 1, a]] * 4, np.float32)
    sc = {
        "surfaces": [], "lights": [],
        "volumes": [{"data": data, "origin": [0, 0, 0], "spacing": [1, 1, 1],
                     "color": tf[:, :3], "opacity": tf[:, 3], "valueRange": [0, 1],
                     "unitDistance": 1.0}],
        "camera": {"type": "orthographic", "position": [7.5, 7.5, 40.0],
                   "direction": [0, 0, -1], "up": [0, 1, 0], "height": 4.0, "aspect": 1.0},
        "renderer": {"type": "raycast", "volumeSamplingRate": 1.0, "background": [0, 0, 0, 1]},
        "frame": {"size": (4, 4)},
    }
    S = oracle.Scene(sc)
    F = oracle.Frame(4, 4)
    oracle.render(S, F)
    # path length through the box is 15 (z from 15 to 0): 16 samples at dt = 1
    k = 16
    alpha = 1.0 - (1.0 - a) ** k
    # colour = alpha * sum(T_i (1-Tr)) -> alpha*alpha; composited over black bg (alpha 1)
    assert np.allclose(F.color[..., 0], alpha * alpha, rtol=1e-4)
    assert np.allclose(F.color[..., 3], alpha + (1 - alpha), rtol=1e-6)


def ramp_volume_scene(gradient_shading, toward_camera):
    """A 16^3 field that rises linearly along z (toward or away from an
    orthographic camera looking down -z), one constant TF colour, a
    directional light."""
    n = 16
    ramp = np.linspace(0.0, 1.0, n, dtype=np.float32)
    if not toward_camera:
        ramp = ramp[::-1].copy()
    data = np.ascontiguousarray(np.broadcast_to(ramp[:, None, None], (n, n, n)))
    tf = np.array([[0.8, 0.6, 0.4, 0.05]] * 4, np.float32)
    return {
        "surfaces": [],
        "lights": [{"direction": [0.3, -0.4, -0.866], "color": [1.0, 1.0, 1.0],
                    "irradiance": 2.0}],
        "volumes": [{"data": data, "origin": [0, 0, 0], "spacing": [1, 1, 1],
                     "color": tf[:, :3], "opacity": tf[:, 3], "valueRange": [0, 1],
                     "unitDistance": 1.0}],
        "camera": {"type": "orthographic", "position": [7.5, 7.5, 40.0],
                   "direction": [0, 0, -1], "up": [0, 1, 0], "height": 10.0, "aspect": 1.0},
        "renderer": {"type": "raycast", "volumeSamplingRate": 1.0, "background": [0, 0, 0, 1],
                     "ambientColor": [1.0, 0.5, 0.25], "ambientRadiance": 0.3,
                     "gradientShading": gradient_shading},
        "frame": {"size": (8, 8)},
    }


@pytest.mark.parametrize("toward_camera", [True, False])
def test_gradient_shading_closed_form(oracle, toward_camera):
    """Raycast gradient shading (VolumeIntegration.h:420-460) of a linear
    ramp: the face-forwarded gradient is +z (toward the viewer) at every
    sample, so each sample's colour is scaled by the same
    E/pi * max(0, N.L) + ambientColor * ambientRadiance, and so is the
    composite (black background)."""
    frames = {}
    for g in (False, True):
        S = oracle.Scene(ramp_volume_scene(g, toward_camera))
        F = oracle.Frame(8, 8)
        oracle.render(S, F)
        frames[g] = F.color.copy()
    plain, shaded = frames[False], frames[True]
    L = -np.array([0.3, -0.4, -0.866])
    L /= np.linalg.norm(L)
    scale = 2.0 / math.pi * max(0.0, float(L[2])) + np.array([1.0, 0.5, 0.25]) * 0.3
    assert plain[..., :3].min() > 1e-3  # every pixel sees the volume
    assert np.allclose(shaded[..., :3], plain[..., :3] * scale, rtol=1e-4, atol=1e-7)
    assert np.array_equal(shaded[..., 3], plain[..., 3])  # opacity is not shaded


def test_bvh_closest_hit_matches_brute_force(oracle, pkg):
    lib = oracle.load()
    rng = np.random.default_rng(3)
    sc = pkg.scenes.config1(res=8, spp=1, num_spheres=12, nu=12, nv=6)
    S = oracle.Scene(sc)
    tris = []
    for s in sc["surfaces"]:
        tris.append(np.asarray(s["vertices"])[np.asarray(s["indices"])])
    T = np.concatenate(tris).astype(np.float64)
    v1, e1, e2 = T[:, 0], T[:, 1] - T[:, 0], T[:, 2] - T[:, 0]
    for _ in range(200):
        o = rng.uniform(-14, 14, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        s1 = np.cross(d, e2)
        div = np.einsum("ij,ij->i", s1, e1)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / div
            dd = o - v1
            b1 = np.einsum("ij,ij->i", dd, s1) * inv
            s2 = np.cross(dd, e1)
            b2 = (s2 @ d) * inv
            t = np.einsum("ij,ij->i", e2, s2) * inv
        ok = (div != 0) & (b1 >= 0) & (b1 <= 1) & (b2 >= 0) & (b1 + b2 <= 1) & (t >= 0)
        of = (ctypes.c_float * 3)(*o)
        df = (ctypes.c_float * 3)(*d)
        tt = ctypes.c_float(0)
        ins, tri = ctypes.c_uint32(0), ctypes.c_uint32(0)
        uv = (ctypes.c_float * 2)()
        hit = lib.or_trace(S.handle, of, df, 0.0, 3.0e38, ctypes.byref(tt), ctypes.byref(ins),
                           ctypes.byref(tri), uv)
        assert bool(hit) == bool(ok.any())
        if hit:
            assert tt.value == pytest.approx(t[ok].min(), rel=1e-4)


def test_dda_visits_a_connected_cell_path(oracle):
    lib = oracle.load()
    rng = np.random.default_rng(5)
    dims = (ctypes.c_int32 * 3)(8, 5, 7)
    lo, hi = oracle.farr(3, [0, 0, 0]), oracle.farr(3, [1, 1, 1])
    for _ in range(50):
        o = rng.uniform(0.05, 0.95, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        cells = (ctypes.c_int32 * 64)()
        t01 = (ctypes.c_float * 128)()
        n = lib.or_dda(oracle.farr(3, o), oracle.farr(3, d), 0.0, 10.0, dims, lo, hi, cells, t01, 64)
        assert 1 <= n <= 8 + 5 + 7
        ids = [cells[i] for i in range(n)]
        xyz = [(c % 8, (c // 8) % 5, c // 40) for c in ids]
        for a, b in zip(xyz, xyz[1:]):
            assert sum(abs(p - q) for p, q in zip(a, b)) >= 1
            assert max(abs(p - q) for p, q in zip(a, b)) == 1
        ts = [t01[i] for i in range(2 * n)]
        assert all(ts[2 * i] <= ts[2 * i + 1] + 1e-6 for i in range(n))
        start = (min(int(o[0] * 8), 7), min(int(o[1] * 5), 4), min(int(o[2] * 7), 6))
        assert xyz[0] == start


def test_brick_majorants_bound_samples(oracle):
    """Every trilinear sample inside a brick has TF alpha <= the brick's majorant."""
    lib = oracle.load()
    rng = np.random.default_rng(7)
    n = 20
    data = rng.uniform(0, 1, (n, n, n)).astype(np.float32)
    tfa = rng.uniform(0, 1, 32).astype(np.float32)
    color = np.ones((32, 3), np.float32)
    vol = {"data": data, "origin": [0, 0, 0], "spacing": [1, 1, 1], "color": color,
           "opacity": tfa, "valueRange": [0, 1], "unitDistance": 1.0, "majorantBrickSize": 8}
    sc = {"surfaces": [], "lights": [], "volumes": [vol],
          "camera": {"type": "perspective", "position": [0, 0, 0], "direction": [0, 0, 1],
                     "up": [0, 1, 0]}, "renderer": {"type": "pathtrace"}, "frame": {"size": (1, 1)}}
    S = oracle.Scene(sc, grid_method=oracle.GRID_BRICK)
    dims = (ctypes.c_int32 * 3)()
    out = np.zeros(64, np.float32)
    nc = lib.or_majorants(S.handle, 0, dims, oracle.fptr(out), 64)
    G = dims[0]
    assert nc == G ** 3 == 27
    V = S.vols[0]
    res = np.zeros(4, np.float32)
    for _ in range(3000):
        p = rng.uniform(0, 1, 3)
        k = np.minimum((p * G).astype(int), G - 1)
        v = lib.or_sample_field(ctypes.byref(V), *p)
        lib.or_tf_lookup(ctypes.byref(V), v, oracle.fptr(res))
        cell = (k[2] * G + k[1]) * G + k[0]
        assert res[3] <= out[cell] + 1e-6


def test_sample_material_invariants(oracle):
    lib = oracle.load()
    rng = np.random.default_rng(9)
    for mtype in ("matte", "physicallyBased"):
        for _ in range(200):
            m = {"type": mtype, "color": [0.5, 0.6, 0.7], "baseColor": [0.5, 0.6, 0.7],
                 "metallic": float(rng.uniform()), "roughness": float(rng.uniform())}
            om = oracle.material(m)
            n = np.array([0.0, 0.0, 1.0])
            v = rng.normal(size=3)
            v[2] = abs(v[2]) + 0.05
            v /= np.linalg.norm(v)
            d = np.zeros(3, np.float32)
            f = np.zeros(3, np.float32)
            pdf, cosT = ctypes.c_float(), ctypes.c_float()
            lib.or_sample_material(ctypes.byref(om), oracle.farr(3, n), oracle.farr(3, n),
                                   oracle.farr(3, v), int(rng.integers(1 << 30)), 7,
                                   oracle.fptr(d), oracle.fptr(f), ctypes.byref(pdf), ctypes.byref(cosT))
            if np.isnan(d).any():
                continue
            assert abs(np.linalg.norm(d) - 1.0) < 1e-4
            assert cosT.value == pytest.approx(max(0.0, d[2]), abs=1e-5)
            if d[2] > 1e-3:
                assert pdf.value > 0
            assert np.all(f >= 0)


def test_render_is_thread_count_independent(oracle, pkg):
    sc = pkg.scenes.config1(res=24, spp=2, num_spheres=6, nu=12, nv=6)
    S = oracle.Scene(sc)
    a, b = oracle.Frame(24, 24), oracle.Frame(24, 24)
    oracle.render(S, a, num_threads=1)
    oracle.render(S, b, num_threads=4)
    assert np.array_equal(a.color, b.color)
    assert np.array_equal(a.depth, b.depth)


def test_taa_resolve_closed_form(oracle, pkg):
    """TAA on pixels that see only the background (a camera looking away
    from the geometry): the frame colour is the background b, the motion
    vector 0 and the albedo 0 in every frame, so the resolve pass blends the
    history (the Catmull-Rom read of a constant image, weights summing to
    one) with weight alpha: after k frames from the zero history the colour
    is b (1 - (1 - alpha)^k). With a static camera the motion vectors are
    exactly zero."""
    sc = pkg.scenes.config1(res=24, spp=2, num_spheres=4, nu=8, nv=4)
    cam = dict(sc["camera"])
    cam["direction"] = [-v for v in cam["direction"]]  # away from the spheres
    cam["position"] = [0.0, 40.0, 60.0]
    sc["camera"] = cam
    bg = [0.2, 0.5, 0.8, 1.0]
    alpha = 0.3
    sc["renderer"].update(background=bg, taa=True, taaAlpha=alpha)
    S = oracle.Scene(sc)
    F = oracle.Frame(24, 24, taa=True)
    for k in range(1, 5):
        oracle.render(S, F)
        want = np.asarray(bg, np.float64) * (1.0 - (1.0 - alpha) ** k)
        assert np.abs(F.color - want).max() < 1e-5, k
        assert np.array_equal(F.taa_prev, F.taa_curr)  # the frame became the history
        assert not F.motion_vec.any()
    assert np.all(F.depth == np.float32(1e31))


def test_taa_motion_vectors_follow_the_camera(oracle, pkg):
    """A camera moved sideways between two frames: on pixels that see the
    ground plane, the motion vector points back to where the hit projected in
    the previous frame (its x component has the sign of the camera's move in
    screen space and no pixel moves more than the shift of the nearest
    point), and pixels that see nothing keep a zero vector."""
    sc = pkg.scenes.config1(res=48, spp=1, num_spheres=6, nu=8, nv=4)
    sc["renderer"].update(taa=True, maxBounce=0)
    S = oracle.Scene(sc)
    F = oracle.Frame(48, 48, taa=True)
    oracle.render(S, F)
    cam = dict(sc["camera"])
    right = np.cross(np.asarray(cam["direction"]), np.asarray(cam["up"]))
    right /= np.linalg.norm(right)
    cam["position"] = [float(p + 0.5 * r) for p, r in zip(cam["position"], right)]
    S2 = oracle.Scene(dict(sc, camera=cam))
    # a camera commit restarts accumulation and the depth buffer, not TAA
    oracle.load().or_frame_reset(ctypes.byref(F.f))
    oracle.render(S2, F)
    hit = F.depth < 1e30
    mv = F.motion_vec
    assert hit.mean() > 0.2
    # the camera moved right: points move left on screen, so the previous
    # window position is to the right of the current one
    assert float((mv[hit][:, 0] > 0).mean()) > 0.999
    assert not mv[~hit].any()
