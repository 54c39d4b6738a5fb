"""Seeded synthetic scenes of the benchmark configurations, and their
construction through the renderer core's object API.

No public dataset is involved: each configuration is generated from a
numpy PCG64 stream seeded with 0x5EED0000 + config index; the draw order
is fixed in each generator. A scene is a plain dict:

  surfaces : [{"vertices": (V,3) f32, "indices": (T,3) u32, "material": {...}} |
              {"geometry": "sphere", "vertices": (V,3) f32 centres, "indices": (N,) u32
               (optional), "radii": (N,) f32 (optional), "radius": f32 (default 0.01),
               "material": {...}} |
              {"geometry": "isosurface", "data": (nz,ny,nx) f32, "origin", "spacing",
               "isovalues": [...], "material": {...}} |
              {"geometry": "quad", "vertices": (V,3) f32, "indices": (Q,4) u32 (optional,
               else consecutive quadruples), "material": {...}} |
              {"geometry": "bezierCurve", "vertices": (V,3) f32 control points,
               "indices": (N,) u32 segment starts (optional), "radii" per index entry
               (optional), "radius" (default 1), "material": {...}} |
              {"geometry": "cone" | "cylinder", "vertices": (V,3) f32 end points,
               "indices": (N,2) u32 (optional, else consecutive pairs), "radii": per
               vertex (cone, required) or per cylinder (optional), "radius": f32
               (cylinder, default 1), "material": {...}}]
  volumes  : [{"data": (nz,ny,nx) f32, "origin", "spacing", "color": (N,3),
               "opacity": (N,), "valueRange", "unitDistance"}]
  lights   : [{"type": "directional" (default), "direction", "color", "irradiance",
                "angularDiameter"} | {"type": "point", "position", "color", "intensity"} |
              {"type": "spot", "position", "direction", "openingAngle", "falloffAngle",
               "color", "intensity"} | {"type": "quad", "position", "edge1", "edge2",
               "color", "intensity", "side"} | {"type": "hdri", "radiance": (H, W, 3) f32,
               "up", "direction", "scale"}; any light may carry "visible" (bool)]
  instances: [{"transform": 12 floats (column-major 3x4), "surfaces": [...],
               "volumes": [...], "lights": [...]}]   (optional)
  camera   : {"type": "perspective", "position", "direction", "up", "fovy", "aspect"}
  renderer : {"type": "raycast"|"pathtrace", parameters...}
  frame    : {"size": (W, H)}

World-level surfaces/volumes/lights go into one group with an identity
instance, which comes before the explicit instances.
"""
import math

import numpy as np

from . import vsr

SEED_BASE = 0x5EED0000


def _look_at_camera(target, eye, fovy_deg, aspect):
    d = np.asarray(target, np.float64) - np.asarray(eye, np.float64)
    d /= np.linalg.norm(d)
    return {"type": "perspective", "position": [float(x) for x in eye],
            "direction": [float(x) for x in d], "up": [0.0, 1.0, 0.0],
            "fovy": math.radians(fovy_deg), "aspect": float(aspect)}


def blob_field(n, rng, num_blobs=16):
    """Sum of isotropic Gaussian blobs at voxel centres (i+0.5)/n, normalised to [0,1]."""
    centres = rng.uniform(0.0, 1.0, size=(num_blobs, 3))
    sigma = rng.uniform(0.05, 0.15, size=num_blobs)
    amp = rng.uniform(0.2, 1.0, size=num_blobs)
    p = (np.arange(n, dtype=np.float64) + 0.5) / n
    field = np.zeros((n, n, n), np.float64)
    for c, s, a in zip(centres, sigma, amp):
        gx = np.exp(-((p - c[0]) ** 2) / (2 * s * s))
        gy = np.exp(-((p - c[1]) ** 2) / (2 * s * s))
        gz = np.exp(-((p - c[2]) ** 2) / (2 * s * s))
        field += a * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    lo, hi = field.min(), field.max()
    return ((field - lo) / (hi - lo)).astype(np.float32)


def linear_tf(n=256, alpha_max=0.05):
    """Colour blue->red, opacity 0->alpha_max, n entries."""
    t = np.linspace(0.0, 1.0, n, dtype=np.float32)
    color = np.stack([t, np.zeros_like(t), 1.0 - t], axis=1).astype(np.float32)
    opacity = (t * alpha_max).astype(np.float32)
    return color, opacity


def config0(res=512, n=128, seed=SEED_BASE + 0):
    """Raycast renderer over a structured-regular Gaussian-blob volume."""
    rng = np.random.default_rng(seed)
    data = blob_field(n, rng)
    color, opacity = linear_tf(256, 0.05)
    extent = float(n - 1)
    centre = [extent / 2] * 3
    diag = math.sqrt(3.0) * extent
    view = np.array([0.6, 0.45, 0.66])
    view /= np.linalg.norm(view)
    eye = np.array(centre) + 2.5 * diag * view
    return {
        "surfaces": [], "lights": [],
        "volumes": [{"data": data, "origin": [0.0, 0.0, 0.0], "spacing": [1.0, 1.0, 1.0],
                     "color": color, "opacity": opacity, "valueRange": [0.0, 1.0],
                     "unitDistance": 1.0}],
        "camera": _look_at_camera(centre, eye, 40.0, 1.0),
        "renderer": {"type": "raycast", "volumeSamplingRate": 2.0, "background": [0, 0, 0, 1]},
        "frame": {"size": (res, res)},
    }


def uv_sphere(centre, radius, nu=64, nv=32):
    """UV sphere without degenerate pole triangles: nu*(2*nv-2) triangles,
    counter-clockwise seen from outside."""
    th = np.pi * np.arange(nv + 1) / nv
    ph = 2 * np.pi * np.arange(nu + 1) / nu
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    sp, cp = np.sin(ph)[None, :], np.cos(ph)[None, :]
    v = np.stack([st * cp, np.broadcast_to(ct, (nv + 1, nu + 1)), st * sp], axis=-1)
    v = (v * radius + np.asarray(centre)).reshape(-1, 3).astype(np.float32)
    j, i = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    a = j * (nu + 1) + i
    b = (j + 1) * (nu + 1) + i
    c = (j + 1) * (nu + 1) + i + 1
    d = j * (nu + 1) + i + 1
    # row r contributes (a,d,b) unless it touches the top pole (r == 0) and
    # (b,d,c) unless it touches the bottom pole (r == nv-1)
    rows = []
    for r in range(nv):
        q = []
        if r > 0:
            q.append(np.stack([a[r], d[r], b[r]], -1))
        if r < nv - 1:
            q.append(np.stack([b[r], d[r], c[r]], -1))
        rows.append(np.concatenate(q))
    return v, np.concatenate(rows).astype(np.uint32)


def sphere_set(rng, num_spheres=256, nu=64, nv=32):
    """The config-1 sphere set: surfaces list (ground quad last)."""
    centres = rng.uniform(-10.0, 10.0, size=(num_spheres, 3))
    radii = rng.uniform(0.3, 1.5, size=num_spheres)
    coin = rng.uniform(0.0, 1.0, size=num_spheres)
    colors = rng.uniform(0.1, 0.9, size=(num_spheres, 3))
    metallic = rng.uniform(0.0, 1.0, size=num_spheres)
    roughness = rng.uniform(0.0, 1.0, size=num_spheres)
    surfaces = []
    for k in range(num_spheres):
        v, t = uv_sphere(centres[k], radii[k], nu, nv)
        if coin[k] < 0.5:
            mat = {"type": "matte", "color": [float(x) for x in colors[k]]}
        else:
            mat = {"type": "physicallyBased", "baseColor": [float(x) for x in colors[k]],
                   "metallic": float(metallic[k]), "roughness": float(roughness[k])}
        surfaces.append({"vertices": v, "indices": t, "material": mat})
    g = 20.0
    quad = np.array([[-g, -11.5, -g], [g, -11.5, -g], [g, -11.5, g], [-g, -11.5, g]], np.float32)
    surfaces.append({"vertices": quad, "indices": np.array([[0, 2, 1], [0, 3, 2]], np.uint32),
                     "material": {"type": "matte", "color": [0.8, 0.8, 0.8]}})
    return surfaces


def config1(res=1024, spp=64, num_spheres=256, nu=64, nv=32, max_bounce=5,
            seed=SEED_BASE + 1):
    """Path tracer over ~1M triangles: 256 UV spheres + a 40x40 ground quad."""
    rng = np.random.default_rng(seed)
    surfaces = sphere_set(rng, num_spheres, nu, nv)
    light_dir = np.array([-0.35, -1.0, -0.45])
    light_dir /= np.linalg.norm(light_dir)
    return {
        "surfaces": surfaces, "volumes": [],
        "lights": [{"direction": [float(x) for x in light_dir], "color": [1.0, 1.0, 1.0],
                    "irradiance": 3.0}],
        "camera": _look_at_camera([0.0, -1.0, 0.0], [6.0, 9.0, 34.0], 45.0, 1.0),
        "renderer": {"type": "pathtrace", "pixelSamples": spp, "maxBounce": max_bounce,
                     "ambientRadiance": 0.2, "background": [0, 0, 0, 1]},
        "frame": {"size": (res, res)},
    }


def value_noise(n, rng, octaves=6, base_freq=4, persistence=0.5):
    """Multi-octave value noise at voxel centres, clamped to [0,1].

    Octave o has a (f+1)^3 lattice (f = base_freq * 2^o) of uniform values,
    smoothstep-weighted trilinear interpolation, amplitude persistence^o:
    field = clamp(0.5 + sum_o persistence^o * (noise_o - 0.5), 0, 1).
    Interpolation is separable, so each octave is three small matrix products.
    """
    p = (np.arange(n, dtype=np.float64) + 0.5) / n
    field = np.full((n, n, n), 0.5, np.float32)
    for o in range(octaves):
        f = base_freq * (2 ** o)
        lat = rng.uniform(0.0, 1.0, size=(f + 1, f + 1, f + 1))
        x = p * f
        i0 = np.minimum(np.floor(x).astype(int), f - 1)
        t = x - i0
        t = t * t * (3 - 2 * t)
        M = np.zeros((n, f + 1))
        M[np.arange(n), i0] = 1 - t
        M[np.arange(n), i0 + 1] += t
        # lat indexed [z, y, x]; interpolate x, then y, then z (BLAS matmuls)
        a = lat @ M.T                                   # (z, y, n)
        a = np.einsum("jy,zyi->zji", M, a)              # (z, n, n)
        a = (M @ a.reshape(f + 1, n * n)).reshape(n, n, n).astype(np.float32)
        field += np.float32(persistence ** o) * (a - np.float32(0.5))
    return np.clip(field, 0.0, 1.0).astype(np.float32)


def smoke_tf(n=256, start=0.5, alpha_max=0.5):
    """Smoke-like TF: zero opacity below `start`, then linear to alpha_max."""
    t = np.linspace(0.0, 1.0, n, dtype=np.float32)
    color = np.stack([0.9 + 0.1 * t, 0.85 - 0.25 * t, 0.8 - 0.5 * t], axis=1).astype(np.float32)
    opacity = (np.clip((t - start) / (1.0 - start), 0.0, 1.0) * alpha_max).astype(np.float32)
    return color, opacity


def config2(res=(1920, 1080), spp=256, n=512, num_spheres=256, nu=64, nv=32, max_bounce=8,
            seed=SEED_BASE + 2):
    """Volumetric path tracing: value-noise volume over [-12,12]^3 (density
    scale 50: unitDistance = 1/50 world units), delta tracking against 16^3
    voxel brick majorants, the config-1 sphere set, clip plane (0,0,1,0)."""
    rng = np.random.default_rng(seed)
    data = value_noise(n, rng)
    color, opacity = smoke_tf()
    surfaces = sphere_set(np.random.default_rng(SEED_BASE + 1), num_spheres, nu, nv)
    spacing = 24.0 / (n - 1)
    light_dir = np.array([-0.35, -1.0, -0.45])
    light_dir /= np.linalg.norm(light_dir)
    W, H = res
    return {
        "surfaces": surfaces,
        "volumes": [{"data": data, "origin": [-12.0, -12.0, -12.0], "spacing": [spacing] * 3,
                     "color": color, "opacity": opacity, "valueRange": [0.0, 1.0],
                     "unitDistance": 1.0 / 50.0, "majorantBrickSize": 16}],
        "lights": [{"direction": [float(x) for x in light_dir], "color": [1.0, 1.0, 1.0],
                    "irradiance": 3.0}],
        "camera": _look_at_camera([0.0, -1.0, 0.0], [6.0, 9.0, 34.0], 45.0, W / H),
        "renderer": {"type": "pathtrace", "pixelSamples": spp, "maxBounce": max_bounce,
                     "ambientRadiance": 0.2, "background": [0, 0, 0, 1],
                     "clipPlanes": [[0.0, 0.0, 1.0, 0.0]]},
        "frame": {"size": (W, H)},
    }


def blob_field_fast(n, rng, num_blobs=16):
    """blob_field's distribution (centres U[0,1]^3, sigma U[0.05,0.15],
    amplitude U[0.2,1]) evaluated separably as one matrix product: the
    Gaussian of blob b factors into gz_b(z) gy_b(y) gx_b(x), so the field is
    Gz (n x B) times the B x n^2 matrix of a_b gy_b(y) gx_b(x). Normalised to
    [0,1]."""
    centres = rng.uniform(0.0, 1.0, size=(num_blobs, 3))
    sigma = rng.uniform(0.05, 0.15, size=num_blobs)
    amp = rng.uniform(0.2, 1.0, size=num_blobs)
    p = (np.arange(n, dtype=np.float64) + 0.5) / n
    inv = 1.0 / (2.0 * sigma * sigma)
    gx = np.exp(-((p[None, :] - centres[:, 0:1]) ** 2) * inv[:, None])   # (B, n)
    gy = np.exp(-((p[None, :] - centres[:, 1:2]) ** 2) * inv[:, None])
    gz = np.exp(-((p[None, :] - centres[:, 2:3]) ** 2) * inv[:, None])
    yx = (amp[:, None, None] * gy[:, :, None] * gx[:, None, :]).reshape(num_blobs, n * n)
    field = (gz.T.astype(np.float32) @ yx.astype(np.float32)).reshape(n, n, n)
    lo, hi = float(field.min()), float(field.max())
    return ((field - lo) / (hi - lo)).astype(np.float32)


def config3(num_scenes=64, seed=SEED_BASE + 3, sizes=(256, 512, 768, 1024), side=(64, 384),
            tris=(10_000, 500_000), spp=(1, 64), max_bounce=5):
    """Batched rendering: independent scenes, each seeded with seed + index.

    Per scene, in draw order: volume side U{side}, raycast or pathtrace
    (coin), spheres or not (coin), triangle count U[tris] as UV spheres of
    64x32 segments (4032 triangles each) over [-10,10]^3, image size from
    `sizes`, spp U{spp} (pixelSamples of the path tracer; the raycast
    renderer takes one sample per pixel). The volume is a config-0 style blob field over
    [-12,12]^3 (unitDistance one voxel spacing, dt half a voxel, opacity
    0..0.05); light, ambient and camera as config 1."""
    scenes = []
    light_dir = np.array([-0.35, -1.0, -0.45])
    light_dir /= np.linalg.norm(light_dir)
    for i in range(num_scenes):
        rng = np.random.default_rng(seed + i)
        n = int(rng.integers(side[0], side[1] + 1))
        kind = "raycast" if rng.uniform() < 0.5 else "pathtrace"
        with_spheres = rng.uniform() < 0.5
        ntri = int(rng.integers(tris[0], tris[1] + 1))
        res = int(sizes[int(rng.integers(0, len(sizes)))])
        s = int(rng.integers(spp[0], spp[1] + 1))
        data = blob_field_fast(n, rng)
        color, opacity = linear_tf(256, 0.05)
        spacing = 24.0 / (n - 1)
        surfaces = []
        if with_spheres:
            surfaces = sphere_set(rng, max(1, round(ntri / 4032)))[:-1]  # no ground quad
        renderer = {"type": kind, "pixelSamples": s, "volumeSamplingRate": 2.0,
                    "ambientRadiance": 0.2, "background": [0, 0, 0, 1]}
        if kind == "pathtrace":
            renderer["maxBounce"] = max_bounce
        scenes.append({
            "surfaces": surfaces,
            "volumes": [{"data": data, "origin": [-12.0] * 3, "spacing": [spacing] * 3,
                         "color": color, "opacity": opacity, "valueRange": [0.0, 1.0],
                         "unitDistance": spacing, "majorantBrickSize": 16}],
            "lights": [{"direction": [float(x) for x in light_dir], "color": [1.0, 1.0, 1.0],
                        "irradiance": 3.0}],
            "camera": _look_at_camera([0.0, -1.0, 0.0], [6.0, 9.0, 34.0], 45.0, 1.0),
            "renderer": renderer,
            "frame": {"size": (res, res)},
        })
    return scenes


def triangle_count(scene):
    return sum(len(s["indices"]) for s in scene["surfaces"])


# --------------------------------------------------------------- build via ABI
def _sampler(dev, d, keep):
    """A sampler object from {"type": "image1D" | "image2D" | "image3D" |
    "transform" | "primitive", "image" / "array": numpy array, "inAttribute",
    "filter", "wrapMode1..3", "inTransform" / "outTransform" (16 floats,
    column-major), "inOffset" / "outOffset" (4 floats), "offset"}."""
    kind = d["type"]
    smp = dev.sampler(kind)
    for k, v in d.items():
        if k == "type":
            continue
        if k == "image":
            a = np.ascontiguousarray(v)
            arr = (dev.array1d if kind == "image1D" else
                   dev.array2d if kind == "image2D" else dev.array3d)(a)
            keep.append(arr)
            dev.set(smp, "image", arr)
        elif k == "array":
            arr = dev.array1d(np.ascontiguousarray(v))
            keep.append(arr)
            dev.set(smp, "array", arr)
        elif k in ("inTransform", "outTransform"):
            dev.set(smp, k, [float(x) for x in v], vsr.FLOAT32_MAT4)
        elif k in ("inOffset", "outOffset"):
            dev.set(smp, k, [float(x) for x in v], vsr.FLOAT32_VEC4)
        elif k == "offset":
            dev.set(smp, k, int(v))
        else:
            dev.set(smp, k, str(v))
    dev.commit(smp)
    keep.append(smp)
    return smp


def _material(dev, m, keep=None):
    mat = dev.material(m["type"])
    for k, v in m.items():
        if k == "type":
            continue
        if isinstance(v, dict):
            # {"sampler": {...}}: the parameter comes from a sampler
            dev.set(mat, k, _sampler(dev, v["sampler"], keep if keep is not None else []))
        elif isinstance(v, str):
            dev.set(mat, k, v)
        elif isinstance(v, (list, tuple)):
            dev.set(mat, k, v, vsr.FLOAT32_VEC3 if len(v) == 3 else vsr.FLOAT32_VEC4)
        else:
            dev.set(mat, k, float(v))
    dev.commit(mat)
    return mat


def _uniform(dev, obj, name, v):
    v = [float(x) for x in (v if isinstance(v, (list, tuple, np.ndarray)) else [v])]
    dev.set(obj, name, v if len(v) > 1 else v[0],
            {1: vsr.FLOAT32, 2: vsr.FLOAT32_VEC2, 3: vsr.FLOAT32_VEC3, 4: vsr.FLOAT32_VEC4}[len(v)])


def _geometry_attributes(dev, g, s, keep):
    """Surface keys "normals" (vertex.normal), "attributes" (vertex.*),
    "faceVarying" (faceVarying.*), "primitive" (primitive.*): {name: array}
    with name "color" or "attribute0".."attribute3"; "uniform": {name:
    value}."""
    if "normals" in s:
        na = dev.array1d(np.asarray(s["normals"], np.float32).reshape(-1, 3))
        dev.set(g, "vertex.normal", na)
        keep.append(na)
    for key, prefix in (("attributes", "vertex."), ("faceVarying", "faceVarying."),
                        ("primitive", "primitive.")):
        for name, arr in s.get(key, {}).items():
            a = dev.array1d(np.ascontiguousarray(arr))
            dev.set(g, prefix + name, a)
            keep.append(a)
    for name, v in s.get("uniform", {}).items():
        _uniform(dev, g, name, v)


def _surfaces(dev, surfs, keep):
    out = []
    for s in surfs:
        kind = s.get("geometry", "triangle")
        g = dev.geometry(kind)
        if kind == "isosurface":
            f = dev.spatial_field("structuredRegular")
            da = dev.array3d(np.asarray(s["data"], np.float32))
            dev.set(f, "data", da)
            dev.set(f, "origin", s.get("origin", [0.0, 0.0, 0.0]), vsr.FLOAT32_VEC3)
            dev.set(f, "spacing", s.get("spacing", [1.0, 1.0, 1.0]), vsr.FLOAT32_VEC3)
            dev.commit(f)
            iv = dev.array1d(np.asarray(s["isovalues"], np.float32).reshape(-1))
            dev.set(g, "field", f)
            dev.set(g, "isovalue", iv)
            dev.commit(g)
            keep += [f, da, iv]
            mat = _material(dev, s["material"])
            sf = dev.surface()
            dev.set(sf, "geometry", g)
            dev.set(sf, "material", mat)
            dev.commit(sf)
            keep += [g, mat]
            out.append(sf)
            continue
        va = dev.array1d(np.asarray(s["vertices"], np.float32))
        dev.set(g, "vertex.position", va)
        keep += [va]
        ia = None
        if kind in ("sphere", "cone", "cylinder"):
            if "indices" in s:
                ia = np.asarray(s["indices"], np.uint32)
                ia = dev.array1d(ia.reshape(-1) if kind == "sphere" else ia.reshape(-1, 2))
            if "radii" in s:
                ra = dev.array1d(np.asarray(s["radii"], np.float32).reshape(-1))
                dev.set(g, "primitive.radius" if kind == "cylinder" else "vertex.radius", ra)
                keep += [ra]
            if "radius" in s:
                dev.set(g, "radius", float(s["radius"]))
        elif kind == "bezierCurve":
            if "indices" in s:
                ia = dev.array1d(np.asarray(s["indices"], np.uint32).reshape(-1))
            if "radii" in s:
                ra = dev.array1d(np.asarray(s["radii"], np.float32).reshape(-1))
                dev.set(g, "primitive.radius", ra)
                keep += [ra]
            if "radius" in s:
                dev.set(g, "radius", float(s["radius"]))
        elif kind == "quad":
            if "indices" in s:
                ia = dev.array1d(np.asarray(s["indices"], np.uint32).reshape(-1, 4))
        else:
            ia = dev.array1d(np.asarray(s["indices"], np.uint32))
        if ia is not None:
            dev.set(g, "primitive.index", ia)
            keep += [ia]
        _geometry_attributes(dev, g, s, keep)
        dev.commit(g)
        mat = _material(dev, s["material"], keep)
        sf = dev.surface()
        dev.set(sf, "geometry", g)
        dev.set(sf, "material", mat)
        dev.commit(sf)
        keep += [g, mat]
        out.append(sf)
    return out


def _volumes(dev, vols, keep):
    out = []
    for v in vols:
        f = dev.spatial_field("structuredRegular")
        da = dev.array3d(np.asarray(v["data"], np.float32))
        dev.set(f, "data", da)
        dev.set(f, "origin", v["origin"], vsr.FLOAT32_VEC3)
        dev.set(f, "spacing", v["spacing"], vsr.FLOAT32_VEC3)
        dev.commit(f)
        vol = dev.volume("transferFunction1D")
        dev.set(vol, "value", f)
        ca = dev.array1d(np.asarray(v["color"], np.float32))
        oa = dev.array1d(np.asarray(v["opacity"], np.float32))
        dev.set(vol, "color", ca)
        dev.set(vol, "opacity", oa)
        dev.set(vol, "valueRange", v["valueRange"], vsr.FLOAT32_BOX1)
        dev.set(vol, "unitDistance", float(v["unitDistance"]))
        if "majorantBrickSize" in v:
            dev.set(vol, "majorantBrickSize", int(v["majorantBrickSize"]))
        dev.commit(vol)
        keep += [f, da, ca, oa]
        out.append(vol)
    return out


def _lights(dev, lights, keep):
    out = []
    for L in lights:
        kind = L.get("type", "directional")
        lt = dev.light(kind)
        dev.set(lt, "color", L.get("color", [1, 1, 1]), vsr.FLOAT32_VEC3)
        if "visible" in L:
            dev.set(lt, "visible", bool(L["visible"]))
        if kind == "hdri":
            rad = dev.array2d(np.ascontiguousarray(L["radiance"], np.float32))
            keep.append(rad)
            dev.set(lt, "radiance", rad)
            for k in ("up", "direction"):
                if k in L:
                    dev.set(lt, k, L[k], vsr.FLOAT32_VEC3)
            if "scale" in L:
                dev.set(lt, "scale", float(L["scale"]))
        elif kind == "directional":
            dev.set(lt, "direction", L["direction"], vsr.FLOAT32_VEC3)
            dev.set(lt, "irradiance", float(L.get("irradiance", 1.0)))
            if "angularDiameter" in L:
                dev.set(lt, "angularDiameter", float(L["angularDiameter"]))
        else:
            for k in ("position", "direction", "edge1", "edge2"):
                if k in L:
                    dev.set(lt, k, L[k], vsr.FLOAT32_VEC3)
            if "side" in L:
                dev.set(lt, "side", L["side"])
            for k in ("intensity", "openingAngle", "falloffAngle"):
                if k in L:
                    dev.set(lt, k, float(L[k]))
        dev.commit(lt)
        out.append(lt)
    return out


def _set_lists(dev, obj, surfs, vols, lights, keep):
    for name, lst in (("surface", surfs), ("volume", vols), ("light", lights)):
        if lst:
            arr = dev.array1d(lst)
            dev.set(obj, name, arr)
            keep.append(arr)
        keep += lst


def apply_renderer(dev, rend, params):
    for k, v in params.items():
        if k == "type":
            continue
        if k == "clipPlanes":
            arr = dev.array1d(np.asarray(v, np.float32).reshape(-1, 4))
            dev.set(rend, "clipPlane", arr)
            dev.release(arr)
        elif k == "background":
            dev.set(rend, k, v, vsr.FLOAT32_VEC4)
        elif k == "ambientColor":
            dev.set(rend, k, v, vsr.FLOAT32_VEC3)
        elif isinstance(v, (str, bool)):
            dev.set(rend, k, v)
        elif isinstance(v, (int, np.integer)):
            dev.set(rend, k, int(v))
        else:
            dev.set(rend, k, float(v))
    dev.commit(rend)


def apply_camera(dev, cam, c):
    for k in ("position", "direction", "up"):
        dev.set(cam, k, c[k], vsr.FLOAT32_VEC3)
    for k in ("fovy", "aspect", "apertureRadius", "focusDistance", "height"):
        if k in c:
            dev.set(cam, k, float(c[k]))
    if "view" in c:
        dev.set(cam, "view", c["view"], vsr.FLOAT32_MAT4)
        dev.set(cam, "proj", c["proj"], vsr.FLOAT32_MAT4)
    dev.commit(cam)


def build(dev, scene, channels=("color", "depth", "normal", "albedo"), collect_stats=False):
    """Create the scene's objects through the C ABI; returns a dict of handles."""
    keep = []
    world = dev.world()
    surfs = _surfaces(dev, scene.get("surfaces", []), keep)
    vols = _volumes(dev, scene.get("volumes", []), keep)
    lights = _lights(dev, scene.get("lights", []), keep)
    _set_lists(dev, world, surfs, vols, lights, keep)
    insts = []
    for I in scene.get("instances", []):
        grp = dev.group()
        _set_lists(dev, grp,
                   _surfaces(dev, I.get("surfaces", []), keep),
                   _volumes(dev, I.get("volumes", []), keep),
                   _lights(dev, I.get("lights", []), keep), keep)
        dev.commit(grp)
        inst = dev.instance("transform")
        dev.set(inst, "group", grp)
        dev.set(inst, "transform", I["transform"], vsr.FLOAT32_MAT3x4)
        for name, v in I.get("attributes", {}).items():
            _uniform(dev, inst, name, v)
        dev.commit(inst)
        keep.append(grp)
        insts.append(inst)
    if insts:
        arr = dev.array1d(insts)
        dev.set(world, "instance", arr)
        keep += [arr] + insts
    if "bvhBuild" in scene:
        dev.set(world, "bvhBuild", scene["bvhBuild"])
    if "bvhWidth" in scene:
        dev.set(world, "bvhWidth", int(scene["bvhWidth"]))
    if "bvhLeafSize" in scene:
        dev.set(world, "bvhLeafSize", int(scene["bvhLeafSize"]))
    dev.commit(world)
    cam = dev.camera(scene["camera"]["type"])
    apply_camera(dev, cam, scene["camera"])
    rend = dev.renderer(scene["renderer"]["type"])
    apply_renderer(dev, rend, scene["renderer"])
    frame = dev.frame()
    W, H = scene["frame"]["size"]
    dev.set(frame, "size", (W, H), vsr.UINT32_VEC2)
    types = {"color": vsr.FLOAT32_VEC4, "depth": vsr.FLOAT32, "normal": vsr.FLOAT32_VEC3,
             "albedo": vsr.FLOAT32_VEC3}
    for ch in channels:
        dev.set(frame, "channel." + ch, types[ch], vsr.DATA_TYPE)
    if collect_stats:
        dev.set(frame, "collectStatistics", True)
    dev.set(frame, "world", world)
    dev.set(frame, "camera", cam)
    dev.set(frame, "renderer", rend)
    dev.commit(frame)
    return {"world": world, "camera": cam, "renderer": rend, "frame": frame, "keep": keep}
