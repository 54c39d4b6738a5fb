"""ctypes binding of the CPU oracle (liboracle.so, built by oracle/Makefile).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the
CPU-baseline leg of bench.py. It converts a scene dict (the format of the
package's scenes.py) into the oracle's flat C structures with the same
group / surface / triangle order the renderer core uses, so triangle and
surface indices agree between the two.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

c_int32, c_uint32, c_float, c_void_p = ctypes.c_int32, ctypes.c_uint32, ctypes.c_float, ctypes.c_void_p
FP = ctypes.POINTER(ctypes.c_float)
DP = ctypes.POINTER(ctypes.c_double)
UP = ctypes.POINTER(ctypes.c_uint32)

MATTE, PBR = 0, 1
CAM_PERSPECTIVE, CAM_MATRIX, CAM_ORTHO, CAM_OMNI = 0, 1, 2, 3
RAYCAST, PATHTRACE = 0, 1
GRID_NONE, GRID_REFERENCE, GRID_BRICK = 0, 1, 2
COLOR_FLOAT4 = 0


class OrMaterial(ctypes.Structure):
    _fields_ = [("type", c_int32), ("baseColor", c_float * 3), ("opacity", c_float),
                ("metallic", c_float), ("roughness", c_float), ("ior", c_float),
                ("clearcoat", c_float), ("clearcoatRoughness", c_float), ("transmission", c_float),
                ("sheenColor", c_float * 3), ("sheenRoughness", c_float), ("alphaMode", c_int32),
                ("alphaCutoff", c_float), ("src", c_int32 * 4)]


class OrAttr(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("len", c_uint32), ("comps", c_int32), ("fixedBits", c_int32)]


class OrSurfAttr(ctypes.Structure):
    _fields_ = [("index", UP), ("vertexNormal", FP), ("numVertexNormals", c_uint32),
                ("fvNormal", c_int32), ("vertex", OrAttr * 5), ("faceVarying", OrAttr * 5),
                ("primitive", OrAttr * 5), ("uniform", (c_float * 4) * 5), ("uniformMask", c_uint32),
                ("isTriangle", c_int32)]


class OrSampler(ctypes.Structure):
    _fields_ = [("type", c_int32), ("inAttribute", c_int32), ("linear", c_int32),
                ("wrap", c_int32 * 3), ("dims", c_int32 * 3), ("image", c_void_p),
                ("imageType", c_int32), ("imageComps", c_int32), ("prim", OrAttr),
                ("primOffset", c_uint32), ("inXfm", c_float * 16), ("inOffset", c_float * 4),
                ("outXfm", c_float * 16), ("outOffset", c_float * 4)]


ATTR_NAMES = ["attribute0", "attribute1", "attribute2", "attribute3", "color", "worldPosition",
              "worldNormal", "objectPosition", "objectNormal"]


def attribute_id(name):
    """toAttribute (scene/surface/common.h:13-37); -1 for none / unknown."""
    return ATTR_NAMES.index(name) if name in ATTR_NAMES else -1


def _attr(arr, keep):
    """An OrAttr over a numpy array of float32 or uint8 / uint16 elements
    (1-D: one component, 2-D: the last axis)."""
    a = OrAttr()
    if arr is None:
        return a
    x = np.ascontiguousarray(arr)
    keep.append(x)
    a.data = x.ctypes.data
    a.len = x.shape[0]
    a.comps = 1 if x.ndim == 1 else x.shape[-1]
    a.fixedBits = {np.dtype(np.float32): 0, np.dtype(np.uint8): 8, np.dtype(np.uint16): 16}[x.dtype]
    return a


def _uniform4(v):
    v = [float(t) for t in (v if isinstance(v, (list, tuple, np.ndarray)) else [v])]
    return v + [0.0, 0.0, 0.0, 1.0][len(v):]


def surface_attributes(s, keep):
    """The OrSurfAttr of a surface dict ("normals", "attributes",
    "faceVarying", "primitive", "uniform"); None when it has none."""
    keys = ("normals", "attributes", "faceVarying", "primitive", "uniform")
    sa = OrSurfAttr()
    tri = s.get("geometry", "triangle") == "triangle"
    sa.isTriangle = 1 if tri else 0
    if tri:
        idx = np.ascontiguousarray(np.asarray(s["indices"], np.uint32).reshape(-1))
        keep.append(idx)
        sa.index = idx.ctypes.data_as(UP)
        if "normals" in s:
            n = np.ascontiguousarray(np.asarray(s["normals"], np.float32).reshape(-1, 3))
            keep.append(n)
            sa.vertexNormal = fptr(n)
            sa.numVertexNormals = len(n)
        for key, field in (("attributes", "vertex"), ("faceVarying", "faceVarying"),
                           ("primitive", "primitive")):
            for name, arr in s.get(key, {}).items():
                getattr(sa, field)[ATTR_NAMES.index(name)] = _attr(arr, keep)
    for name, v in s.get("uniform", {}).items():
        k = ATTR_NAMES.index(name)
        sa.uniform[k] = (c_float * 4)(*_uniform4(v))
        sa.uniformMask |= 1 << k
    return sa, any(k in s for k in keys)


def sampler_struct(d, keep):
    """An OrSampler from a sampler dict (the keys the scene builder takes)."""
    sp = OrSampler()
    kind = d["type"]
    sp.type = {"image1D": 0, "image2D": 1, "image3D": 2, "transform": 3, "primitive": 4}[kind]
    ia = attribute_id(d.get("inAttribute", "attribute0"))
    sp.inAttribute = ia if ia >= 0 else 15
    sp.linear = 0 if d.get("filter", "linear") == "nearest" else 1
    wm = {"repeat": 1, "mirrorRepeat": 2}
    sp.wrap = (c_int32 * 3)(*[wm.get(d.get(f"wrapMode{k}", "clampToEdge"), 0) for k in (1, 2, 3)])
    eye = [1.0 if i % 5 == 0 else 0.0 for i in range(16)]
    sp.inXfm = (c_float * 16)(*[float(x) for x in d.get("inTransform", eye)])
    sp.outXfm = (c_float * 16)(*[float(x) for x in d.get("outTransform", eye)])
    sp.inOffset = (c_float * 4)(*[float(x) for x in d.get("inOffset", [0, 0, 0, 0])])
    sp.outOffset = (c_float * 4)(*[float(x) for x in d.get("outOffset", [0, 0, 0, 0])])
    sp.dims = (c_int32 * 3)(1, 1, 1)
    if kind == "primitive":
        sp.prim = _attr(d["array"], keep)
        sp.primOffset = int(d.get("offset", 0))
    elif kind != "transform":
        img = np.ascontiguousarray(d["image"])
        keep.append(img)
        axes = {"image1D": 1, "image2D": 2, "image3D": 3}[kind]
        shape = img.shape[:axes][::-1]  # x fastest
        sp.dims = (c_int32 * 3)(*(list(shape) + [1] * (3 - axes)))
        sp.image = img.ctypes.data
        sp.imageComps = 1 if img.ndim == axes else img.shape[-1]
        srgb = d.get("srgb", False)
        sp.imageType = 0 if img.dtype == np.float32 else (2 if srgb else 1)
    return sp


class OrVolume(ctypes.Structure):
    _fields_ = [("data", FP), ("dims", c_int32 * 3), ("origin", c_float * 3),
                ("spacing", c_float * 3), ("tf", FP), ("tfSize", c_int32),
                ("valueRange", c_float * 2), ("unitDistance", c_float), ("gridMethod", c_int32),
                ("gridDims", c_int32 * 3), ("brickSize", c_int32)]


class OrGroup(ctypes.Structure):
    _fields_ = [("triBegin", c_int32), ("triEnd", c_int32), ("volBegin", c_int32), ("volEnd", c_int32),
                ("apBegin", c_int32), ("apEnd", c_int32), ("isoBegin", c_int32),
                ("isoEnd", c_int32)]


class OrIso(ctypes.Structure):
    _fields_ = [("field", c_int32), ("numValues", c_int32), ("values", FP), ("surface", c_uint32)]


class OrInstance(ctypes.Structure):
    _fields_ = [("xfm", c_float * 12), ("group", c_int32), ("userID", c_uint32),
                ("attr", (c_float * 4) * 5), ("attrMask", c_uint32)]


def _linear32(m, v):
    """m v in float32, each row summed left to right without contraction
    (the order the runtime uses to move light positions and edges)."""
    v = np.asarray(v, np.float32)
    f = np.float32
    return np.array([(f(m[k, 0]) * v[0] + f(m[k, 1]) * v[1]) + f(m[k, 2]) * v[2] for k in range(3)],
                    np.float32)


class OrLight(ctypes.Structure):
    _fields_ = [("type", c_int32), ("direction", c_float * 3), ("color", c_float * 3),
                ("irradiance", c_float), ("angularDiameter", c_float), ("visible", c_int32),
                ("position", c_float * 3), ("intensity", c_float), ("openingAngle", c_float),
                ("falloffAngle", c_float), ("edge1", c_float * 3), ("edge2", c_float * 3),
                ("radiance", FP), ("hdriW", c_int32), ("hdriH", c_int32), ("scale", c_float),
                ("up", c_float * 3)]


class OrScene(ctypes.Structure):
    _fields_ = [("numTriangles", c_int32), ("triVerts", FP), ("triSurface", UP), ("triPrimID", UP),
                ("numSurfaces", c_int32), ("surfMaterial", ctypes.POINTER(OrMaterial)),
                ("surfObjID", UP), ("numVolumes", c_int32), ("volumes", ctypes.POINTER(OrVolume)),
                ("numGroups", c_int32), ("groups", ctypes.POINTER(OrGroup)),
                ("numInstances", c_int32), ("instances", ctypes.POINTER(OrInstance)),
                ("numLights", c_int32), ("lights", ctypes.POINTER(OrLight)),
                ("numPrims", c_int32), ("prims", FP), ("primKind", ctypes.POINTER(c_int32)),
                ("primSurface", UP), ("triNormalFrom", ctypes.POINTER(c_int32)),
                ("numIsos", c_int32), ("isos", ctypes.POINTER(OrIso)),
                ("isoFields", ctypes.POINTER(OrVolume)), ("surfAttr", ctypes.POINTER(OrSurfAttr)),
                ("numSamplers", c_int32), ("samplers", ctypes.POINTER(OrSampler))]


class OrCamera(ctypes.Structure):
    _fields_ = [("type", c_int32), ("position", c_float * 3), ("direction", c_float * 3),
                ("up", c_float * 3), ("fovy", c_float), ("aspect", c_float),
                ("apertureRadius", c_float), ("focusDistance", c_float),
                ("imageRegion", c_float * 4), ("shutter", c_float * 2), ("height", c_float),
                ("view", c_float * 16), ("proj", c_float * 16)]


class OrRenderer(ctypes.Structure):
    _fields_ = [("type", c_int32), ("background", c_float * 4), ("ambientColor", c_float * 3),
                ("ambientRadiance", c_float), ("occlusionDistance", c_float),
                ("ambientSamples", c_int32), ("maxBounce", c_int32), ("pixelSamples", c_int32),
                ("volumeSamplingRate", c_float), ("numClipPlanes", c_int32), ("clipPlanes", FP),
                ("gradientShading", c_int32), ("taa", c_int32), ("taaAlpha", c_float)]


class OrFrame(ctypes.Structure):
    _fields_ = [("width", c_int32), ("height", c_int32), ("accumID", c_int32),
                ("colorType", c_int32), ("color", c_void_p), ("depth", FP), ("normal", FP),
                ("albedo", FP), ("accum", FP), ("sampleSum", DP), ("sampleSumSq", DP),
                ("rowBegin", c_int32), ("rowEnd", c_int32), ("tileSize", c_int32),
                ("taaCurr", FP), ("taaPrev", FP), ("taaCurrAlbedo", FP), ("taaPrevAlbedo", FP),
                ("motionVec", FP), ("prevMVP", c_float * 16), ("currMVP", c_float * 16)]


class OrStats(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_uint64), ("nodeVisits", ctypes.c_uint64),
                ("triTests", ctypes.c_uint64), ("marchSamples", ctypes.c_uint64),
                ("trackingSamples", ctypes.c_uint64), ("cellsVisited", ctypes.c_uint64)]


_lib = None


def build():
    """Compile liboracle.so with the committed Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        lib.or_scene_commit.restype = c_void_p
        lib.or_scene_commit.argtypes = [ctypes.POINTER(OrScene)]
        lib.or_scene_release.argtypes = [c_void_p]
        lib.or_frame_reset.argtypes = [ctypes.POINTER(OrFrame)]
        lib.or_render_frame.restype = ctypes.c_int
        lib.or_render_frame.argtypes = [c_void_p, ctypes.POINTER(OrCamera), ctypes.POINTER(OrRenderer),
                                        ctypes.POINTER(OrFrame), ctypes.c_int, ctypes.POINTER(OrStats)]
        lib.or_lcg_sequence.argtypes = [c_uint32, c_uint32, ctypes.c_int, FP]
        lib.or_sample_field.restype = c_float
        lib.or_sample_field.argtypes = [ctypes.POINTER(OrVolume), c_float, c_float, c_float]
        lib.or_tf_lookup.argtypes = [ctypes.POINTER(OrVolume), c_float, FP]
        lib.or_primary_ray.argtypes = [ctypes.POINTER(OrCamera), c_float, c_float, c_float, c_float,
                                       c_uint32, c_uint32, FP, FP]
        lib.or_eval_material.argtypes = [ctypes.POINTER(OrMaterial), FP, FP, FP, FP, FP]
        lib.or_sample_material.argtypes = [ctypes.POINTER(OrMaterial), FP, FP, FP, c_uint32, c_uint32,
                                           FP, FP, FP, FP]
        lib.or_majorants.restype = ctypes.c_int
        lib.or_majorants.argtypes = [c_void_p, ctypes.c_int, ctypes.POINTER(c_int32), FP, ctypes.c_int]
        lib.or_dda.restype = ctypes.c_int
        lib.or_dda.argtypes = [FP, FP, c_float, c_float, ctypes.POINTER(c_int32), FP, FP,
                               ctypes.POINTER(c_int32), FP, ctypes.c_int]
        lib.or_cvt.argtypes = [FP, ctypes.c_int, ctypes.c_int, UP]
        lib.or_trace.restype = ctypes.c_int
        lib.or_trace.argtypes = [c_void_p, FP, FP, c_float, c_float, FP, UP, UP, FP]
        _lib = lib
    return _lib


def fptr(a):
    return a.ctypes.data_as(FP)


def farr(n, vals):
    return (c_float * n)(*[float(v) for v in vals])


def material(m, samplers=None, keep=None):
    """An OrMaterial; a parameter given as an attribute name or as
    {"sampler": {...}} sets its source (the sampler appended to
    `samplers`) and keeps the parameter's default value."""
    om = OrMaterial()
    om.src = (c_int32 * 4)(-1, -1, -1, -1)

    def param(name, slot, default):
        v = m.get(name, default)
        if isinstance(v, dict):
            samplers.append(sampler_struct(v["sampler"], keep))
            om.src[slot] = 16 + len(samplers) - 1
            return default
        if isinstance(v, str):
            a = attribute_id(v)
            if a >= 0:
                om.src[slot] = a
            return default
        return v

    om.opacity = float(param("opacity", 1, 1.0))
    mode = m.get("alphaMode", "opaque")
    om.alphaMode = {"opaque": 0, "blend": 1, "mask": 2}[mode]
    om.alphaCutoff = float(m.get("alphaCutoff", 0.5))
    if m["type"] == "matte":
        om.type = MATTE
        c = param("color", 0, [1, 1, 1])
        om.baseColor = farr(3, c[:3])
    else:
        om.type = PBR
        c = param("baseColor", 0, [1, 1, 1])
        om.baseColor = farr(3, c[:3])
        om.metallic = float(param("metallic", 2, 1.0))
        om.roughness = float(param("roughness", 3, 1.0))
        om.ior = float(m.get("ior", 1.5))
        om.clearcoat = float(m.get("clearcoat", 0.0))
        om.clearcoatRoughness = float(m.get("clearcoatRoughness", 0.0))
        om.transmission = float(m.get("transmission", 0.0))
        om.sheenColor = farr(3, m.get("sheenColor", [0, 0, 0]))
        om.sheenRoughness = float(m.get("sheenRoughness", 0.0))
    return om


def build_tf(color, opacity):
    """TF table restated from TransferFunction1D::finalize
    (scene/volume/TransferFunction1D.cpp:50-112), colour float3 + opacity array."""
    color = np.asarray(color, np.float32)
    opacity = np.asarray(opacity, np.float32)
    nc, no = len(color), len(opacity)
    n = max(nc, no)
    out = np.zeros((n, 4), np.float32)
    f32 = np.float32
    for i in range(n):
        cp = f32((f32(i) / f32(n - 1)) * f32(nc - 1)) if n > 1 else f32(0)
        cf = f32(cp - f32(math.floor(cp)))
        c0 = np.append(color[int(math.floor(cp))], f32(1))
        c1 = np.append(color[int(math.ceil(cp))], f32(1))
        c = (c0 * (f32(1) - cf) + c1 * cf).astype(np.float32)
        ap = f32((f32(i) / f32(n - 1)) * f32(no - 1)) if n > 1 else f32(0)
        af = f32(ap - f32(math.floor(ap)))
        a0, a1 = opacity[int(math.floor(ap))], opacity[int(math.ceil(ap))]
        c[3] = f32(c[3] * f32(a0 * (f32(1) - af) + a1 * af))
        out[i] = c
    return out


def analytic_prims(s):
    """(N, 16) float32 records of a sphere (c, r), cone or cylinder (p0, r0,
    p1, r1) or Bezier curve (w0, r, w1, -, w2, -, w3, -) surface, following
    Sphere.cpp:46-75, Cone.cpp:49-82, Cylinder.cpp:49-82, BezierCurve.cpp:
    34-100: sphere centres through 'indices' when given, per-sphere 'radii'
    (else 'radius', default 0.01); cone / cylinder end points from
    'indices' pairs (else consecutive vertices), cone radii per end vertex
    ('radii' required), cylinder radii per cylinder ('radii') else 'radius'
    (default 1); curve segments every 3 vertices from each index entry to
    the next (one for the last), or from vertex 0 without indices, radius
    'radii' per index entry (per segment start / 3 without), else 'radius'
    (default 1), segments past the vertices left out."""
    kind = s["geometry"]
    pos = np.asarray(s["vertices"], np.float32).reshape(-1, 3)
    if kind == "bezierCurve":
        nv = len(pos)
        radii = np.asarray(s["radii"], np.float32).reshape(-1) if "radii" in s else None
        R = float(s.get("radius", 1.0))
        starts = []
        if "indices" in s:
            I = np.asarray(s["indices"], np.int64).reshape(-1)
            for i in range(len(I)):
                first = int(I[i])
                last = first + 3 if i == len(I) - 1 else int(I[i + 1])
                r = float(radii[i]) if radii is not None and i < len(radii) else R
                starts += [(j, r) for j in range(first, last, 3)]
        elif nv > 3:
            for i in range(0, nv - 3, 3):
                r = float(radii[i // 3]) if radii is not None and i // 3 < len(radii) else R
                starts.append((i, r))
        starts = [(j, r) for j, r in starts if j + 3 < nv]
        q = np.zeros((len(starts), 16), np.float32)
        for k, (j, r) in enumerate(starts):
            for c in range(4):
                q[k, 4 * c:4 * c + 3] = pos[j + c]
            q[k, 3] = r
        return q
    if kind == "sphere":
        c = pos[np.asarray(s["indices"], np.int64).reshape(-1)] if "indices" in s else pos
        r = (np.asarray(s["radii"], np.float32).reshape(-1)[:len(c)] if "radii" in s
             else np.full(len(c), s.get("radius", 0.01), np.float32))
        q = np.zeros((len(c), 16), np.float32)
        q[:, :3], q[:, 3] = c, r
        return q
    if "indices" in s:
        ab = np.asarray(s["indices"], np.int64).reshape(-1, 2)
    else:
        n = len(pos) // 2
        ab = np.stack([2 * np.arange(n), 2 * np.arange(n) + 1], axis=1)
    q = np.zeros((len(ab), 16), np.float32)
    q[:, :3], q[:, 4:7] = pos[ab[:, 0]], pos[ab[:, 1]]
    if kind == "cone":
        radii = np.asarray(s["radii"], np.float32).reshape(-1)
        q[:, 3], q[:, 7] = radii[ab[:, 0]], radii[ab[:, 1]]
    else:
        r = (np.asarray(s["radii"], np.float32).reshape(-1)[:len(ab)] if "radii" in s
             else np.full(len(ab), s.get("radius", 1.0), np.float32))
        q[:, 3], q[:, 7] = r, r
    return q


class Scene:
    """A scene dict committed to the oracle (owns all buffers it points to)."""

    def __init__(self, scene, grid_method=GRID_BRICK, grid_dims=(16, 16, 16)):
        lib = load()
        self._keep = []
        groups = []   # (surfaces, volumes, lights, xfm)
        if scene.get("surfaces") or scene.get("volumes") or scene.get("lights"):
            groups.append((scene.get("surfaces", []), scene.get("volumes", []),
                           scene.get("lights", []), [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]))
        inst_attrs = [{}] if groups else []
        for inst in scene.get("instances", []):
            groups.append((inst.get("surfaces", []), inst.get("volumes", []),
                           inst.get("lights", []), inst["transform"]))
            inst_attrs.append(inst.get("attributes", {}))
        verts, tsurf, tprim, mats, vols, ogroups, oinsts, lights = [], [], [], [], [], [], [], []
        sattrs, samplers, any_attr = [], [], False

        def add_material(s):
            nonlocal any_attr
            sa, has = surface_attributes(s, self._keep)
            om = material(s["material"], samplers, self._keep)
            sattrs.append(sa)
            any_attr = any_attr or has or any(x != -1 for x in om.src)
            mats.append(om)
        aps, akind, asurf = [], [], []
        nfrom, has_quads = [], False
        isos, iso_fields = [], []
        ntri = nap = 0
        for gi, (surfs, vls, lts, xfm) in enumerate(groups):
            g = OrGroup()
            g.triBegin = ntri
            g.apBegin = nap
            g.isoBegin = len(isos)
            for s in surfs:
                if s.get("geometry") == "isosurface":
                    data = np.ascontiguousarray(s["data"], np.float32)
                    vals = np.ascontiguousarray(s["isovalues"], np.float32).reshape(-1)
                    self._keep += [data, vals]
                    ov = OrVolume()
                    ov.data = fptr(data)
                    nz, ny, nx = data.shape
                    ov.dims = (c_int32 * 3)(nx, ny, nz)
                    ov.origin = farr(3, s.get("origin", [0, 0, 0]))
                    ov.spacing = farr(3, s.get("spacing", [1, 1, 1]))
                    oi = OrIso()
                    oi.field = len(iso_fields)
                    oi.numValues = len(vals)
                    oi.values = fptr(vals)
                    oi.surface = len(mats)
                    add_material(s)
                    iso_fields.append(ov)
                    isos.append(oi)
                    continue
                kind = s.get("geometry", "triangle")
                if kind in ("sphere", "cone", "cylinder", "bezierCurve"):
                    q = analytic_prims(s)
                    aps.append(q)
                    akind.append(np.full(len(q), {"sphere": 0, "cone": 1, "cylinder": 2,
                                                  "bezierCurve": 3}[kind], np.int32))
                    asurf.append(np.full(len(q), len(mats), np.uint32))
                    add_material(s)
                    nap += len(q)
                    continue
                v = np.asarray(s["vertices"], np.float32)
                if kind == "quad":
                    # Quad.cpp:69-110: (v1, v2, v4) and (v3, v4, v2) per quad;
                    # triangle k of the list shades quad k's two triangles
                    q = (np.asarray(s["indices"], np.int64).reshape(-1, 4) if "indices" in s
                         else np.arange(len(v) // 4 * 4).reshape(-1, 4))
                    t = np.stack([q[:, [0, 1, 3]], q[:, [2, 3, 1]]], axis=1).reshape(-1, 3)
                    nfrom.append(ntri + np.arange(len(t)) // 2)
                    has_quads = True
                else:
                    t = np.asarray(s["indices"], np.uint32)
                    nfrom.append(np.full(len(t), -1, np.int64))
                verts.append(v[t].reshape(-1, 9))
                sid = len(mats)
                add_material(s)
                tsurf.append(np.full(len(t), sid, np.uint32))
                tprim.append(np.arange(len(t), dtype=np.uint32))
                ntri += len(t)
            g.triEnd = ntri
            g.apEnd = nap
            g.isoEnd = len(isos)
            g.volBegin = len(vols)
            for v in vls:
                ov = OrVolume()
                data = np.ascontiguousarray(v["data"], np.float32)
                tf = build_tf(v["color"], v["opacity"])
                self._keep += [data, tf]
                ov.data = fptr(data)
                nz, ny, nx = data.shape
                ov.dims = (c_int32 * 3)(nx, ny, nz)
                ov.origin = farr(3, v["origin"])
                ov.spacing = farr(3, v["spacing"])
                ov.tf = fptr(tf)
                ov.tfSize = len(tf)
                ov.valueRange = farr(2, v["valueRange"])
                ov.unitDistance = float(v["unitDistance"]) or 1.0
                ov.gridMethod = grid_method
                ov.gridDims = (c_int32 * 3)(*grid_dims)
                ov.brickSize = int(v.get("majorantBrickSize", 16))
                vols.append(ov)
            g.volEnd = len(vols)
            ogroups.append(g)
            oi = OrInstance()
            oi.xfm = farr(12, xfm)
            oi.group = gi
            oi.userID = 0xffffffff
            for name, v in inst_attrs[gi].items():
                k = ATTR_NAMES.index(name)
                oi.attr[k] = (c_float * 4)(*_uniform4(v))
                oi.attrMask |= 1 << k
                any_attr = True
            oinsts.append(oi)
            lin = np.asarray(xfm, np.float64)[:9].reshape(3, 3).T  # column-major -> matrix
            tr = np.asarray(xfm, np.float32)[9:12]
            for L in lts:
                ol = OrLight()
                kind = L.get("type", "directional")
                ol.type = {"directional": 0, "point": 1, "spot": 2, "quad": 3, "hdri": 4}[kind]
                ol.color = farr(3, L.get("color", [1, 1, 1]))
                ol.visible = 1 if L.get("visible", True) else 0
                if kind == "hdri":
                    # no instance transform (xfmLight leaves HDRI lights as they are)
                    rad = np.ascontiguousarray(L["radiance"], np.float32)
                    self._keep.append(rad)
                    ol.radiance = fptr(rad)
                    ol.hdriH, ol.hdriW = int(rad.shape[0]), int(rad.shape[1])
                    ol.scale = float(L.get("scale", 1.0))
                    ol.up = farr(3, L.get("up", [1, 0, 0]))
                    ol.direction = farr(3, L.get("direction", [0, 0, 1]))
                elif kind == "directional":
                    d = lin @ np.asarray(L["direction"], np.float64)
                    ol.direction = farr(3, d / np.linalg.norm(d))
                    ol.irradiance = float(L.get("irradiance", 1.0))
                    ol.angularDiameter = float(L.get("angularDiameter", 0.0))
                else:
                    # positions by the instance's affine transform, the spot
                    # axis by its linear part, in float32 as the device does
                    lin32 = lin.astype(np.float32)
                    p0 = np.asarray(L.get("position", [0, 0, -1] if kind == "point" else [0, 0, 0]),
                                    np.float32)
                    ol.position = farr(3, _linear32(lin32, p0) + tr)
                    if kind == "quad":
                        ol.edge1 = farr(3, _linear32(lin32, L.get("edge1", [1, 0, 0])))
                        ol.edge2 = farr(3, _linear32(lin32, L.get("edge2", [0, 1, 0])))
                    ol.intensity = float(min(max(L.get("intensity", 1.0), 0.0), 3.4e38))
                    if kind == "spot":
                        ol.direction = farr(3, lin32 @ np.asarray(L.get("direction", [0, 0, -1]),
                                                                  np.float32))
                        ol.openingAngle = float(L.get("openingAngle", math.pi))
                        ol.falloffAngle = float(L.get("falloffAngle", 0.1))
                lights.append(ol)
        tri = np.ascontiguousarray(np.concatenate(verts) if verts else np.zeros((0, 9), np.float32))
        ts = np.ascontiguousarray(np.concatenate(tsurf) if tsurf else np.zeros(0, np.uint32))
        tp = np.ascontiguousarray(np.concatenate(tprim) if tprim else np.zeros(0, np.uint32))
        ap = np.ascontiguousarray(np.concatenate(aps) if aps else np.zeros((0, 16), np.float32),
                                  np.float32)
        ak = np.ascontiguousarray(np.concatenate(akind) if akind else np.zeros(0, np.int32))
        asf = np.ascontiguousarray(np.concatenate(asurf) if asurf else np.zeros(0, np.uint32))
        nf = np.ascontiguousarray(np.concatenate(nfrom) if nfrom else np.zeros(0), np.int32)
        self._keep += [tri, ts, tp, ap, ak, asf, nf]
        self.mats = (OrMaterial * max(1, len(mats)))(*mats)
        self.vols = (OrVolume * max(1, len(vols)))(*vols)
        self.groups = (OrGroup * max(1, len(ogroups)))(*ogroups)
        self.insts = (OrInstance * max(1, len(oinsts)))(*oinsts)
        self.lights = (OrLight * max(1, len(lights)))(*lights)
        objid = np.zeros(max(1, len(mats)), np.uint32)
        self._keep.append(objid)
        self.sattrs = (OrSurfAttr * max(1, len(sattrs)))(*sattrs)
        self.samplers = (OrSampler * max(1, len(samplers)))(*samplers)
        sc = OrScene()
        if any_attr:
            sc.surfAttr = self.sattrs
            sc.numSamplers = len(samplers)
            sc.samplers = self.samplers
        sc.numTriangles = len(tri)
        sc.triVerts = fptr(tri)
        sc.triSurface = ts.ctypes.data_as(UP)
        sc.triPrimID = tp.ctypes.data_as(UP)
        sc.numSurfaces = len(mats)
        sc.surfMaterial = self.mats
        sc.surfObjID = objid.ctypes.data_as(UP)
        sc.numVolumes = len(vols)
        sc.volumes = self.vols
        sc.numGroups = len(ogroups)
        sc.groups = self.groups
        sc.numInstances = len(oinsts)
        sc.instances = self.insts
        sc.numLights = len(lights)
        sc.lights = self.lights
        sc.numPrims = len(ap)
        sc.prims = fptr(ap)
        sc.primKind = ak.ctypes.data_as(ctypes.POINTER(c_int32))
        sc.primSurface = asf.ctypes.data_as(UP)
        sc.triNormalFrom = (nf.ctypes.data_as(ctypes.POINTER(c_int32)) if has_quads
                            else ctypes.POINTER(c_int32)())
        self.isos = (OrIso * max(1, len(isos)))(*isos)
        self.iso_fields = (OrVolume * max(1, len(iso_fields)))(*iso_fields)
        sc.numIsos = len(isos)
        sc.isos = self.isos
        sc.isoFields = self.iso_fields
        self.scene = sc
        self.handle = lib.or_scene_commit(ctypes.byref(sc))
        self.camera = camera(scene["camera"])
        self.renderer = renderer(scene["renderer"])
        self.sample_chunks = sample_chunks(scene["renderer"])
        self.size = tuple(scene["frame"]["size"])

    def close(self):
        if self.handle:
            load().or_scene_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def camera(c):
    oc = OrCamera()
    oc.type = {"perspective": CAM_PERSPECTIVE, "matrix": CAM_MATRIX, "orthographic": CAM_ORTHO,
               "omnidirectional": CAM_OMNI}[c["type"]]
    oc.position = farr(3, c.get("position", [0, 0, 0]))
    oc.direction = farr(3, c.get("direction", [0, 0, 1]))
    oc.up = farr(3, c.get("up", [0, 1, 0]))
    oc.fovy = float(c.get("fovy", math.radians(60.0)))
    oc.aspect = float(c.get("aspect", 1.0))
    oc.apertureRadius = float(c.get("apertureRadius", 0.0))
    oc.focusDistance = float(c.get("focusDistance", 1.0))
    oc.imageRegion = farr(4, c.get("imageRegion", [0, 0, 1, 1]))
    oc.shutter = farr(2, c.get("shutter", [0.5, 0.5]))
    oc.height = float(c.get("height", 1.0))
    oc.view = farr(16, c.get("view", np.eye(4).reshape(-1)))
    oc.proj = farr(16, c.get("proj", np.eye(4).reshape(-1)))
    return oc


def sample_chunks(r):
    """The renderer's sample chunks as the renderer core resolves them: a
    divisor of pixelSamples, at most 16 (path tracer only)."""
    if r.get("type", "pathtrace") == "raycast" or r.get("taa", False):
        return 1
    spp = int(r.get("pixelSamples", 1))
    k = min(max(int(r.get("sampleChunks", 1)), 1), min(16, spp))
    while spp % k:
        k -= 1
    return k


def renderer(r):
    orr = OrRenderer()
    orr.type = RAYCAST if r["type"] == "raycast" else PATHTRACE
    orr.background = farr(4, r.get("background", [0, 0, 0, 1]))
    orr.ambientColor = farr(3, r.get("ambientColor", [1, 1, 1]))
    orr.ambientRadiance = float(r.get("ambientRadiance", 0.2))
    orr.occlusionDistance = float(r.get("ambientOcclusionDistance", 1e20))
    orr.ambientSamples = int(r.get("ambientSamples", 1))
    orr.maxBounce = int(r.get("maxBounce", 7))
    orr.pixelSamples = int(r.get("pixelSamples", 1)) if orr.type == PATHTRACE else 1
    orr.volumeSamplingRate = float(r.get("volumeSamplingRate", 0.5))
    planes = np.asarray(r.get("clipPlanes", np.zeros((0, 4))), np.float32).reshape(-1, 4)
    orr.numClipPlanes = len(planes)
    orr._planes = np.ascontiguousarray(planes)
    orr.clipPlanes = fptr(orr._planes)
    orr.gradientShading = 1 if r.get("gradientShading", False) else 0
    orr.taa = 1 if (r.get("taa", False) and orr.type == PATHTRACE) else 0
    orr.taaAlpha = float(r.get("taaAlpha", 0.3))
    return orr


class Frame:
    """Frame buffers of the oracle (float4 colour, depth, normal, albedo)."""

    def __init__(self, w, h, stats=False, taa=False):
        self.w, self.h = w, h
        self.color = np.zeros((h, w, 4), np.float32)
        self.depth = np.zeros((h, w), np.float32)
        self.normal = np.zeros((h, w, 3), np.float32)
        self.albedo = np.zeros((h, w, 3), np.float32)
        self.accum = np.zeros((h, w, 4), np.float32)
        self.sum = np.zeros((h, w, 3), np.float64) if stats else None
        self.sumsq = np.zeros((h, w, 3), np.float64) if stats else None
        f = OrFrame()
        f.width, f.height = w, h
        f.colorType = COLOR_FLOAT4
        f.color = self.color.ctypes.data
        f.depth = fptr(self.depth)
        f.normal = fptr(self.normal)
        f.albedo = fptr(self.albedo)
        f.accum = fptr(self.accum)
        if stats:
            f.sampleSum = self.sum.ctypes.data_as(DP)
            f.sampleSumSq = self.sumsq.ctypes.data_as(DP)
        eye = [1.0 if i % 5 == 0 else 0.0 for i in range(16)]
        f.prevMVP = (c_float * 16)(*eye)
        f.currMVP = (c_float * 16)(*eye)
        if taa:
            # TAA buffers, zero at first (frame/Frame.cpp:535-540)
            self.taa_curr = np.zeros((h, w, 4), np.float32)
            self.taa_prev = np.zeros((h, w, 4), np.float32)
            self.taa_curr_albedo = np.zeros((h, w, 3), np.float32)
            self.taa_prev_albedo = np.zeros((h, w, 3), np.float32)
            self.motion_vec = np.zeros((h, w, 2), np.float32)
            f.taaCurr = fptr(self.taa_curr)
            f.taaPrev = fptr(self.taa_prev)
            f.taaCurrAlbedo = fptr(self.taa_curr_albedo)
            f.taaPrevAlbedo = fptr(self.taa_prev_albedo)
            f.motionVec = fptr(self.motion_vec)
        self.f = f
        load().or_frame_reset(ctypes.byref(f))


def render(sc, frame, num_threads=0, rows=None, stats=None, tile=None):
    """Render one frame of committed scene `sc` into `frame` (accumulating).
    tile: pixel tile edge handed to each thread (default 64, the reference
    CPU device's); smaller tiles spread small frames over more threads."""
    if rows is not None:
        frame.f.rowBegin, frame.f.rowEnd = rows
    if tile is not None:
        frame.f.tileSize = int(tile)
    k = getattr(sc, "sample_chunks", 1)
    if k > 1:
        # a frame of K sample chunks is K accumulated sub-frames of spp / K
        # samples with accumulation IDs K * accumID + c
        spp = sc.renderer.pixelSamples
        base = frame.f.accumID
        sc.renderer.pixelSamples = spp // k
        try:
            for c in range(k):
                frame.f.accumID = base * k + c
                render_once(sc, frame, num_threads, stats)
        finally:
            sc.renderer.pixelSamples = spp
        frame.f.accumID = base + 1
        return stats
    return render_once(sc, frame, num_threads, stats)


def render_once(sc, frame, num_threads=0, stats=None):
    st = stats if stats is not None else OrStats()
    load().or_render_frame(sc.handle, ctypes.byref(sc.camera), ctypes.byref(sc.renderer),
                           ctypes.byref(frame.f), num_threads, ctypes.byref(st))
    return st
