"""Python binding of the renderer core's C ABI (include/vsr.h).

A thin ctypes layer with the call sequence of the ANARI API that the
reference device implements: create objects, set parameters, commit,
render, wait, map channels. It is what the tests and the benchmark drive;
the work happens in libvsr.so (CUDA). There is no CPU fallback: creating a
Device fails loudly when the library is missing or no GPU is present.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvsr.so")

# VSRDataType (include/vsr.h)
UNKNOWN, STRING, OBJECT, ARRAY1D, ARRAY2D, ARRAY3D, CAMERA, FRAME, GEOMETRY, GROUP, INSTANCE, \
    LIGHT, MATERIAL, RENDERER, SURFACE, SPATIAL_FIELD, VOLUME, WORLD, DATA_TYPE, BOOL, INT32, \
    UINT32, INT32_VEC2, UINT32_VEC2, UINT32_VEC3, FLOAT32, FLOAT32_VEC2, FLOAT32_VEC3, \
    FLOAT32_VEC4, FLOAT32_BOX1, FLOAT32_MAT4, FLOAT32_MAT3x4, UFIXED8, UFIXED8_VEC4, \
    UFIXED8_RGBA_SRGB, UFIXED16, FLOAT64_BOX1, UINT64, FLOAT64, UINT32_VEC4, SAMPLER, \
    UFIXED8_VEC2, UFIXED8_VEC3 = range(43)

OK = 0
WAIT, NO_WAIT = 1, 0

_OBJECT_KINDS = set(range(OBJECT, WORLD + 1)) | {SAMPLER}

_CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                             ctypes.c_int, ctypes.c_int, ctypes.c_char_p)

# exported symbols of include/vsr.h: (name, restype, argtypes)
_P = ctypes.c_void_p
_SIGNATURES = [
    ("vsrNewDevice", _P, [ctypes.c_char_p, _CALLBACK, _P]),
    ("vsrReleaseDevice", ctypes.c_int, [_P]),
    ("vsrNewArray1D", _P, [_P, _P, ctypes.c_int, ctypes.c_uint64]),
    ("vsrNewArray2D", _P, [_P, _P, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]),
    ("vsrNewArray3D", _P, [_P, _P, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]),
    ("vsrNewSpatialField", _P, [_P, ctypes.c_char_p]),
    ("vsrNewVolume", _P, [_P, ctypes.c_char_p]),
    ("vsrNewGeometry", _P, [_P, ctypes.c_char_p]),
    ("vsrNewMaterial", _P, [_P, ctypes.c_char_p]),
    ("vsrNewLight", _P, [_P, ctypes.c_char_p]),
    ("vsrNewSurface", _P, [_P]),
    ("vsrNewGroup", _P, [_P]),
    ("vsrNewInstance", _P, [_P, ctypes.c_char_p]),
    ("vsrNewWorld", _P, [_P]),
    ("vsrNewCamera", _P, [_P, ctypes.c_char_p]),
    ("vsrNewRenderer", _P, [_P, ctypes.c_char_p]),
    ("vsrNewSampler", _P, [_P, ctypes.c_char_p]),
    ("vsrNewFrame", _P, [_P]),
    ("vsrSetParameter", ctypes.c_int, [_P, _P, ctypes.c_char_p, ctypes.c_int, _P]),
    ("vsrUnsetParameter", ctypes.c_int, [_P, _P, ctypes.c_char_p]),
    ("vsrCommitParameters", ctypes.c_int, [_P, _P]),
    ("vsrRelease", ctypes.c_int, [_P, _P]),
    ("vsrRetain", ctypes.c_int, [_P, _P]),
    ("vsrGetProperty", ctypes.c_int, [_P, _P, ctypes.c_char_p, ctypes.c_int, _P, ctypes.c_uint64,
                                      ctypes.c_int]),
    ("vsrRenderFrame", ctypes.c_int, [_P, _P]),
    ("vsrRenderFrames", ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.c_uint32]),
    ("vsrPlanBatch", ctypes.c_uint64, [ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                       ctypes.POINTER(ctypes.c_float), ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint64]),
    ("vsrNewDenoiser", _P, [_P, ctypes.c_uint64]),
    ("vsrReleaseDenoiser", ctypes.c_int, [_P, _P]),
    ("vsrDenoiserParameterCount", ctypes.c_uint64, [_P, _P]),
    ("vsrDenoiserSetTensorPath", ctypes.c_int, [_P, _P, ctypes.c_int]),
    ("vsrDenoiserErrors", ctypes.c_uint32, [_P, _P]),
    ("vsrDenoiserTestWaitTimeout", ctypes.c_int, [_P, _P]),
    ("vsrDenoiserGetParameters", ctypes.c_int, [_P, _P, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64]),
    ("vsrDenoiserSetParameters", ctypes.c_int, [_P, _P, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64]),
    ("vsrDenoiserForward", ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _P]),
    ("vsrDenoiserGradients", ctypes.c_int, [_P, _P, _P, _P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.c_uint32, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64,
                                            ctypes.POINTER(ctypes.c_float)]),
    ("vsrDenoiserTrainStep", ctypes.c_int, [_P, _P, _P, _P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.c_uint32, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    ("vsrDenoiserFrameInput", ctypes.c_int, [_P, _P, _P]),
    ("vsrDenoiseFrame", ctypes.c_int, [_P, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P,
                                       ctypes.POINTER(ctypes.c_uint32)]),
    ("vsrFrameReady", ctypes.c_int, [_P, _P, ctypes.c_int]),
    ("vsrDiscardFrame", ctypes.c_int, [_P, _P]),
    ("vsrFrameSampleMask", ctypes.c_int, [_P, _P, _P]),
    ("vsrMapFrame", _P, [_P, _P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint32),
                         ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)]),
    ("vsrUnmapFrame", ctypes.c_int, [_P, _P, ctypes.c_char_p]),
    ("vsrMapFrameDevice", _P, [_P, _P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint32),
                               ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)]),
    ("vsrDeviceStream", _P, [_P]),
    ("vsrBuildTriangleBVH", ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, _P, _P, _P]),
    ("vsrBuildTriangleBVHNoAlloc", ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, _P, _P, _P]),
]

EXPORTED_SYMBOLS = [s[0] for s in _SIGNATURES]

_lib = None


def plan_batch(widths, heights, costs, tile_width, lib=None):
    """Work list of a batch (vsrPlanBatch): an (n, 2) uint32 array of (job,
    tile) pairs. Needs no GPU."""
    import numpy as np
    lib = lib or load_library()
    n = len(widths)
    w = (ctypes.c_uint32 * n)(*widths)
    h = (ctypes.c_uint32 * n)(*heights)
    c = (ctypes.c_float * n)(*costs)
    count = lib.vsrPlanBatch(w, h, c, n, tile_width, None, 0)
    out = np.zeros((count, 2), dtype=np.uint32)
    if count:
        lib.vsrPlanBatch(w, h, c, n, tile_width,
                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), count)
    return out


def load_library(path=LIB_PATH):
    """Load libvsr.so and declare its prototypes. Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"renderer core library not built: {path} (run anari-visionaray_gb300/build.py)")
    lib = ctypes.CDLL(path)
    for name, res, args in _SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class Obj:
    """Handle of one object of the renderer core."""

    def __init__(self, ptr, kind, subtype=""):
        if not ptr:
            raise RuntimeError(f"object creation failed (kind {kind}, subtype '{subtype}')")
        self.ptr = ptr
        self.kind = kind
        self.subtype = subtype


_ARRAY_TYPES = {
    (np.dtype(np.float32), 1): FLOAT32,
    (np.dtype(np.float32), 2): FLOAT32_VEC2,
    (np.dtype(np.float32), 3): FLOAT32_VEC3,
    (np.dtype(np.float32), 4): FLOAT32_VEC4,
    (np.dtype(np.uint32), 1): UINT32,
    (np.dtype(np.uint32), 2): UINT32_VEC2,
    (np.dtype(np.uint32), 3): UINT32_VEC3,
    (np.dtype(np.uint32), 4): UINT32_VEC4,
    (np.dtype(np.uint8), 1): UFIXED8,
    (np.dtype(np.uint8), 2): UFIXED8_VEC2,
    (np.dtype(np.uint8), 3): UFIXED8_VEC3,
    (np.dtype(np.uint8), 4): UFIXED8_VEC4,
    (np.dtype(np.uint16), 1): UFIXED16,
}


class Denoiser:
    """The learned denoiser (vsrNewDenoiser). Image arguments are device
    pointers (ints), e.g. torch's data_ptr(); inputs NHWC bf16 with 16
    channels, outputs NHWC fp32 with 16 channels (log(1 + colour) in 0..2)."""

    IN_C = 16
    OUT_C = 16

    def __init__(self, dev, seed=0):
        self.dev = dev
        self.lib = dev.lib
        self.handle = self.lib.vsrNewDenoiser(dev.handle, seed)
        if not self.handle:
            raise RuntimeError("vsrNewDenoiser failed: " + "; ".join(m[2] for m in dev.messages))
        self.count = int(self.lib.vsrDenoiserParameterCount(dev.handle, self.handle))

    def close(self):
        if self.handle:
            self.lib.vsrReleaseDenoiser(self.dev.handle, self.handle)
            self.handle = None

    def set_tensor_path(self, path):
        """0: mma.sync convolutions; 1: tcgen05 (persistent warp-specialised
        kernel with TMA loads) where a level is at least 128 pixels wide,
        mma.sync below; 2 (default): that kernel at every width; 3: as 1 on
        the one-tile-per-CTA tcgen05 kernel; 4: as 2 with the weight
        gradients on tcgen05 as well."""
        rc = self.lib.vsrDenoiserSetTensorPath(self.dev.handle, self.handle, path)
        if rc:
            raise RuntimeError(f"vsrDenoiserSetTensorPath failed ({rc})")

    def errors(self):
        """The tcgen05 path's device error word (1: a bounded wait ran out);
        reading clears it."""
        return int(self.lib.vsrDenoiserErrors(self.dev.handle, self.handle))

    def test_wait_timeout(self):
        """Arm the timeout-path test for the next tcgen05 convolution launch
        (its waits run out after one second; error word 1)."""
        rc = self.lib.vsrDenoiserTestWaitTimeout(self.dev.handle, self.handle)
        if rc:
            raise RuntimeError(f"vsrDenoiserTestWaitTimeout failed ({rc})")

    def params(self):
        out = np.zeros(self.count, np.float32)
        rc = self.lib.vsrDenoiserGetParameters(self.dev.handle, self.handle,
                                               out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.count)
        if rc:
            raise RuntimeError(f"vsrDenoiserGetParameters failed ({rc})")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        rc = self.lib.vsrDenoiserSetParameters(self.dev.handle, self.handle,
                                               p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.count)
        if rc:
            raise RuntimeError(f"vsrDenoiserSetParameters failed ({rc})")

    def forward(self, x_ptr, n, h, w, out_ptr):
        rc = self.lib.vsrDenoiserForward(self.dev.handle, self.handle, x_ptr, n, h, w, out_ptr)
        if rc:
            raise RuntimeError(f"vsrDenoiserForward failed ({rc})")

    def gradients(self, x_ptr, t_ptr, t_stride, n, h, w):
        g = np.zeros(self.count, np.float32)
        loss = ctypes.c_float(0)
        rc = self.lib.vsrDenoiserGradients(self.dev.handle, self.handle, x_ptr, t_ptr, t_stride, n, h, w,
                                           g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.count,
                                           ctypes.byref(loss))
        if rc:
            raise RuntimeError(f"vsrDenoiserGradients failed ({rc})")
        return g, loss.value

    def train_step(self, x_ptr, t_ptr, t_stride, n, h, w, lr, want_loss=True):
        loss = ctypes.c_float(0)
        rc = self.lib.vsrDenoiserTrainStep(self.dev.handle, self.handle, x_ptr, t_ptr, t_stride, n, h, w,
                                           lr, ctypes.byref(loss) if want_loss else None)
        if rc:
            raise RuntimeError(f"vsrDenoiserTrainStep failed ({rc})")
        return loss.value if want_loss else None

    def frame_input(self, frame, x_ptr):
        rc = self.lib.vsrDenoiserFrameInput(self.dev.handle, frame.ptr, x_ptr)
        if rc:
            raise RuntimeError(f"vsrDenoiserFrameInput failed ({rc})")

    def denoise_frame(self, frame, color_ptr, k=3.0, floor=0.0, retry_ptr=None):
        n = ctypes.c_uint32(0)
        rc = self.lib.vsrDenoiseFrame(self.dev.handle, self.handle, frame.ptr, k, floor, color_ptr,
                                      retry_ptr, ctypes.byref(n))
        if rc:
            raise RuntimeError(f"vsrDenoiseFrame failed ({rc})")
        return n.value


class Device:
    """A renderer-core device (anariNewDevice counterpart)."""

    def __init__(self, lib_path=LIB_PATH):
        self.lib = load_library(lib_path)
        self.messages = []

        def cb(user, dev, src, srcType, severity, code, msg):
            self.messages.append((severity, code, msg.decode() if msg else ""))

        self._cb = _CALLBACK(cb)
        self.handle = self.lib.vsrNewDevice(b"default", self._cb, None)
        if not self.handle:
            raise RuntimeError("vsrNewDevice failed: " + "; ".join(m[2] for m in self.messages))
        self._keep = []

    def close(self):
        if self.handle:
            self.lib.vsrReleaseDevice(self.handle)
            self.handle = None

    # -- objects -----------------------------------------------------------
    def array1d(self, data, dtype=None):
        return self._array(data, dtype, 1)

    def array2d(self, data, dtype=None):
        """data indexed [y, x] or [y, x, component] (x fastest in memory)."""
        return self._array(data, dtype, 2)

    def array3d(self, data, dtype=None):
        """data indexed [z, y, x] (x fastest in memory)."""
        return self._array(data, dtype, 3)

    def _array(self, data, dtype, dims):
        if isinstance(data, (list, tuple)) and data and isinstance(data[0], Obj):
            kind = data[0].kind
            ptrs = (ctypes.c_void_p * len(data))(*[o.ptr for o in data])
            h = self.lib.vsrNewArray1D(self.handle, ctypes.cast(ptrs, ctypes.c_void_p), kind, len(data))
            return Obj(h, ARRAY1D)
        a = np.ascontiguousarray(data)
        if dims == 3:
            nz, ny, nx = a.shape[:3]
            comps = 1 if a.ndim == 3 else a.shape[-1]
            t = dtype if dtype is not None else _ARRAY_TYPES[(a.dtype, comps)]
            h = self.lib.vsrNewArray3D(self.handle, a.ctypes.data, t, nx, ny, nz)
            return Obj(h, ARRAY3D)
        if dims == 2:
            ny, nx = a.shape[:2]
            comps = 1 if a.ndim == 2 else a.shape[-1]
            t = dtype if dtype is not None else _ARRAY_TYPES[(a.dtype, comps)]
            h = self.lib.vsrNewArray2D(self.handle, a.ctypes.data, t, nx, ny)
            return Obj(h, ARRAY2D)
        comps = 1 if a.ndim == 1 else a.shape[-1]
        t = dtype if dtype is not None else _ARRAY_TYPES[(a.dtype, comps)]
        h = self.lib.vsrNewArray1D(self.handle, a.ctypes.data, t, a.shape[0])
        return Obj(h, ARRAY1D)

    def _new(self, fn, kind, subtype=None):
        f = getattr(self.lib, fn)
        h = f(self.handle, subtype.encode()) if subtype is not None else f(self.handle)
        return Obj(h, kind, subtype or "")

    def spatial_field(self, subtype="structuredRegular"):
        return self._new("vsrNewSpatialField", SPATIAL_FIELD, subtype)

    def volume(self, subtype="transferFunction1D"):
        return self._new("vsrNewVolume", VOLUME, subtype)

    def geometry(self, subtype="triangle"):
        return self._new("vsrNewGeometry", GEOMETRY, subtype)

    def material(self, subtype):
        return self._new("vsrNewMaterial", MATERIAL, subtype)

    def light(self, subtype="directional"):
        return self._new("vsrNewLight", LIGHT, subtype)

    def surface(self):
        return self._new("vsrNewSurface", SURFACE)

    def group(self):
        return self._new("vsrNewGroup", GROUP)

    def instance(self, subtype="transform"):
        return self._new("vsrNewInstance", INSTANCE, subtype)

    def world(self):
        return self._new("vsrNewWorld", WORLD)

    def camera(self, subtype):
        return self._new("vsrNewCamera", CAMERA, subtype)

    def renderer(self, subtype):
        return self._new("vsrNewRenderer", RENDERER, subtype)

    def sampler(self, subtype):
        return self._new("vsrNewSampler", SAMPLER, subtype)

    def frame(self):
        return self._new("vsrNewFrame", FRAME)

    # -- parameters --------------------------------------------------------
    def set(self, obj, name, value, type_=None):
        """Set a parameter; the type is inferred unless given."""
        if isinstance(value, Obj):
            h = ctypes.c_void_p(value.ptr)
            return self.lib.vsrSetParameter(self.handle, obj.ptr, name.encode(), type_ or value.kind,
                                            ctypes.byref(h))
        if isinstance(value, str):
            s = ctypes.c_char_p(value.encode())
            self._keep.append(s)
            return self.lib.vsrSetParameter(self.handle, obj.ptr, name.encode(), STRING,
                                            ctypes.cast(s, ctypes.c_void_p))
        if type_ is None:
            if isinstance(value, bool):
                type_ = BOOL
            elif isinstance(value, (int, np.integer)):
                type_ = INT32
            elif isinstance(value, (float, np.floating)):
                type_ = FLOAT32
            else:
                n = len(value)
                type_ = {2: FLOAT32_VEC2, 3: FLOAT32_VEC3, 4: FLOAT32_VEC4, 16: FLOAT32_MAT4,
                         12: FLOAT32_MAT3x4}[n]
        if type_ in (BOOL, INT32, UINT32, DATA_TYPE):
            buf = np.array([int(value)], dtype=np.int64).astype(np.uint32 if type_ == UINT32 else np.int32)
        elif type_ in (UINT32_VEC2, UINT32_VEC3, UINT32_VEC4):
            buf = np.asarray(value, dtype=np.uint32)
        elif type_ == INT32_VEC2:
            buf = np.asarray(value, dtype=np.int32)
        elif type_ in (FLOAT64, FLOAT64_BOX1):
            buf = np.asarray(value, dtype=np.float64).reshape(-1)
        else:
            buf = np.asarray(value, dtype=np.float32).reshape(-1)
        buf = np.ascontiguousarray(buf)
        return self.lib.vsrSetParameter(self.handle, obj.ptr, name.encode(), type_, buf.ctypes.data)

    def unset(self, obj, name):
        return self.lib.vsrUnsetParameter(self.handle, obj.ptr, name.encode())

    def commit(self, obj):
        return self.lib.vsrCommitParameters(self.handle, obj.ptr)

    def release(self, obj):
        return self.lib.vsrRelease(self.handle, obj.ptr)

    # -- frames ------------------------------------------------------------
    def render(self, frame):
        return self.lib.vsrRenderFrame(self.handle, frame.ptr)

    def denoise_input(self, frame, x_ptr):
        """The denoiser's input image of a frame (vsrDenoiserFrameInput) into
        a device buffer of W8 x H8 x 16 bf16."""
        rc = self.lib.vsrDenoiserFrameInput(self.handle, frame.ptr, x_ptr)
        if rc:
            raise RuntimeError(f"vsrDenoiserFrameInput failed ({rc})")

    def sample_mask(self, frame, mask_ptr):
        """Restrict the frame's path tracer to pixels whose mask byte is
        nonzero (a device pointer, one byte per pixel; None or 0 for all)."""
        rc = self.lib.vsrFrameSampleMask(self.handle, frame.ptr, mask_ptr or None)
        if rc:
            raise RuntimeError(f"vsrFrameSampleMask failed ({rc})")

    def render_batch(self, frames):
        """Render several frames as one batch (vsrRenderFrames)."""
        arr = (_P * len(frames))(*[f.ptr for f in frames])
        return self.lib.vsrRenderFrames(self.handle, arr, len(frames))

    def wait(self, frame):
        return self.lib.vsrFrameReady(self.handle, frame.ptr, WAIT)

    def get_float(self, obj, name):
        v = ctypes.c_float(0)
        ok = self.lib.vsrGetProperty(self.handle, obj.ptr, name.encode(), FLOAT32, ctypes.byref(v), 4, WAIT)
        return v.value if ok else None

    def get_uint(self, obj, name):
        v = ctypes.c_uint32(0)
        ok = self.lib.vsrGetProperty(self.handle, obj.ptr, name.encode(), UINT32, ctypes.byref(v), 4, WAIT)
        return v.value if ok else None

    def get_int(self, obj, name):
        v = ctypes.c_int32(0)
        ok = self.lib.vsrGetProperty(self.handle, obj.ptr, name.encode(), INT32, ctypes.byref(v), 4, WAIT)
        return v.value if ok else None

    def get_u64(self, obj, name, count=1):
        v = (ctypes.c_uint64 * count)()
        ok = self.lib.vsrGetProperty(self.handle, obj.ptr, name.encode(), UINT64, v, 8 * count, WAIT)
        return list(v) if ok else None

    def map(self, frame, channel):
        """Map a channel and return a numpy copy shaped (H, W[, C])."""
        w, h, t = ctypes.c_uint32(0), ctypes.c_uint32(0), ctypes.c_int(0)
        p = self.lib.vsrMapFrame(self.handle, frame.ptr, channel.encode(), ctypes.byref(w),
                                 ctypes.byref(h), ctypes.byref(t))
        if not p:
            raise RuntimeError(f"channel {channel} not available")
        W, H, T = w.value, h.value, t.value
        if T == FLOAT32_VEC4:
            n, dt = 4, np.float32
        elif T == FLOAT32_VEC3:
            n, dt = 3, np.float32
        elif T == FLOAT32:
            n, dt = 1, np.float32
        else:
            n, dt = 1, np.uint32
        count = W * H * n
        buf = (ctypes.c_char * (count * np.dtype(dt).itemsize)).from_address(p)
        arr = np.frombuffer(buf, dtype=dt, count=count).copy()
        self.lib.vsrUnmapFrame(self.handle, frame.ptr, channel.encode())
        return arr.reshape((H, W, n)) if n > 1 else arr.reshape((H, W))

    def map_raw(self, frame, channel):
        """Map a channel without the numpy copy; returns (pointer, W, H, type)."""
        w, h, t = ctypes.c_uint32(0), ctypes.c_uint32(0), ctypes.c_int(0)
        p = self.lib.vsrMapFrame(self.handle, frame.ptr, channel.encode(), ctypes.byref(w),
                                 ctypes.byref(h), ctypes.byref(t))
        return p, w.value, h.value, t.value
