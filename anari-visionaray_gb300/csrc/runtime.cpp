// Host runtime of the renderer core: the C ABI of include/vsr.h.
//
// Object model and parameter handling follow the reference ANARI device
// (VisionarayDevice.cpp, the per-object commitParameters()/finalize() of
// camera/, scene/, renderer/, frame/). Differences by design:
//  * all scene data lives in device memory owned by the objects (the
//    reference keeps frame buffers in pinned host memory, DeviceArray.h:50);
//  * one BVH per group over all its triangle surfaces, built on the device at
//    render time when any object reachable from the world changed;
//  * kernels take the scene/camera/renderer/frame records by value, with no
//    per-frame allocations (renderer/Renderer.cpp:19-22 allocates four).
#include "vsr.h"

#include "kernels.h"
#include "vsr_device.h"
#include "denoiser.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <limits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

namespace vsr {

struct Object;

// ------------------------------------------------------------------ device
struct BatchState;
void destroyBatch(BatchState *);

struct Device {
  VSRStatusCallback cb = nullptr;
  BatchState *batch = nullptr;  // batched rendering: plans, tuner, CUDA graph
  std::set<Denoiser *> denoisers;
  const void *cbUser = nullptr;
  int cudaDevice = 0;
  cudaStream_t stream = nullptr;
  uint64_t stamp = 0;
  std::recursive_mutex mtx;
  std::set<Object *> live;

  uint64_t nextStamp() { return ++stamp; }
  void report(Object *src, VSRDataType srcType, VSRSeverity sev, VSRStatus code, const char *fmt,
              ...) {
    if (!cb) return;
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    cb(cbUser, (VSRDevice)this, (VSRObject)src, srcType, sev, code, buf);
  }
};

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t b) {
    release();
    bytes = b;
    if (!b) return cudaSuccess;
    return cudaMalloc(&p, b);
  }
  cudaError_t upload(const void *src, size_t b, cudaStream_t s) {
    cudaError_t e = alloc(b);
    if (e != cudaSuccess || !b) return e;
    return cudaMemcpyAsync(p, src, b, cudaMemcpyHostToDevice, s);
  }
  template <class T> T *as() const { return (T *)p; }
};

static size_t typeSize(VSRDataType t) {
  switch (t) {
  case VSR_BOOL: case VSR_INT32: case VSR_UINT32: case VSR_FLOAT32: case VSR_DATA_TYPE: return 4;
  case VSR_UFIXED8: return 1;
  case VSR_UFIXED8_VEC2: return 2;
  case VSR_UFIXED8_VEC3: return 3;
  case VSR_UFIXED16: return 2;
  case VSR_INT32_VEC2: case VSR_UINT32_VEC2: case VSR_FLOAT32_VEC2: case VSR_FLOAT32_BOX1: return 8;
  case VSR_UINT32_VEC3: case VSR_FLOAT32_VEC3: return 12;
  case VSR_FLOAT32_VEC4: case VSR_UINT32_VEC4: return 16;
  case VSR_UFIXED8_VEC4: case VSR_UFIXED8_RGBA_SRGB: return 4;
  case VSR_FLOAT32_MAT4: return 64;
  case VSR_FLOAT32_MAT3x4: return 48;
  case VSR_FLOAT64_BOX1: return 16;
  case VSR_UINT64: case VSR_FLOAT64: return 8;
  default: return 0;
  }
}

static bool isObjectType(VSRDataType t) {
  return (t >= VSR_OBJECT && t <= VSR_WORLD) || t == VSR_SAMPLER;
}

// ------------------------------------------------------------------ objects
struct Param {
  VSRDataType type = VSR_UNKNOWN;
  std::vector<uint8_t> data;
  Object *obj = nullptr;
  std::string str;
};

void retainObj(Object *o);
void releaseObj(Object *o);

struct Object {
  Device *dev;
  VSRDataType kind;
  std::string subtype;
  int refs = 1;
  std::map<std::string, Param> params;
  uint64_t stamp = 0;  // last commit
  bool valid = false;

  Object(Device *d, VSRDataType k, std::string st) : dev(d), kind(k), subtype(std::move(st)) {
    dev->live.insert(this);
  }
  virtual ~Object() {
    for (auto &kv : params)
      if (kv.second.obj) releaseObj(kv.second.obj);
    dev->live.erase(this);
  }
  // commitParameters + finalize: read committed params into typed state.
  virtual void commit() { valid = true; }
  // largest commit stamp of this object and everything it references
  virtual uint64_t deepStamp() {
    uint64_t s = stamp;
    for (auto &kv : params)
      if (kv.second.obj) s = std::max(s, kv.second.obj->deepStamp());
    return s;
  }

  void warn(const char *fmt, const char *a = "", const char *b = "") {
    dev->report(this, kind, VSR_SEVERITY_WARNING, VSR_ERROR_INVALID_ARGUMENT, fmt, a, b);
  }

  const Param *find(const char *name) const {
    auto it = params.find(name);
    return it == params.end() ? nullptr : &it->second;
  }
  bool getf(const char *name, float &out) const {
    const Param *p = find(name);
    if (!p) return false;
    if (p->type == VSR_FLOAT32) { memcpy(&out, p->data.data(), 4); return true; }
    if (p->type == VSR_FLOAT64) { double d; memcpy(&d, p->data.data(), 8); out = (float)d; return true; }
    return false;
  }
  bool geti(const char *name, int &out) const {
    const Param *p = find(name);
    if (!p) return false;
    if (p->type == VSR_INT32 || p->type == VSR_UINT32) { memcpy(&out, p->data.data(), 4); return true; }
    if (p->type == VSR_BOOL) { uint32_t b; memcpy(&b, p->data.data(), 4); out = b ? 1 : 0; return true; }
    return false;
  }
  bool getv(const char *name, VSRDataType t, float *out) const {
    const Param *p = find(name);
    if (!p || p->type != t) return false;
    memcpy(out, p->data.data(), typeSize(t));
    return true;
  }
  bool getType(const char *name, VSRDataType &out) const {
    const Param *p = find(name);
    if (!p || p->type != VSR_DATA_TYPE) return false;
    int32_t v;
    memcpy(&v, p->data.data(), 4);
    out = (VSRDataType)v;
    return true;
  }
  std::string gets(const char *name, const char *def) const {
    const Param *p = find(name);
    return (p && p->type == VSR_STRING) ? p->str : std::string(def);
  }
  template <class T> T *geto(const char *name, VSRDataType k) const {
    const Param *p = find(name);
    if (!p || !p->obj || p->obj->kind != k) return nullptr;
    return static_cast<T *>(p->obj);
  }
};

void retainObj(Object *o) { o->refs++; }
void releaseObj(Object *o) {
  if (--o->refs == 0) delete o;
}

struct Array : Object {
  VSRDataType elemType;
  uint64_t n[3];
  std::vector<uint8_t> data;
  std::vector<Object *> objs;
  Array(Device *d, VSRDataType kind, VSRDataType et, uint64_t n1, uint64_t n2, uint64_t n3)
      : Object(d, kind, ""), elemType(et) {
    n[0] = n1; n[1] = n2; n[2] = n3;
    stamp = d->nextStamp();
    valid = true;
  }
  ~Array() override {
    for (Object *o : objs)
      if (o) releaseObj(o);
  }
  uint64_t size() const { return n[0] * n[1] * n[2]; }
  template <class T> const T *as() const { return (const T *)data.data(); }
  uint64_t deepStamp() override {
    uint64_t s = stamp;
    for (Object *o : objs)
      if (o) s = std::max(s, o->deepStamp());
    return s;
  }
};

// structuredRegular field, scene/volume/spatial_field/StructuredRegularField.cpp:16-93
struct SpatialField : Object {
  int dims[3] = {0, 0, 0};
  float origin[3] = {0, 0, 0}, spacing[3] = {1, 1, 1};
  DevBuf data;
  // texture copy for hardware trilinear filtering (the reference's CUDA
  // device samples structured fields with tex3D, StructuredRegularField.cpp:42-76)
  cudaArray_t array = nullptr;
  cudaTextureObject_t tex = 0;
  using Object::Object;
  ~SpatialField() override { releaseTexture(); }
  void releaseTexture() {
    if (tex) cudaDestroyTextureObject(tex);
    if (array) cudaFreeArray(array);
    tex = 0;
    array = nullptr;
  }
  bool makeTexture() {
    releaseTexture();
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float>();
    cudaExtent ext = make_cudaExtent((size_t)dims[0], (size_t)dims[1], (size_t)dims[2]);
    if (cudaMalloc3DArray(&array, &ch, ext) != cudaSuccess) return false;
    cudaMemcpy3DParms cp = {};
    cp.srcPtr = make_cudaPitchedPtr(data.p, (size_t)dims[0] * sizeof(float), (size_t)dims[0],
                                    (size_t)dims[1]);
    cp.dstArray = array;
    cp.extent = ext;
    cp.kind = cudaMemcpyDeviceToDevice;
    if (cudaMemcpy3DAsync(&cp, dev->stream) != cudaSuccess) return false;
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = array;
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    return cudaCreateTextureObject(&tex, &rd, &td, nullptr) == cudaSuccess;
  }
  void commit() override {
    valid = false;
    Array *a = geto<Array>("data", VSR_ARRAY3D);
    getv("origin", VSR_FLOAT32_VEC3, origin);
    getv("spacing", VSR_FLOAT32_VEC3, spacing);
    if (!a) {
      warn("missing required parameter 'data' on 'structuredRegular' field");
      return;
    }
    for (int i = 0; i < 3; ++i) dims[i] = (int)a->n[i];
    size_t nv = a->size();
    std::vector<float> host;
    const float *src = nullptr;
    if (a->elemType == VSR_FLOAT32) {
      src = a->as<float>();
    } else if (a->elemType == VSR_UFIXED8) {
      host.resize(nv);
      for (size_t i = 0; i < nv; ++i) host[i] = a->as<uint8_t>()[i] / 255.f;
      src = host.data();
    } else if (a->elemType == VSR_UFIXED16) {
      host.resize(nv);
      for (size_t i = 0; i < nv; ++i) host[i] = a->as<uint16_t>()[i] / 65535.f;
      src = host.data();
    } else {
      warn("unsupported element type of 'data' on 'structuredRegular' field");
      return;
    }
    if (data.upload(src, nv * sizeof(float), dev->stream) != cudaSuccess) {
      dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY, "field upload failed");
      return;
    }
    valid = dims[0] >= 2 && dims[1] >= 2 && dims[2] >= 2;
    if (valid && !makeTexture()) {
      dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY, "field texture creation failed");
      valid = false;
    }
    cudaStreamSynchronize(dev->stream);
  }
  void bounds(float lo[3], float hi[3]) const {
    for (int i = 0; i < 3; ++i) {
      lo[i] = origin[i];
      hi[i] = origin[i] + ((float)dims[i] - 1.f) * spacing[i];
    }
  }
  // the sampling part of a volume record: data, texture, bounds, voxel
  // space (S * (p + T) maps the bounds to [0,1]^3), cellSize = min spacing
  DVolume fieldRecord() const {
    DVolume v{};
    v.tex = tex;
    v.data = data.as<float>();
    for (int a = 0; a < 3; ++a) v.dims[a] = dims[a];
    bounds(v.boundsLo, v.boundsHi);
    float minSp = spacing[0];
    for (int a = 0; a < 3; ++a) {
      v.S[a] = 1.f / (v.boundsHi[a] - v.boundsLo[a]);
      v.T[a] = -v.boundsLo[a];
      minSp = std::min(minSp, spacing[a]);
    }
    v.cellSize = minSp;
    return v;
  }
};

// transferFunction1D volume, scene/volume/TransferFunction1D.cpp:22-165
struct Volume : Object {
  DevBuf tf, majorant;
  std::vector<float> tfHost;
  int tfSize = 0;
  float vr[2] = {0.f, 1.f};
  float unitDistance = 1.f;
  int gdims[3] = {0, 0, 0};
  int brick = 16;
  SpatialField *field = nullptr;
  using Object::Object;
  void commit() override {
    valid = false;
    field = geto<SpatialField>("value", VSR_SPATIAL_FIELD);
    if (!field) field = geto<SpatialField>("field", VSR_SPATIAL_FIELD);
    vr[0] = 0.f; vr[1] = 1.f;
    getv("valueRange", VSR_FLOAT32_BOX1, vr);
    if (const Param *p = find("valueRange"))
      if (p->type == VSR_FLOAT64_BOX1) {
        double d[2];
        memcpy(d, p->data.data(), 16);
        vr[0] = (float)d[0]; vr[1] = (float)d[1];
      }
    float uniformColor[4] = {1, 1, 1, 1};
    Array *colorArr = geto<Array>("color", VSR_ARRAY1D);
    if (!getv("color", VSR_FLOAT32_VEC3, uniformColor)) getv("color", VSR_FLOAT32_VEC4, uniformColor);
    Array *opacityArr = geto<Array>("opacity", VSR_ARRAY1D);
    float opacity = 1.f;
    getf("opacity", opacity);
    float uniformOpacity = opacity * uniformColor[3];
    unitDistance = 1.f;
    getf("unitDistance", unitDistance);
    int b = 16;
    if (geti("majorantBrickSize", b) && b > 0) brick = b;
    if (!field) {
      warn("no spatial field provided to transferFunction1D volume");
      return;
    }
    if (!field->valid) {
      warn("invalid spatial field provided to transferFunction1D volume");
      return;
    }
    int nch = 4;
    if (colorArr && colorArr->elemType == VSR_FLOAT32_VEC3) nch = 3;
    const float *colorData = colorArr ? colorArr->as<float>() : nullptr;
    const float *opacityData = opacityArr ? opacityArr->as<float>() : nullptr;
    size_t numColors = colorArr ? colorArr->size() : 1;
    size_t numOpac = opacityArr ? opacityArr->size() : 1;
    size_t n = std::max(numColors, numOpac);
    tfHost.assign(4 * n, 0.f);
    auto lerp = [](float a, float b2, float t) { return a * (1.f - t) + b2 * t; };
    for (size_t i = 0; i < n; ++i) {
      float colorPos = n > 1 ? (float(i) / (n - 1)) * (numColors - 1) : 0.f;
      float colorFrac = colorPos - floorf(colorPos);
      float c0[4] = {uniformColor[0], uniformColor[1], uniformColor[2], uniformOpacity};
      float c1[4] = {uniformColor[0], uniformColor[1], uniformColor[2], uniformOpacity};
      if (colorData) {
        int i0 = (int)floorf(colorPos), i1 = (int)ceilf(colorPos);
        for (int k = 0; k < nch; ++k) {
          c0[k] = colorData[nch * i0 + k];
          c1[k] = colorData[nch * i1 + k];
        }
      }
      float c[4];
      for (int k = 0; k < 4; ++k) c[k] = lerp(c0[k], c1[k], colorFrac);
      if (opacityData) {
        float ap = n > 1 ? (float(i) / (n - 1)) * (numOpac - 1) : 0.f;
        float af = ap - floorf(ap);
        float a0 = opacityData[(int)floorf(ap)], a1 = opacityData[(int)ceilf(ap)];
        c[3] *= lerp(a0, a1, af);
      }
      for (int k = 0; k < 4; ++k) tfHost[4 * i + k] = c[k];
    }
    tfSize = (int)n;
    if (unitDistance == 0.f) unitDistance = 1.f;
    if (tf.upload(tfHost.data(), tfHost.size() * sizeof(float), dev->stream) != cudaSuccess) return;
    for (int a = 0; a < 3; ++a) gdims[a] = (field->dims[a] + brick - 1) / brick;
    size_t nc = (size_t)gdims[0] * gdims[1] * gdims[2];
    if (majorant.alloc(nc * sizeof(float)) != cudaSuccess) return;
    if (launchBrickMajorants(field->data.as<float>(), field->dims, brick, tf.as<float4>(), tfSize,
                             vr[0], vr[1], majorant.as<float>(), gdims, dev->stream) != cudaSuccess)
      return;
    cudaStreamSynchronize(dev->stream);
    valid = true;
  }
  DVolume record() const {
    DVolume v{};
    v.tex = field->tex;
    v.data = field->data.as<float>();
    v.tf = tf.as<float4>();
    v.majorant = majorant.as<float>();
    for (int a = 0; a < 3; ++a) {
      v.dims[a] = field->dims[a];
      v.gdims[a] = gdims[a];
    }
    v.tfSize = tfSize;
    v.unitDistance = unitDistance;
    field->bounds(v.boundsLo, v.boundsHi);
    float minSp = field->spacing[0];
    for (int a = 0; a < 3; ++a) {
      v.S[a] = 1.f / (v.boundsHi[a] - v.boundsLo[a]);
      v.T[a] = -v.boundsLo[a];
      minSp = std::min(minSp, field->spacing[a]);
    }
    v.cellSize = minSp;
    v.vrMin = vr[0];
    v.vrMax = vr[1];
    v.vrScale = 1.f / (vr[1] - vr[0]);
    return v;
  }
};

// triangle geometry, scene/surface/geometry/Triangle.cpp:46-133
// ------------------------------------------------------ attributes
// toAttribute (scene/surface/common.h:13-37); -1 for "none" or unknown.
static int attributeId(const std::string &n) {
  static const char *names[] = {"attribute0", "attribute1", "attribute2", "attribute3", "color",
                                "worldPosition", "worldNormal", "objectPosition", "objectNormal"};
  for (int i = 0; i < 9; ++i)
    if (n == names[i]) return i;
  return -1;
}
static const char *kAttrNames[5] = {"attribute0", "attribute1", "attribute2", "attribute3",
                                    "color"};

// An attribute array's layout: components and element encoding, from its
// ANARI type (getInfo, common.h:110-262); false for unsupported types.
static bool attrLayout(VSRDataType t, uint16_t &comps, uint16_t &bits) {
  switch (t) {
  case VSR_FLOAT32: comps = 1; bits = 0; return true;
  case VSR_FLOAT32_VEC2: comps = 2; bits = 0; return true;
  case VSR_FLOAT32_VEC3: comps = 3; bits = 0; return true;
  case VSR_FLOAT32_VEC4: comps = 4; bits = 0; return true;
  case VSR_UFIXED8: comps = 1; bits = 8; return true;
  case VSR_UFIXED8_VEC2: comps = 2; bits = 8; return true;
  case VSR_UFIXED8_VEC3: comps = 3; bits = 8; return true;
  case VSR_UFIXED8_VEC4: comps = 4; bits = 8; return true;
  case VSR_UFIXED16: comps = 1; bits = 16; return true;
  default: return false;
  }
}

// A device copy of an attribute array and its record.
struct AttrBuf {
  DevBuf buf;
  DAttr rec{};
  bool load(Array *a, cudaStream_t s) {
    rec = DAttr{};
    if (!a) return true;
    uint16_t comps, bits;
    if (!attrLayout(a->elemType, comps, bits)) return false;
    if (buf.upload(a->data.data(), a->data.size(), s) != cudaSuccess) return false;
    rec.data = buf.p;
    rec.len = (uint32_t)a->size();
    rec.comps = comps;
    rec.fixedBits = bits;
    return true;
  }
};

// A uniform attribute value (FLOAT32 .. FLOAT32_VEC4), the rest of
// (0, 0, 0, 1).
static bool uniformAttr(const Object *o, const char *name, float *v4) {
  const Param *p = o->find(name);
  if (!p) return false;
  float v[4] = {0, 0, 0, 1};
  const int n = p->type == VSR_FLOAT32 ? 1 : p->type == VSR_FLOAT32_VEC2 ? 2
              : p->type == VSR_FLOAT32_VEC3 ? 3 : p->type == VSR_FLOAT32_VEC4 ? 4 : 0;
  if (!n) return false;
  memcpy(v, p->data.data(), 4 * n);
  memcpy(v4, v, sizeof(v));
  return true;
}

// Samplers (scene/surface/material/sampler/*.cpp).
struct Sampler : Object {
  DSampler rec{};
  DevBuf texels;
  AttrBuf prim;
  using Object::Object;
  static int wrapMode(const std::string &m) {
    return m == "repeat" ? WRAP_REPEAT : (m == "mirrorRepeat" ? WRAP_MIRROR : WRAP_CLAMP);
  }
  // imageSamplerUpdateData (sampler/common.h:27-60): every format as RGBA8,
  // missing channels 0 and alpha 1; floats clamped to [0, 1] and scaled by
  // 255 with truncation (the conversion frame/common.h:31-48 uses); sRGB
  // texels decoded to linear.
  bool loadImage(Array *img, int dims) {
    const size_t n = img->size();
    std::vector<uint8_t> rgba(4 * n);
    auto cv = [](float f) { return (uint8_t)(255.f * std::min(std::max(f, 0.f), 1.f)); };
    const VSRDataType t = img->elemType;
    for (size_t i = 0; i < n; ++i) {
      uint8_t *o = &rgba[4 * i];
      o[0] = o[1] = o[2] = 0;
      o[3] = 255;
      if (t == VSR_FLOAT32 || t == VSR_FLOAT32_VEC2 || t == VSR_FLOAT32_VEC3 ||
          t == VSR_FLOAT32_VEC4) {
        const int c = t == VSR_FLOAT32 ? 1 : t == VSR_FLOAT32_VEC2 ? 2 : t == VSR_FLOAT32_VEC3 ? 3 : 4;
        const float *p = img->as<float>() + c * i;
        for (int k = 0; k < c; ++k) o[k] = cv(p[k]);
      } else if (t == VSR_UFIXED8 || t == VSR_UFIXED8_VEC2 || t == VSR_UFIXED8_VEC3 ||
                 t == VSR_UFIXED8_VEC4) {
        const int c = t == VSR_UFIXED8 ? 1 : t == VSR_UFIXED8_VEC2 ? 2 : t == VSR_UFIXED8_VEC3 ? 3 : 4;
        const uint8_t *p = img->as<uint8_t>() + c * i;
        for (int k = 0; k < c; ++k) o[k] = p[k];
      } else if (t == VSR_UFIXED8_RGBA_SRGB) {
        const uint8_t *p = img->as<uint8_t>() + 4 * i;
        for (int k = 0; k < 3; ++k) {
          const float c = p[k] / 255.f;
          const float lin = c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f);
          o[k] = cv(lin);
        }
        o[3] = p[3];
      } else {
        return false;
      }
    }
    for (int a = 0; a < 3; ++a) rec.dims[a] = a < dims ? (int)img->n[a] : 1;
    if (texels.upload(rgba.data(), rgba.size(), dev->stream) != cudaSuccess ||
        cudaStreamSynchronize(dev->stream) != cudaSuccess)
      return false;
    rec.texels = texels.as<uchar4>();
    return true;
  }
  void commit() override {
    valid = false;
    rec = DSampler{};
    const float id4[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    memcpy(rec.inXfm, id4, sizeof(id4));
    memcpy(rec.outXfm, id4, sizeof(id4));
    getv("inTransform", VSR_FLOAT32_MAT4, rec.inXfm);
    getv("outTransform", VSR_FLOAT32_MAT4, rec.outXfm);
    getv("inOffset", VSR_FLOAT32_VEC4, rec.inOffset);
    getv("outOffset", VSR_FLOAT32_VEC4, rec.outOffset);
    rec.inAttribute = attributeId(gets("inAttribute", "attribute0"));
    if (rec.inAttribute < 0) rec.inAttribute = ATTR_NONE;
    rec.linear = gets("filter", "linear") != "nearest";
    rec.wrap[0] = wrapMode(gets("wrapMode1", "clampToEdge"));
    rec.wrap[1] = wrapMode(gets("wrapMode2", "clampToEdge"));
    rec.wrap[2] = wrapMode(gets("wrapMode3", "clampToEdge"));
    if (subtype == "transform") {
      rec.type = SAMP_TRANSFORM;
      valid = true;
      return;
    }
    if (subtype == "primitive") {
      rec.type = SAMP_PRIMITIVE;
      Array *a = geto<Array>("array", VSR_ARRAY1D);
      if (!a || !prim.load(a, dev->stream) || cudaStreamSynchronize(dev->stream) != cudaSuccess) {
        warn("primitive sampler needs an 'array' of a supported type");
        return;
      }
      rec.prim = prim.rec;
      int off = 0;
      geti("offset", off);
      rec.primOffset = (uint32_t)off;
      valid = true;
      return;
    }
    const int dims = subtype == "image1D" ? 1 : subtype == "image2D" ? 2 : 3;
    rec.type = dims == 1 ? SAMP_IMAGE1D : dims == 2 ? SAMP_IMAGE2D : SAMP_IMAGE3D;
    const VSRDataType ak = dims == 1 ? VSR_ARRAY1D : dims == 2 ? VSR_ARRAY2D : VSR_ARRAY3D;
    Array *img = geto<Array>("image", ak);
    if (!img || img->size() == 0) {
      warn("image sampler needs a non-empty 'image'");
      return;
    }
    if (!loadImage(img, dims)) {
      warn("unsupported element type of image sampler 'image'");
      return;
    }
    valid = true;
  }
};

// An analytic primitive's box: a sphere's centre +- radius, a cone's or
// cylinder's end points grown by their radii (get_bounds, DeviceCopyable
// Objects.h:1009-1018), a curve's control points grown by its radius (the
// convex hull holds the curve; the reference's tighter box, :1291-1346,
// can drop the end points of an axis where the cubic term is zero).
static void apBounds(const float *q, uint32_t kind, float *lo, float *hi) {
  for (int a = 0; a < 3; ++a) {
    lo[a] = q[a] - q[3];
    hi[a] = q[a] + q[3];
    if (kind == AP_CONE || kind == AP_CYLINDER) {
      lo[a] = std::min(lo[a], q[4 + a] - q[7]);
      hi[a] = std::max(hi[a], q[4 + a] + q[7]);
    } else if (kind == AP_CURVE) {
      for (int c = 1; c < 4; ++c) {
        lo[a] = std::min(lo[a], q[4 * c + a] - q[3]);
        hi[a] = std::max(hi[a], q[4 * c + a] + q[3]);
      }
    }
  }
}

struct Geometry : Object {
  std::vector<float> v1, e1, e2;  // per triangle, float3 packed
  // spheres, cones, cylinders, curves: kApFloats (16) floats per primitive:
  // (p0, r0, p1, r1, 0...) (a sphere uses (center, radius) and zeros), a
  // curve (w0, r, w1, 0, w2, 0, w3, 0); all of kind apKind
  std::vector<float> prims;
  int apKind = AP_SPHERE;
  // quads: the object-space shading normal of each tessellated triangle
  std::vector<float> quadNormals;
  // iso-surface: the field and its iso values
  SpatialField *isoField = nullptr;
  std::vector<float> isoValues;
  // attributes (Geometry.cpp: vertex.*, faceVarying.*, primitive.*, and
  // the uniform "color" / "attribute0..3"); vertex normals and the index
  // buffer (triangles)
  AttrBuf vattr[5], fvattr[5], pattr[5];
  DevBuf dIndex, dVertexNormal;
  uint32_t numVertexNormals = 0;
  bool fvNormal = false, triangleAttrs = false;
  float uniformV[5][4] = {};
  uint32_t uniformMask = 0;
  using Object::Object;
  bool hasAttributes() const {
    bool any = uniformMask != 0 || dVertexNormal.p != nullptr;
    for (int k = 0; k < 5; ++k) any = any || vattr[k].rec.comps || fvattr[k].rec.comps || pattr[k].rec.comps;
    return any;
  }
  DSurfAttr attrRecord() const {
    DSurfAttr a{};
    a.index = dIndex.as<uint32_t>();
    a.vertexNormal = dVertexNormal.as<float>();
    a.numVertexNormals = numVertexNormals;
    a.fvNormal = fvNormal ? 1 : 0;
    for (int k = 0; k < 5; ++k) {
      a.vertex[k] = vattr[k].rec;
      a.faceVarying[k] = fvattr[k].rec;
      a.primitive[k] = pattr[k].rec;
      memcpy(a.uniform[k], uniformV[k], sizeof(uniformV[k]));
    }
    a.uniformMask = uniformMask;
    a.isTriangle = triangleAttrs ? 1 : 0;
    return a;
  }
  // getAttribute's inputs for a triangle geometry (renderer/common.h:365-
  // 521, getNormals :241-264): per-vertex, face-varying and per-primitive
  // arrays, vertex normals, the index buffer
  bool loadTriangleAttributes(Array *idx, size_t nv, size_t nprim) {
    cudaStream_t st = dev->stream;
    for (int k = 0; k < 5; ++k) {
      const std::string n = kAttrNames[k];
      Array *va = geto<Array>(("vertex." + n).c_str(), VSR_ARRAY1D);
      Array *fa = geto<Array>(("faceVarying." + n).c_str(), VSR_ARRAY1D);
      Array *pa = geto<Array>(("primitive." + n).c_str(), VSR_ARRAY1D);
      if ((va && va->size() < nv) || (fa && fa->size() < 3 * nprim) || (pa && pa->size() < nprim))
        warn("attribute array shorter than its geometry ('%s'); reads past it give (0, 0, 0, 1)",
             n.c_str());
      if (!vattr[k].load(va, st) || !fvattr[k].load(fa, st) || !pattr[k].load(pa, st)) {
        warn("unsupported element type of geometry attribute '%s'", n.c_str());
        return false;
      }
    }
    Array *vn = geto<Array>("vertex.normal", VSR_ARRAY1D);
    if (vn && vn->elemType == VSR_FLOAT32_VEC3) {
      if (dVertexNormal.upload(vn->data.data(), vn->data.size(), st) != cudaSuccess) return false;
      numVertexNormals = (uint32_t)vn->size();
    }
    Array *fn = geto<Array>("faceVarying.normal", VSR_ARRAY1D);
    fvNormal = fn && fn->elemType == VSR_FLOAT32_VEC3 && fn->size() > 0;
    if (idx && dIndex.upload(idx->data.data(), idx->data.size(), st) != cudaSuccess) return false;
    triangleAttrs = true;
    return cudaStreamSynchronize(st) == cudaSuccess;
  }
  void commit() override {
    valid = false;
    v1.clear(); e1.clear(); e2.clear();
    prims.clear();
    quadNormals.clear();
    isoField = nullptr;
    isoValues.clear();
    for (int k = 0; k < 5; ++k) {
      vattr[k].buf.release(); fvattr[k].buf.release(); pattr[k].buf.release();
      vattr[k].rec = fvattr[k].rec = pattr[k].rec = DAttr{};
    }
    dIndex.release();
    dVertexNormal.release();
    numVertexNormals = 0;
    fvNormal = triangleAttrs = false;
    uniformMask = 0;
    for (int k = 0; k < 5; ++k)
      if (uniformAttr(this, kAttrNames[k], uniformV[k])) uniformMask |= 1u << k;
    if (subtype == "quad") {
      commitQuads();
      return;
    }
    if (subtype == "isosurface") {
      commitIso();
      return;
    }
    if (subtype == "sphere") {
      commitSpheres();
      return;
    }
    if (subtype == "cone" || subtype == "cylinder") {
      commitConesCylinders(subtype == "cone");
      return;
    }
    if (subtype == "bezierCurve") {
      commitCurves();
      return;
    }
    Array *pos = geto<Array>("vertex.position", VSR_ARRAY1D);
    Array *idx = geto<Array>("primitive.index", VSR_ARRAY1D);
    if (!pos || pos->elemType != VSR_FLOAT32_VEC3) {
      warn("missing required parameter 'vertex.position' on triangle geometry");
      return;
    }
    const float *P = pos->as<float>();
    size_t nv = pos->size();
    auto add = [&](size_t a, size_t b, size_t c) {
      for (int k = 0; k < 3; ++k) {
        float p1 = P[3 * a + k], p2 = P[3 * b + k], p3 = P[3 * c + k];
        v1.push_back(p1);
        e1.push_back(p2 - p1);
        e2.push_back(p3 - p1);
      }
    };
    if (idx) {
      if (idx->elemType != VSR_UINT32_VEC3) {
        warn("unsupported type for 'primitive.index' on triangle geometry");
        return;
      }
      const uint32_t *I = idx->as<uint32_t>();
      for (size_t i = 0; i < idx->size(); ++i) {
        if (I[3 * i] >= nv || I[3 * i + 1] >= nv || I[3 * i + 2] >= nv) {
          warn("'primitive.index' out of range on triangle geometry");
          return;
        }
        add(I[3 * i], I[3 * i + 1], I[3 * i + 2]);
      }
    } else {
      for (size_t i = 0; i + 2 < nv; i += 3) add(i, i + 1, i + 2);
    }
    if (!loadTriangleAttributes(idx, nv, v1.size() / 3)) return;
    valid = true;
  }
  // ISOSurface.cpp:19-60: a structured field ('field') and its iso values
  // ('isovalue', FLOAT32 array)
  void commitIso() {
    isoField = geto<SpatialField>("field", VSR_SPATIAL_FIELD);
    Array *iv = geto<Array>("isovalue", VSR_ARRAY1D);
    if (!isoField) {
      warn("no spatial field provided to isosurface geometry");
      return;
    }
    if (!iv || iv->size() == 0 || iv->elemType != VSR_FLOAT32) {
      warn("no iso values (FLOAT32 'isovalue') provided to isosurface geometry");
      return;
    }
    if (!isoField->valid) {
      warn("spatial field not valid on isosurface geometry");
      isoField = nullptr;
      return;
    }
    isoValues.assign(iv->as<float>(), iv->as<float>() + iv->size());
    valid = true;
  }
  bool isIso() const { return isoField != nullptr; }

  // Quad.cpp:46-110: each quad (v1..v4, from primitive.index as UINT32_VEC4
  // or consecutive vertices) becomes the triangles (v1, v2-v1, v4-v1) and
  // (v3, v4-v3, v2-v3). Shading normals follow getNormals
  // (renderer/common.h:266-267), which takes the triangle whose position in
  // the geometry's triangle list equals the quad's index: quad q is shaded
  // with the normal of triangle q (of quad q / 2), not of the one hit.
  void commitQuads() {
    Array *pos = geto<Array>("vertex.position", VSR_ARRAY1D);
    Array *idx = geto<Array>("primitive.index", VSR_ARRAY1D);
    if (!pos || pos->elemType != VSR_FLOAT32_VEC3) {
      warn("missing required parameter 'vertex.position' on quad geometry");
      return;
    }
    if (idx && idx->elemType != VSR_UINT32_VEC4) {
      warn("unsupported type for 'primitive.index' on quad geometry");
      return;
    }
    const float *P = pos->as<float>();
    const size_t nv = pos->size();
    const size_t nq = idx ? idx->size() : nv / 4;
    auto tri = [&](size_t a, size_t b, size_t c) {
      for (int k = 0; k < 3; ++k) {
        const float p1 = P[3 * a + k];
        v1.push_back(p1);
        e1.push_back(P[3 * b + k] - p1);
        e2.push_back(P[3 * c + k] - p1);
      }
    };
    for (size_t q = 0; q < nq; ++q) {
      size_t i[4];
      for (int k = 0; k < 4; ++k) i[k] = idx ? idx->as<uint32_t>()[4 * q + k] : 4 * q + k;
      if (i[0] >= nv || i[1] >= nv || i[2] >= nv || i[3] >= nv) {
        warn("'primitive.index' out of range on quad geometry");
        v1.clear(); e1.clear(); e2.clear();
        return;
      }
      tri(i[0], i[1], i[3]);
      tri(i[2], i[3], i[1]);
    }
    const size_t nt = 2 * nq;
    quadNormals.resize(3 * nt);
    for (size_t t = 0; t < nt; ++t) {
      const size_t src = 3 * (t / 2);  // triangle number (quad index), float offset
      const float *a = &e1[src], *b = &e2[src];
      float n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                    a[0] * b[1] - a[1] * b[0]};
      const float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int k = 0; k < 3; ++k) quadNormals[3 * t + k] = n[k] / l;
    }
    valid = true;
  }

  // Sphere.cpp:19-83: centers from vertex.position (through primitive.index
  // when given), radius from vertex.radius indexed by the sphere (not by the
  // vertex), else the global 'radius' (default 0.01)
  void commitSpheres() {
    apKind = AP_SPHERE;
    Array *pos = geto<Array>("vertex.position", VSR_ARRAY1D);
    Array *idx = geto<Array>("primitive.index", VSR_ARRAY1D);
    Array *rad = geto<Array>("vertex.radius", VSR_ARRAY1D);
    if (!pos || pos->elemType != VSR_FLOAT32_VEC3) {
      warn("missing required parameter 'vertex.position' on sphere geometry");
      return;
    }
    if (idx && idx->elemType != VSR_UINT32) {
      warn("unsupported type for 'primitive.index' on sphere geometry");
      return;
    }
    if (rad && rad->elemType != VSR_FLOAT32) {
      warn("unsupported type for 'vertex.radius' on sphere geometry");
      return;
    }
    float globalRadius = 0.01f;
    getf("radius", globalRadius);
    const float *P = pos->as<float>();
    const size_t nv = pos->size();
    const size_t n = idx ? idx->size() : nv;
    if (rad && rad->size() < n) {
      warn("'vertex.radius' shorter than the number of spheres");
      return;
    }
    prims.assign(kApFloats * n, 0.f);
    for (size_t i = 0; i < n; ++i) {
      const size_t v = idx ? idx->as<uint32_t>()[i] : i;
      if (v >= nv) {
        warn("'primitive.index' out of range on sphere geometry");
        prims.clear();
        return;
      }
      for (int k = 0; k < 3; ++k) prims[kApFloats * i + k] = P[3 * v + k];
      prims[kApFloats * i + 3] = rad ? rad->as<float>()[i] : globalRadius;
    }
    valid = true;
  }

  // BezierCurve.cpp:19-100: cubic segments from vertex.position; with
  // primitive.index (UINT32) entry i starts segments at indices[i], every
  // 3 vertices up to indices[i + 1] (one segment for the last entry), with
  // radius primitive.radius[i]; without it, segments start at vertex 0, 3,
  // 6, ... (consecutive segments share an end vertex) with radius
  // primitive.radius[start / 3]; else 'radius' (default 1). Segments that
  // would read past the vertices are left out.
  void commitCurves() {
    apKind = AP_CURVE;
    Array *pos = geto<Array>("vertex.position", VSR_ARRAY1D);
    Array *idx = geto<Array>("primitive.index", VSR_ARRAY1D);
    Array *rad = geto<Array>("primitive.radius", VSR_ARRAY1D);
    if (!pos || pos->elemType != VSR_FLOAT32_VEC3) {
      warn("missing required parameter 'vertex.position' on bezierCurve geometry");
      return;
    }
    if ((idx && idx->elemType != VSR_UINT32) || (rad && rad->elemType != VSR_FLOAT32)) {
      warn("unsupported type for 'primitive.index' or 'primitive.radius' on bezierCurve geometry");
      return;
    }
    float globalRadius = 1.f;
    getf("radius", globalRadius);
    const float *P = pos->as<float>();
    const size_t nv = pos->size(), nr = rad ? rad->size() : 0;
    bool dropped = false;
    auto add = [&](size_t j, float r) {
      if (j + 3 >= nv) { dropped = true; return; }
      std::vector<float> q(kApFloats, 0.f);
      for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 3; ++a) q[4 * c + a] = P[3 * (j + c) + a];
      q[3] = r;
      prims.insert(prims.end(), q.begin(), q.end());
    };
    if (idx) {
      const uint32_t *I = idx->as<uint32_t>();
      const size_t n = idx->size();
      for (size_t i = 0; i < n; ++i) {
        const size_t first = I[i], last = i == n - 1 ? first + 3 : I[i + 1];
        const float r = rad ? (i < nr ? rad->as<float>()[i] : globalRadius) : globalRadius;
        for (size_t j = first; j < last; j += 3) add(j, r);
      }
    } else if (nv > 3) {
      for (size_t i = 0; i < nv - 3; i += 3)
        add(i, rad ? (i / 3 < nr ? rad->as<float>()[i / 3] : globalRadius) : globalRadius);
    }
    if (dropped) warn("bezierCurve segments past 'vertex.position' are left out");
    valid = !prims.empty();
    if (!valid) warn("bezierCurve geometry has no segments");
  }

  // Cone.cpp:31-82 and Cylinder.cpp:31-82: end points from vertex.position
  // pairs (primitive.index as UINT32_VEC2, else consecutive vertices). A
  // cone's radii are vertex.radius at the two end vertices (required); a
  // cylinder's is primitive.radius indexed by the cylinder, else the global
  // 'radius' (default 1).
  void commitConesCylinders(bool cone) {
    apKind = cone ? AP_CONE : AP_CYLINDER;
    const char *what = cone ? "cone" : "cylinder";
    Array *pos = geto<Array>("vertex.position", VSR_ARRAY1D);
    Array *idx = geto<Array>("primitive.index", VSR_ARRAY1D);
    Array *rad = geto<Array>(cone ? "vertex.radius" : "primitive.radius", VSR_ARRAY1D);
    if (!pos || pos->elemType != VSR_FLOAT32_VEC3) {
      warn("missing required parameter 'vertex.position' on %s geometry", what);
      return;
    }
    if (cone && !rad) {
      warn("missing required parameter 'vertex.radius' on cone geometry");
      return;
    }
    if (idx && idx->elemType != VSR_UINT32_VEC2) {
      warn("unsupported type for 'primitive.index' on %s geometry", what);
      return;
    }
    if (rad && rad->elemType != VSR_FLOAT32) {
      warn("unsupported type for the radius array on %s geometry", what);
      return;
    }
    float globalRadius = 1.f;
    if (!cone) getf("radius", globalRadius);
    const float *P = pos->as<float>();
    const size_t nv = pos->size();
    const size_t n = idx ? idx->size() : nv / 2;
    const size_t nr = rad ? rad->size() : 0;
    prims.assign(kApFloats * n, 0.f);
    for (size_t i = 0; i < n; ++i) {
      const size_t a = idx ? idx->as<uint32_t>()[2 * i] : 2 * i;
      const size_t b = idx ? idx->as<uint32_t>()[2 * i + 1] : 2 * i + 1;
      const size_t ra = cone ? a : i, rb = cone ? b : i;
      if (a >= nv || b >= nv || (rad && (ra >= nr || rb >= nr))) {
        warn("'primitive.index' or the radius array out of range on %s geometry", what);
        prims.clear();
        return;
      }
      for (int k = 0; k < 3; ++k) {
        prims[kApFloats * i + k] = P[3 * a + k];
        prims[kApFloats * i + 4 + k] = P[3 * b + k];
      }
      prims[kApFloats * i + 3] = rad ? rad->as<float>()[ra] : globalRadius;
      prims[kApFloats * i + 7] = rad ? rad->as<float>()[rb] : globalRadius;
    }
    valid = true;
  }
  size_t numTris() const { return v1.size() / 3; }
  size_t numAnalytic() const { return prims.size() / kApFloats; }
};

// matte / physicallyBased, scene/surface/material/{Matte,PBM}.cpp
struct Material : Object {
  DMaterial m{};
  // per MSRC_* slot: a sampler, else an attribute (or SRC_VALUE)
  Sampler *samp[4] = {};
  short attrSrc[4] = {SRC_VALUE, SRC_VALUE, SRC_VALUE, SRC_VALUE};
  using Object::Object;
  // MaterialParam* (Matte.cpp:11-31, PBM.cpp:11-86): a sampler object, else
  // an attribute name, else the value
  void source(const char *name, int slot) {
    samp[slot] = geto<Sampler>(name, VSR_SAMPLER);
    const int a = attributeId(gets(name, "none"));
    attrSrc[slot] = (short)(a >= 0 ? a : SRC_VALUE);
  }
  bool usesAttributes() const {
    for (int k = 0; k < 4; ++k)
      if ((samp[k] && samp[k]->valid) || attrSrc[k] != SRC_VALUE) return true;
    return false;
  }
  void commit() override {
    m = DMaterial{};
    for (int k = 0; k < 4; ++k) {
      samp[k] = nullptr;
      attrSrc[k] = SRC_VALUE;
      m.src[k] = SRC_VALUE;
    }
    source(subtype == "matte" ? "color" : "baseColor", MSRC_COLOR);
    source("opacity", MSRC_OPACITY);
    if (subtype != "matte") {
      source("metallic", MSRC_METALLIC);
      source("roughness", MSRC_ROUGHNESS);
    }
    float c4[4] = {1, 1, 1, 1};
    m.opacity = 1.f;
    getf("opacity", m.opacity);
    std::string am = gets("alphaMode", "opaque");
    m.alphaMode = am == "blend" ? ALPHA_BLEND : (am == "mask" ? ALPHA_MASK : ALPHA_OPAQUE);
    m.alphaCutoff = 0.5f;
    getf("alphaCutoff", m.alphaCutoff);
    if (subtype == "matte") {
      m.type = MAT_MATTE;
      if (!getv("color", VSR_FLOAT32_VEC3, c4)) getv("color", VSR_FLOAT32_VEC4, c4);
    } else {
      m.type = MAT_PBR;
      if (!getv("baseColor", VSR_FLOAT32_VEC3, c4)) getv("baseColor", VSR_FLOAT32_VEC4, c4);
      m.metallic = 1.f; getf("metallic", m.metallic);
      m.roughness = 1.f; getf("roughness", m.roughness);
      m.ior = 1.5f; getf("ior", m.ior);
      m.clearcoat = 0.f; getf("clearcoat", m.clearcoat);
      m.clearcoatRoughness = 0.f; getf("clearcoatRoughness", m.clearcoatRoughness);
      m.transmission = 0.f; getf("transmission", m.transmission);
      float sc[3] = {0, 0, 0};
      getv("sheenColor", VSR_FLOAT32_VEC3, sc);
      for (int k = 0; k < 3; ++k) m.sheenColor[k] = sc[k];
      m.sheenRoughness = 0.f; getf("sheenRoughness", m.sheenRoughness);
    }
    for (int k = 0; k < 3; ++k) m.baseColor[k] = c4[k];
    valid = true;
  }
};

// Lights: Light.cpp:27-35 (color, visible) and the subtypes'
// commitParameters: directional (Directional.cpp:17-28), point (Point.cpp:
// 18-24), spot (Spot.cpp:19-47; the cone cosines are taken of the angles as
// given).
// Inverse of a column-major 3x3 matrix by cofactors over the determinant,
// in double, rounded to float; false (and inv untouched) when singular.
static bool mat3Inverse(const float *m, float *inv) {
  double a[9];
  for (int i = 0; i < 9; ++i) a[i] = m[i];
  const double c00 = a[4] * a[8] - a[7] * a[5], c01 = a[7] * a[2] - a[1] * a[8],
               c02 = a[1] * a[5] - a[4] * a[2];
  const double det = a[0] * c00 + a[3] * c01 + a[6] * c02;
  if (det == 0.0) return false;
  inv[0] = (float)(c00 / det);
  inv[1] = (float)(c01 / det);
  inv[2] = (float)(c02 / det);
  inv[3] = (float)((a[6] * a[5] - a[3] * a[8]) / det);
  inv[4] = (float)((a[0] * a[8] - a[6] * a[2]) / det);
  inv[5] = (float)((a[3] * a[2] - a[0] * a[5]) / det);
  inv[6] = (float)((a[3] * a[7] - a[6] * a[4]) / det);
  inv[7] = (float)((a[6] * a[1] - a[0] * a[7]) / det);
  inv[8] = (float)((a[0] * a[4] - a[3] * a[1]) / det);
  return true;
}

// makeCDF (scene/light/HDRI.cpp:30-68): per texel the largest of r, g, b;
// each row's running sum, its total kept for the row-sum table, then the row
// divided by its last entry (if that is not 0); the row sums scanned and
// normalised the same way. Sums run left to right in float.
static void hdriCdf(const float *rgb, int W, int H, std::vector<float> &rows,
                    std::vector<float> &lastCol) {
  rows.assign((size_t)W * H, 0.f);
  lastCol.assign(H, 0.f);
  std::vector<float> sums(H);
  for (int y = 0; y < H; ++y) {
    float *r = rows.data() + (size_t)y * W;
    for (int x = 0; x < W; ++x) {
      const float *c = rgb + 3 * ((size_t)y * W + x);
      const float lum = std::max(std::max(c[0], c[1]), c[2]);
      r[x] = x == 0 ? lum : r[x - 1] + lum;
    }
    sums[y] = r[W - 1];
    const float back = r[W - 1];
    if (back != 0.f)
      for (int x = 0; x < W; ++x) r[x] /= back;
  }
  for (int y = 0; y < H; ++y) lastCol[y] = y == 0 ? sums[0] : lastCol[y - 1] + sums[y];
  const float back = lastCol[H - 1];
  if (back != 0.f)
    for (int y = 0; y < H; ++y) lastCol[y] /= back;
}

struct Light : Object {
  int type = LIGHT_DIRECTIONAL;
  float direction[3] = {0, 0, -1}, color[3] = {1, 1, 1}, position[3] = {0, 0, 0};
  float edge1[3] = {1, 0, 0}, edge2[3] = {0, 1, 0};  // quad (Quad.cpp:18-27)
  float irradiance = 1.f, angularDiameter = 0.f, intensity = 1.f;
  float cosOuter = -1.f, cosInner = -1.f;
  int visible = 1;
  // hdri (HDRI.cpp:99-164): radiance image, CDFs, scale, frame
  DevBuf hdriTex, hdriRows, hdriLastCol;
  int hdriW = 0, hdriH = 0;
  float scale = 1.f;
  float toWorld[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, toLocal[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  using Object::Object;
  bool commitHdri() {
    float up[3] = {1, 0, 0}, dir[3] = {0, 0, 1};
    getv("up", VSR_FLOAT32_VEC3, up);
    getv("direction", VSR_FLOAT32_VEC3, dir);
    scale = 1.f; getf("scale", scale);
    Array *rad = geto<Array>("radiance", VSR_ARRAY2D);
    if (!rad) {
      warn("missing required parameter 'radiance' on 'hdri' light");
      return false;
    }
    if (rad->elemType != VSR_FLOAT32_VEC3 || rad->n[0] == 0 || rad->n[1] == 0) {
      warn("'radiance' on 'hdri' light must be a non-empty FLOAT32_VEC3 Array2D");
      return false;
    }
    hdriW = (int)rad->n[0];
    hdriH = (int)rad->n[1];
    const float *rgb = rad->as<float>();
    std::vector<float> rows, lastCol;
    hdriCdf(rgb, hdriW, hdriH, rows, lastCol);
    std::vector<float> rgba((size_t)hdriW * hdriH * 4);
    for (size_t i = 0; i < (size_t)hdriW * hdriH; ++i) {
      rgba[4 * i] = rgb[3 * i];
      rgba[4 * i + 1] = rgb[3 * i + 1];
      rgba[4 * i + 2] = rgb[3 * i + 2];
      rgba[4 * i + 3] = 1.f;
    }
    if (hdriTex.upload(rgba.data(), rgba.size() * sizeof(float), dev->stream) != cudaSuccess ||
        hdriRows.upload(rows.data(), rows.size() * sizeof(float), dev->stream) != cudaSuccess ||
        hdriLastCol.upload(lastCol.data(), lastCol.size() * sizeof(float), dev->stream) != cudaSuccess ||
        cudaStreamSynchronize(dev->stream) != cudaSuccess) {
      dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY, "hdri light upload failed");
      return false;
    }
    // toWorld's columns: -up, then normalize(cross(col1, direction)), then
    // normalize(cross(col0, col1)) (HDRI.cpp:146-150), each normalised by
    // division by its length; toLocal its inverse by cofactors
    auto norm = [](float *v) {
      const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      for (int k = 0; k < 3; ++k) v[k] = v[k] / l;
    };
    auto cross = [](const float *a, const float *b, float *o) {
      o[0] = a[1] * b[2] - a[2] * b[1];
      o[1] = a[2] * b[0] - a[0] * b[2];
      o[2] = a[0] * b[1] - a[1] * b[0];
    };
    float c0[3], c1[3] = {up[0], up[1], up[2]}, c2[3];
    norm(c1);
    for (float &v : c1) v = -v;
    cross(c1, dir, c0);
    norm(c0);
    cross(c0, c1, c2);
    norm(c2);
    for (int k = 0; k < 3; ++k) {
      toWorld[k] = c0[k];
      toWorld[3 + k] = c1[k];
      toWorld[6 + k] = c2[k];
    }
    mat3Inverse(toWorld, toLocal);
    return true;
  }
  void commit() override {
    type = subtype == "point"  ? LIGHT_POINT
           : subtype == "spot" ? LIGHT_SPOT
           : subtype == "quad" ? LIGHT_QUAD
           : subtype == "hdri" ? LIGHT_HDRI
                               : LIGHT_DIRECTIONAL;
    color[0] = color[1] = color[2] = 1.f;
    getv("color", VSR_FLOAT32_VEC3, color);
    visible = 1; geti("visible", visible);
    const float maxF = std::numeric_limits<float>::max();
    if (type == LIGHT_HDRI) {
      valid = commitHdri();
      return;
    }
    if (type == LIGHT_DIRECTIONAL) {
      direction[0] = 0; direction[1] = 0; direction[2] = -1;
      getv("direction", VSR_FLOAT32_VEC3, direction);
      float l = std::sqrt(direction[0] * direction[0] + direction[1] * direction[1] +
                          direction[2] * direction[2]);
      for (float &d : direction) d /= l;
      irradiance = 1.f; getf("irradiance", irradiance);
      irradiance = std::max(irradiance, 0.f);
      angularDiameter = 0.f; getf("angularDiameter", angularDiameter);
      angularDiameter = std::max(angularDiameter, 0.f);
    } else if (type == LIGHT_QUAD) {
      // Quad.cpp:18-55: position, edge1, edge2, intensity (clamped to >= 0),
      // side (read and checked; the reference lights both sides)
      position[0] = position[1] = position[2] = 0.f;
      getv("position", VSR_FLOAT32_VEC3, position);
      const float d1[3] = {1, 0, 0}, d2[3] = {0, 1, 0};
      memcpy(edge1, d1, sizeof(edge1));
      memcpy(edge2, d2, sizeof(edge2));
      getv("edge1", VSR_FLOAT32_VEC3, edge1);
      getv("edge2", VSR_FLOAT32_VEC3, edge2);
      intensity = 1.f; getf("intensity", intensity);
      intensity = std::min(std::max(intensity, 0.f), maxF);
      const std::string side = gets("side", "front");
      const float l1 = std::sqrt(edge1[0] * edge1[0] + edge1[1] * edge1[1] + edge1[2] * edge1[2]);
      const float l2 = std::sqrt(edge2[0] * edge2[0] + edge2[1] * edge2[1] + edge2[2] * edge2[2]);
      if (l1 == 0.f || l2 == 0.f) {
        warn("quad light has zero-length edges");
        valid = false;
        return;
      }
      if (side != "front" && side != "back" && side != "both") {
        warn("quad light has invalid side");
        valid = false;
        return;
      }
    } else if (type == LIGHT_POINT) {
      position[0] = 0; position[1] = 0; position[2] = -1;
      getv("position", VSR_FLOAT32_VEC3, position);
      intensity = 1.f; getf("intensity", intensity);
      intensity = std::min(std::max(intensity, 0.f), maxF);
    } else {
      position[0] = position[1] = position[2] = 0.f;
      getv("position", VSR_FLOAT32_VEC3, position);
      direction[0] = 0; direction[1] = 0; direction[2] = -1;
      getv("direction", VSR_FLOAT32_VEC3, direction);
      float opening = (float)M_PI, falloff = 0.1f;
      getf("openingAngle", opening);
      getf("falloffAngle", falloff);
      intensity = 1.f; getf("intensity", intensity);
      intensity = std::min(std::max(intensity, 0.f), maxF);
      const float inner = opening - 2.f * falloff;
      if (inner < 0.f) warn("falloffAngle should be smaller than half of openingAngle");
      cosOuter = std::cos(opening);
      cosInner = std::cos(inner);
    }
    valid = true;
  }
};

struct Surface : Object {
  Geometry *geom = nullptr;
  Material *mat = nullptr;
  using Object::Object;
  void commit() override {
    geom = geto<Geometry>("geometry", VSR_GEOMETRY);
    mat = geto<Material>("material", VSR_MATERIAL);
    valid = geom && mat;
    if (!valid) warn("surface requires 'geometry' and 'material'");
  }
};

template <class T> static std::vector<T *> objectList(Array *a, VSRDataType k) {
  std::vector<T *> out;
  if (!a) return out;
  for (Object *o : a->objs)
    if (o && o->kind == k) out.push_back(static_cast<T *>(o));
  return out;
}

struct Group : Object {
  std::vector<Surface *> surfaces;
  std::vector<Volume *> volumes;
  std::vector<Light *> lights;
  using Object::Object;
  void commit() override {
    surfaces = objectList<Surface>(geto<Array>("surface", VSR_ARRAY1D), VSR_SURFACE);
    volumes = objectList<Volume>(geto<Array>("volume", VSR_ARRAY1D), VSR_VOLUME);
    lights = objectList<Light>(geto<Array>("light", VSR_ARRAY1D), VSR_LIGHT);
    valid = true;
  }
};

struct Instance : Object {
  Group *group = nullptr;
  float xfm[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
  uint32_t userID = ~0u;
  DInstAttr attr{};  // uniform "color" / "attribute0..3" (Instance.cpp)
  using Object::Object;
  void commit() override {
    group = geto<Group>("group", VSR_GROUP);
    attr = DInstAttr{};
    for (int k = 0; k < 5; ++k)
      if (uniformAttr(this, kAttrNames[k], attr.v[k])) attr.mask |= 1u << k;
    float m4[16];
    float i12[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    memcpy(xfm, i12, sizeof(xfm));
    if (getv("transform", VSR_FLOAT32_MAT4, m4)) {
      for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 3; ++r) xfm[3 * c + r] = m4[4 * c + r];
    } else {
      getv("transform", VSR_FLOAT32_MAT3x4, xfm);
    }
    int id;
    if (geti("id", id)) userID = (uint32_t)id;
    valid = group != nullptr;
    if (!valid) warn("instance requires 'group'");
  }
};

// perspective(fovy, aspect, 0.001, 1000) * lookAt(eye, eye + dir, up),
// column-major, evaluated in double from dir and up as given (normalised
// here) and rounded once to float.
static void perspectiveViewProj(const float *eye, const float *dir, const float *up, float fovy,
                                float aspect, float *out) {
  const double n = 0.001, f = 1000.0;
  double F[3] = {dir[0], dir[1], dir[2]}, Up[3] = {up[0], up[1], up[2]};
  const double fl = std::sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
  const double ul = std::sqrt(Up[0] * Up[0] + Up[1] * Up[1] + Up[2] * Up[2]);
  for (int k = 0; k < 3; ++k) {
    F[k] /= fl;
    Up[k] /= ul;
  }
  double S[3] = {F[1] * Up[2] - F[2] * Up[1], F[2] * Up[0] - F[0] * Up[2],
                 F[0] * Up[1] - F[1] * Up[0]};
  const double sl = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
  for (double &v : S) v /= sl;
  const double U[3] = {S[1] * F[2] - S[2] * F[1], S[2] * F[0] - S[0] * F[2],
                       S[0] * F[1] - S[1] * F[0]};
  double V[16] = {0};  // column-major view matrix
  for (int k = 0; k < 3; ++k) {
    V[4 * k + 0] = S[k];
    V[4 * k + 1] = U[k];
    V[4 * k + 2] = -F[k];
  }
  V[12] = -(S[0] * eye[0] + S[1] * eye[1] + S[2] * eye[2]);
  V[13] = -(U[0] * eye[0] + U[1] * eye[1] + U[2] * eye[2]);
  V[14] = F[0] * eye[0] + F[1] * eye[1] + F[2] * eye[2];
  V[15] = 1.0;
  const double t = 1.0 / std::tan(0.5 * (double)fovy);
  double P[16] = {0};
  P[0] = t / aspect;
  P[5] = t;
  P[10] = (f + n) / (n - f);
  P[11] = -1.0;
  P[14] = 2.0 * f * n / (n - f);
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      double acc = 0.0;
      for (int k = 0; k < 4; ++k) acc += P[4 * k + row] * V[4 * col + k];
      out[4 * col + row] = (float)acc;
    }
}

struct Camera : Object {
  DCamera c{};
  // view-projection matrix (column-major) for the TAA motion vectors:
  // perspective cameras as Visionaray's pinhole camera (look-at view,
  // perspective projection with near 0.001 and far 1000, Perspective.cpp:
  // 35-40), matrix cameras proj * view; none for the others
  float mvp[16];
  bool hasMVP = false;
  using Object::Object;
  static void normalize3(float *v) {
    float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int i = 0; i < 3; ++i) v[i] /= l;
  }
  static void cross3(const float *a, const float *b, float *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  }
  static bool inv44(const float *m, float *out) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
      for (int k = 0; k < 4; ++k) {
        a[r][k] = m[k * 4 + r];
        a[r][k + 4] = r == k ? 1.0 : 0.0;
      }
    for (int k = 0; k < 4; ++k) {
      int p = k;
      for (int r = k + 1; r < 4; ++r)
        if (std::fabs(a[r][k]) > std::fabs(a[p][k])) p = r;
      if (a[p][k] == 0.0) return false;
      if (p != k)
        for (int j = 0; j < 8; ++j) std::swap(a[p][j], a[k][j]);
      double d = a[k][k];
      for (int j = 0; j < 8; ++j) a[k][j] /= d;
      for (int r = 0; r < 4; ++r)
        if (r != k) {
          double f = a[r][k];
          for (int j = 0; j < 8; ++j) a[r][j] -= f * a[k][j];
        }
    }
    for (int r = 0; r < 4; ++r)
      for (int k = 0; k < 4; ++k) out[k * 4 + r] = (float)a[r][k + 4];
    return true;
  }
  // Camera::commitParameters camera/Camera.cpp:30-36; Perspective.cpp:13-44;
  // Matrix.cpp:13-27; DCO ortho/omni init DeviceCopyableObjects.h:2506-2575.
  void commit() override {
    c = DCamera{};
    float pos[3] = {0, 0, 0}, dir[3] = {0, 0, 1}, up[3] = {0, 1, 0};
    getv("position", VSR_FLOAT32_VEC3, pos);
    getv("direction", VSR_FLOAT32_VEC3, dir);
    getv("up", VSR_FLOAT32_VEC3, up);
    const float rawDir[3] = {dir[0], dir[1], dir[2]}, rawUp[3] = {up[0], up[1], up[2]};
    normalize3(dir);
    normalize3(up);
    float region[4] = {0, 0, 1, 1};
    float r4[4];
    if (getv("imageRegion", VSR_FLOAT32_VEC4, r4)) memcpy(region, r4, sizeof(region));
    float shutter[2] = {0.5f, 0.5f};
    getv("shutter", VSR_FLOAT32_BOX1, shutter);
    memcpy(c.eye, pos, sizeof(pos));
    memcpy(c.dir, dir, sizeof(dir));
    memcpy(c.region, region, sizeof(region));
    memcpy(c.shutter, shutter, sizeof(shutter));
    float aspect = 1.f;
    getf("aspect", aspect);
    valid = true;
    hasMVP = false;
    if (subtype == "perspective") {
      c.type = CAM_PERSPECTIVE;
      float fovy = 60.f * 3.14159265358979f / 180.f;
      getf("fovy", fovy);
      perspectiveViewProj(pos, rawDir, rawUp, fovy, aspect, mvp);
      hasMVP = true;
      c.lensRadius = 0.f; getf("apertureRadius", c.lensRadius);
      c.focusDistance = 1.f; getf("focusDistance", c.focusDistance);
      float th = std::tan(0.5f * fovy);
      float U[3], V[3];
      cross3(dir, up, U);
      normalize3(U);
      for (float &u : U) u *= th * aspect;
      cross3(U, dir, V);
      normalize3(V);
      for (float &v : V) v *= th;
      memcpy(c.U, U, sizeof(U));
      memcpy(c.V, V, sizeof(V));
      memcpy(c.W, dir, sizeof(dir));
    } else if (subtype == "orthographic" || subtype == "omnidirectional") {
      bool ortho = subtype == "orthographic";
      c.type = ortho ? CAM_ORTHO : CAM_OMNI;
      float height = 1.f;
      getf("height", height);
      float U[3], V[3], W[3];
      cross3(dir, up, U);
      normalize3(U);
      if (ortho) for (float &u : U) u *= height * aspect;
      cross3(U, dir, V);
      normalize3(V);
      if (ortho) for (float &v : V) v *= height;
      for (int i = 0; i < 3; ++i) W[i] = pos[i] - 0.5f * U[i] - 0.5f * V[i];
      memcpy(c.U, U, sizeof(U));
      memcpy(c.V, V, sizeof(V));
      memcpy(c.W, W, sizeof(W));
    } else if (subtype == "matrix") {
      c.type = CAM_MATRIX;
      float proj[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
      float view[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
      getv("proj", VSR_FLOAT32_MAT4, proj);
      getv("view", VSR_FLOAT32_MAT4, view);
      float pv[16];
      for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
          float s = 0.f;
          for (int k = 0; k < 4; ++k) s += proj[k * 4 + row] * view[col * 4 + k];
          pv[col * 4 + row] = s;
        }
      if (!inv44(pv, c.inv)) {
        warn("singular proj*view on matrix camera");
        valid = false;
      }
      memcpy(mvp, pv, sizeof(pv));
      hasMVP = true;
    }
  }
};

struct Renderer : Object {
  DRenderer r{};
  int sampleLimit = 1024;
  bool wavefront = false;
  // TAA: the view-projection matrices of the previous and the current frame
  // rendered with this renderer (rendererState.prevMV/currMV and PR,
  // renderer/common.h:75-78; identity at first, as there)
  float prevMVP[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  float currMVP[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  using Object::Object;
  // Renderer.cpp:34-45, Raycast.cpp:16-20, Pathtrace.cpp:16-28
  void commit() override {
    r = DRenderer{};
    r.type = subtype == "raycast" ? REND_RAYCAST : REND_PATHTRACE;
    float bg[4] = {0, 0, 0, 1};
    getv("background", VSR_FLOAT32_VEC4, bg);
    memcpy(r.bg, bg, sizeof(bg));
    float ac[3] = {1, 1, 1};
    getv("ambientColor", VSR_FLOAT32_VEC3, ac);
    float ar = 0.2f;
    getf("ambientRadiance", ar);
    for (int k = 0; k < 3; ++k) {
      r.ambient[k] = ac[k] * ar;
      r.ambientColor[k] = ac[k];
    }
    r.ambientRadiance = ar;
    std::string mode = gets("mode", "default");
    if (mode != "default")
      dev->report(this, kind, VSR_SEVERITY_WARNING, VSR_ERROR_INVALID_ARGUMENT,
                  "render mode '%s' is not supported; using 'default'", mode.c_str());
    int b = 0;
    // Renderer.cpp:50: volume samples (raycast) and volume scatter events
    // (path tracer) lit along the field gradient
    r.gradientShading = geti("gradientShading", b) && b ? 1 : 0;
    // Pathtrace.cpp:24-25: taa (path tracer only), taaAlpha
    r.taa = r.type == REND_PATHTRACE && geti("taa", b) && b ? 1 : 0;
    r.taaAlpha = 0.3f;
    getf("taaAlpha", r.taaAlpha);
    int v;
    r.maxBounce = 7;
    if (geti("maxBounce", v)) r.maxBounce = std::min(std::max(v, 0), 256);
    r.occlusionDistance = 1e20f;
    getf("ambientOcclusionDistance", r.occlusionDistance);
    r.ambientSamples = 1;
    if (geti("ambientSamples", v)) r.ambientSamples = std::min(std::max(v, 0), 256);
    r.pixelSamples = 1;
    if (r.type == REND_PATHTRACE && geti("pixelSamples", v)) r.pixelSamples = std::min(std::max(v, 1), 256);
    // sample chunks (path tracer): a divisor of pixelSamples, at most 16
    r.sampleChunks = 1;
    if (r.type == REND_PATHTRACE && geti("sampleChunks", v)) {
      int k = std::min(std::max(v, 1), std::min(16, r.pixelSamples));
      while (r.pixelSamples % k) --k;
      if (k != v)
        dev->report(this, kind, VSR_SEVERITY_WARNING, VSR_ERROR_INVALID_ARGUMENT,
                    "sampleChunks %d does not divide pixelSamples %d (or is above 16): using %d",
                    v, r.pixelSamples, k);
      r.sampleChunks = k;
    }
    if (r.taa && r.sampleChunks > 1) {
      dev->report(this, kind, VSR_SEVERITY_WARNING, VSR_ERROR_INVALID_ARGUMENT,
                  "sampleChunks is not used with taa");
      r.sampleChunks = 1;
    }
    sampleLimit = 1024;
    if (geti("sampleLimit", v)) sampleLimit = std::max(v, 1);
    // path tracer execution: one thread per pixel for the whole frame
    // (default, measured faster on the 1M-triangle sphere scene) or wavefront
    // queues; both follow the same per-pixel random stream and give the same
    // image
    wavefront = false;
    if (geti("wavefront", v)) wavefront = v != 0;
    float vsr = 0.5f;
    getf("volumeSamplingRate", vsr);
    r.samplingRateInv = vsr > 0.f ? 1.f / vsr : 0.f;
    // field filtering: "hardware" (texture unit, as the reference's CUDA
    // device) or "exact" (fp32 trilinear, bit-compatible with the CPU
    // device). Default: hardware for raycast, exact for the path tracer,
    // whose delta tracking then follows the CPU device's random stream.
    std::string vf = gets("volumeFilter", r.type == REND_RAYCAST ? "hardware" : "exact");
    r.hwFilter = vf == "hardware" ? 1 : 0;
    r.numClipPlanes = 0;
    if (Array *cp = geto<Array>("clipPlane", VSR_ARRAY1D)) {
      if (cp->elemType != VSR_FLOAT32_VEC4) {
        warn("'clipPlane' must be an array of FLOAT32_VEC4");
      } else {
        size_t n = std::min<size_t>(cp->size(), kMaxClipPlanes);
        if (cp->size() > kMaxClipPlanes) warn("more than 8 clip planes; extra planes ignored");
        for (size_t i = 0; i < n; ++i)
          for (int k = 0; k < 4; ++k) r.clip[i][k] = cp->as<float>()[4 * i + k];
        r.numClipPlanes = (int)n;
      }
    }
    valid = true;
  }
};

// ----------------------------------------------------------------- world
struct GroupGPU {
  DevBuf v1, e1, e2, nodes, nodes4, tris, triSurface, triPrim;
  DevBuf apSrc, apKinds, apNodes, apLeaf, apPrims, apLocal, apSurface, triNormal;
  DevBuf isos, isoValues;
  int numTris = 0, numNodes = 0, width = 2;
  int numAP = 0, apNumNodes = 0;
  float buildMs = 0.f;
};

// world parameter bvhLeafSize when unset: leaves of up to 8 triangles in
// worlds without volumes, one triangle per leaf in worlds with volumes
// (measured on 256 spheres of 1M triangles, surfaces only, 1024x1024 at
// 64 spp: 205.4 -> 200.0 ms per frame with leaves of up to 8; the same
// spheres in a 512^3 volume at 1920x1080, 256 spp: 2862 -> 2975 ms)
constexpr int kDefaultLeafSize = 8;

struct World : Object {
  Group implicitGroup;
  bool implicitUsed = false;
  std::vector<Instance *> instances;
  // device scene
  uint64_t builtStamp = 0;
  std::vector<std::unique_ptr<GroupGPU>> groupsGPU;
  DevBuf dInstances, dGroups, dMaterials, dLights, dVolumes, dGroupVolumes;
  DScene scene{};
  std::vector<DVolume> volsHost;
  float commitMs = 0.f;
  uint64_t bvhNodes = 0, bvhTris = 0;
  bool fastBuild = false;
  int bvhWidth = 2;
  int bvhLeafSize = 0;  // 0: unset (kDefaultLeafSize, or 1 in worlds with volumes)

  World(Device *d, VSRDataType k, std::string st)
      : Object(d, k, st), implicitGroup(d, VSR_GROUP, "") {
    d->live.erase(&implicitGroup);
  }
  void commit() override {
    instances = objectList<Instance>(geto<Array>("instance", VSR_ARRAY1D), VSR_INSTANCE);
    // world-level surfaces/volumes/lights go into a group with an identity
    // instance, as the reference's World does (scene/World.cpp).
    for (auto &kv : implicitGroup.params)
      if (kv.second.obj) releaseObj(kv.second.obj);
    implicitGroup.params.clear();
    const char *names[3] = {"surface", "volume", "light"};
    for (const char *n : names) {
      const Param *p = find(n);
      if (p && p->obj) {
        Param q = *p;
        retainObj(q.obj);
        implicitGroup.params[n] = q;
      }
    }
    implicitGroup.commit();
    // BVH build policy, as the reference's DeviceBVH build flags
    // (PREFER_FAST_BUILD vs a quality build): "quality" (default) or "fast"
    fastBuild = gets("bvhBuild", "quality") == "fast";
    // node width of the traversal BVH: 2 (default, measured faster on the
    // benchmark scene) or 4
    int w = 2;
    geti("bvhWidth", w);
    bvhWidth = w == 4 ? 4 : 2;
    // most triangles per leaf of the 2-wide triangle BVHs (1: one per leaf,
    // as built; up to 32): small subtrees become leaves where the surface-
    // area heuristic expects fewer node visits
    int leaf = 0;
    bvhLeafSize = geti("bvhLeafSize", leaf) ? std::min(std::max(leaf, 1), 32) : 0;
    implicitUsed = !implicitGroup.surfaces.empty() || !implicitGroup.volumes.empty() ||
                   !implicitGroup.lights.empty();
    valid = true;
  }

  // The group's spheres, cones and cylinders get their own BVH2 from the
  // triangle builder: each enters as a triangle spanning its bounding box
  // (get_bounds, DeviceCopyableObjects.h:1009-1018: the end points grown by
  // their radii), then a gather puts the primitives, their group indices
  // and kinds in leaf order.
  bool buildAnalytic(GroupGPU &gg, const std::vector<float> &prims,
                     const std::vector<uint32_t> &kinds, const std::vector<uint32_t> &surf,
                     cudaStream_t s) {
    const int n = (int)surf.size();
    std::vector<float> v1(3 * n), e1(3 * n), e2(3 * n);
    for (int k = 0; k < n; ++k) {
      float blo[3], bhi[3];
      apBounds(&prims[kApFloats * k], kinds[k], blo, bhi);
      for (int a = 0; a < 3; ++a) {
        const float lo = blo[a], hi = bhi[a];
        v1[3 * k + a] = lo;
        e1[3 * k + a] = hi - lo;
        e2[3 * k + a] = a == 1 ? 0.f : hi - lo;
      }
    }
    const size_t fb = (size_t)n * 3 * sizeof(float);
    DevBuf bv1, be1, be2;
    if (bv1.upload(v1.data(), fb, s) || be1.upload(e1.data(), fb, s) ||
        be2.upload(e2.data(), fb, s) ||
        gg.apSrc.upload(prims.data(), (size_t)n * kApStride * sizeof(float4), s) ||
        gg.apKinds.upload(kinds.data(), (size_t)n * sizeof(uint32_t), s) ||
        gg.apSurface.upload(surf.data(), (size_t)n * sizeof(uint32_t), s) ||
        gg.apNodes.alloc((size_t)std::max(n - 1, 1) * 4 * sizeof(float4)) ||
        gg.apLeaf.alloc((size_t)n * 3 * sizeof(float4)) ||
        gg.apPrims.alloc((size_t)n * kApStride * sizeof(float4)) ||
        gg.apLocal.alloc((size_t)n * sizeof(uint32_t))) {
      dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY, "scene upload failed");
      return false;
    }
    BvhBuildStats st{};
    auto build = fastBuild ? buildGroupBVH : buildGroupBVHQuality;
    cudaError_t e = build(bv1.as<float>(), be1.as<float>(), be2.as<float>(), n,
                          gg.apNodes.as<float4>(), gg.apLeaf.as<float4>(), &st, s);
    if (e == cudaSuccess)
      e = launchGatherAnalytic(gg.apLeaf.as<float4>(), gg.apSrc.as<float4>(),
                               gg.apKinds.as<uint32_t>(), n, gg.apPrims.as<float4>(),
                               gg.apLocal.as<uint32_t>(), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA,
                  "sphere / cone / cylinder BVH build failed: %s", cudaGetErrorString(e));
      return false;
    }
    gg.apLeaf.release();
    gg.apSrc.release();
    gg.apKinds.release();
    gg.numAP = n;
    gg.apNumNodes = st.numNodes;
    gg.buildMs += st.buildMs;
    bvhNodes += (uint64_t)st.numNodes;
    return true;
  }

  bool buildScene(uint64_t deep) {
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = dev->stream;
    struct InstRec { Group *g; float xfm[12]; uint32_t userID; DInstAttr attr; };
    std::vector<InstRec> insts;
    if (implicitUsed)
      insts.push_back({&implicitGroup, {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0}, ~0u, DInstAttr{}});
    for (Instance *I : instances) {
      if (!I->valid || !I->group) continue;
      InstRec r;
      r.g = I->group;
      r.attr = I->attr;
      memcpy(r.xfm, I->xfm, sizeof(r.xfm));
      r.userID = I->userID;
      insts.push_back(r);
    }
    std::vector<Group *> groups;
    std::map<Group *, int> gidx;
    for (auto &r : insts)
      if (!gidx.count(r.g)) { gidx[r.g] = (int)groups.size(); groups.push_back(r.g); }

    std::vector<DMaterial> mats;
    std::vector<Geometry *> surfGeom;
    std::vector<Material *> surfMat;
    std::vector<DGroup> dgroups(groups.size());
    std::vector<DVolume> vols;
    std::vector<int> groupVols;
    std::map<Volume *, int> vidx;
    groupsGPU.clear();
    bvhNodes = bvhTris = 0;
    bool allOpaque = true, anySurf = false;
    int numAnalytic = 0, quadGroups = 0, numIso = 0;
    bool anyVolume = false;
    for (Group *g : groups)
      for (Volume *v : g->volumes)
        if (v && v->valid) anyVolume = true;
    const int leafSize = bvhLeafSize ? bvhLeafSize : (anyVolume ? 1 : kDefaultLeafSize);
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      Group *g = groups[gi];
      auto gg = std::make_unique<GroupGPU>();
      std::vector<float> v1, e1, e2;
      std::vector<uint32_t> triSurf, triPrim;
      std::vector<float> apPrims;
      std::vector<uint32_t> apKinds, apSurf;
      std::vector<float> triNormal;  // 4 floats per triangle, w = 1 where set
      bool anyQuad = false;
      std::vector<DIso> isos;
      std::vector<float> isoVals;
      std::vector<size_t> isoValOffset;
      float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
      for (Surface *sf : g->surfaces) {
        if (!sf->valid || !sf->geom->valid || !sf->mat->valid) continue;
        uint32_t sid = (uint32_t)mats.size();
        mats.push_back(sf->mat->m);
        surfGeom.push_back(sf->geom);
        surfMat.push_back(sf->mat);
        if (sf->mat->m.alphaMode != ALPHA_OPAQUE) allOpaque = false;
        Geometry *G = sf->geom;
        if (G->isIso()) {
          DIso di{};
          di.field = G->isoField->fieldRecord();
          di.numValues = (int)G->isoValues.size();
          di.surface = sid;
          di.step = 0.5f * di.field.cellSize;
          isoValOffset.push_back(isoVals.size());
          isoVals.insert(isoVals.end(), G->isoValues.begin(), G->isoValues.end());
          isos.push_back(di);
          for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], di.field.boundsLo[a]);
            hi[a] = std::max(hi[a], di.field.boundsHi[a]);
          }
          continue;
        }
        if (G->numAnalytic()) {
          apPrims.insert(apPrims.end(), G->prims.begin(), G->prims.end());
          for (size_t k = 0; k < G->numAnalytic(); ++k) {
            apSurf.push_back(sid);
            apKinds.push_back((uint32_t)G->apKind);
            float blo[3], bhi[3];
            apBounds(&G->prims[kApFloats * k], (uint32_t)G->apKind, blo, bhi);
            for (int a = 0; a < 3; ++a) {
              lo[a] = std::min(lo[a], blo[a]);
              hi[a] = std::max(hi[a], bhi[a]);
            }
          }
          continue;
        }
        size_t nt = G->numTris();
        triNormal.resize(4 * (triSurf.size() + nt), 0.f);
        if (!G->quadNormals.empty()) {
          anyQuad = true;
          for (size_t t = 0; t < nt; ++t) {
            float *n = &triNormal[4 * (triSurf.size() + t)];
            for (int k = 0; k < 3; ++k) n[k] = G->quadNormals[3 * t + k];
            n[3] = 1.f;
          }
        }
        v1.insert(v1.end(), G->v1.begin(), G->v1.end());
        e1.insert(e1.end(), G->e1.begin(), G->e1.end());
        e2.insert(e2.end(), G->e2.begin(), G->e2.end());
        for (size_t t = 0; t < nt; ++t) {
          triSurf.push_back(sid);
          triPrim.push_back((uint32_t)t);
        }
        for (size_t i = 0; i < G->v1.size(); ++i) {
          int a = (int)(i % 3);
          float p = G->v1[i];
          lo[a] = std::min(lo[a], std::min(p, std::min(p + G->e1[i], p + G->e2[i])));
          hi[a] = std::max(hi[a], std::max(p, std::max(p + G->e1[i], p + G->e2[i])));
        }
      }
      int nt = (int)triSurf.size();
      if (nt >= (1 << 27)) {
        dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_INVALID_ARGUMENT,
                    "group has more than 2^27 triangles");
        return false;
      }
      DGroup dg{};
      dg.volBegin = (int)groupVols.size();
      for (Volume *v : g->volumes) {
        if (!v->valid) continue;
        if (!vidx.count(v)) { vidx[v] = (int)vols.size(); vols.push_back(v->record()); }
        groupVols.push_back(vidx[v]);
      }
      dg.volEnd = (int)groupVols.size();
      if (nt > 0) {
        anySurf = true;
        size_t fb = (size_t)nt * 3 * sizeof(float);
        if (gg->v1.upload(v1.data(), fb, s) || gg->e1.upload(e1.data(), fb, s) ||
            gg->e2.upload(e2.data(), fb, s) ||
            gg->triSurface.upload(triSurf.data(), nt * sizeof(uint32_t), s) ||
            gg->triPrim.upload(triPrim.data(), nt * sizeof(uint32_t), s) ||
            gg->nodes.alloc((size_t)std::max(nt - 1, 1) * 4 * sizeof(float4)) ||
            gg->tris.alloc((size_t)nt * 3 * sizeof(float4))) {
          dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY, "scene upload failed");
          return false;
        }
        BvhBuildStats st{};
        auto build = fastBuild ? buildGroupBVH : buildGroupBVHQuality;
        cudaError_t e = build(gg->v1.as<float>(), gg->e1.as<float>(), gg->e2.as<float>(), nt,
                              gg->nodes.as<float4>(), gg->tris.as<float4>(), &st, s);
        if (e != cudaSuccess) {
          dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA, "BVH build failed: %s",
                      cudaGetErrorString(e));
          return false;
        }
        gg->numTris = nt;
        gg->numNodes = st.numNodes;
        gg->buildMs = st.buildMs;
        gg->width = 2;
        if (bvhWidth == 2 && leafSize > 1) {
          auto tl = std::chrono::steady_clock::now();
          int kept = st.numNodes;
          e = collapseLeaves(gg->nodes.as<float4>(), st.numNodes, gg->tris.as<float4>(), nt,
                             leafSize, &kept, s);
          if (e == cudaSuccess) e = cudaStreamSynchronize(s);
          gg->numNodes = st.numNodes = kept;
          if (e != cudaSuccess) {
            dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA, "BVH leaf collapse failed: %s",
                        cudaGetErrorString(e));
            return false;
          }
          gg->buildMs += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - tl).count();
        }
        if (bvhWidth == 4 && st.numNodes > 0) {
          int n4 = 0;
          auto t4 = std::chrono::steady_clock::now();
          if (gg->nodes4.alloc((size_t)st.numNodes * 8 * sizeof(float4)) != cudaSuccess ||
              (e = collapseBVH4(gg->nodes.as<float4>(), st.numNodes, gg->nodes4.as<float4>(), &n4,
                                s)) != cudaSuccess) {
            dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA, "BVH4 collapse failed: %s",
                        cudaGetErrorString(e));
            return false;
          }
          gg->buildMs += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t4).count();
          gg->nodes.release();
          std::swap(gg->nodes.p, gg->nodes4.p);
          std::swap(gg->nodes.bytes, gg->nodes4.bytes);
          gg->numNodes = n4;
          gg->width = 4;
          st.numNodes = n4;
        }
        // the build inputs are not needed once the leaf-ordered copy exists
        gg->v1.release();
        gg->e1.release();
        gg->e2.release();
        bvhNodes += (uint64_t)st.numNodes;
        bvhTris += (uint64_t)nt;
      }
      const int na = (int)apSurf.size();
      if (na >= (1 << kApKindShift)) {
        dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_INVALID_ARGUMENT,
                    "group has more than 2^28 spheres, cones and cylinders");
        return false;
      }
      if (na > 0 && !buildAnalytic(*gg, apPrims, apKinds, apSurf, s)) return false;
      if (na > 0) anySurf = true;
      if (anyQuad) {
        if (gg->triNormal.upload(triNormal.data(), triNormal.size() * sizeof(float), s)) {
          dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                      "scene upload failed");
          return false;
        }
        ++quadGroups;
      }
      dg.triNormal = anyQuad ? gg->triNormal.as<float4>() : nullptr;
      if (!isos.empty()) {
        if (gg->isoValues.upload(isoVals.data(), isoVals.size() * sizeof(float), s)) {
          dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                      "scene upload failed");
          return false;
        }
        for (size_t k = 0; k < isos.size(); ++k)
          isos[k].values = gg->isoValues.as<float>() + isoValOffset[k];
        if (gg->isos.upload(isos.data(), isos.size() * sizeof(DIso), s)) {
          dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                      "scene upload failed");
          return false;
        }
        anySurf = true;
        numIso += (int)isos.size();
      }
      dg.isos = gg->isos.as<DIso>();
      dg.numIso = (int)isos.size();
      dg.apNodes = gg->apNodes.as<float4>();
      dg.apPrims = gg->apPrims.as<float4>();
      dg.apLocal = gg->apLocal.as<uint32_t>();
      dg.apSurface = gg->apSurface.as<uint32_t>();
      dg.numAP = gg->numAP;
      dg.apNumNodes = gg->apNumNodes;
      numAnalytic += na;
      dg.nodes = gg->nodes.as<float4>();
      dg.tris = gg->tris.as<float4>();
      dg.triSurface = gg->triSurface.as<uint32_t>();
      dg.triPrim = gg->triPrim.as<uint32_t>();
      dg.numTris = nt;
      dg.numNodes = gg->numNodes;
      dg.width = gg->width;
      for (int a = 0; a < 3; ++a) { dg.boundsLo[a] = lo[a]; dg.boundsHi[a] = hi[a]; }
      dgroups[gi] = dg;
      groupsGPU.push_back(std::move(gg));
    }
    std::vector<DInstance> dinst;
    std::vector<DInstAttr> instAttrs;
    std::vector<DLight> lights;
    for (auto &r : insts) {
      DInstance di{};
      // affineInv = inverse(top_left), transInv = -translation,
      // normalXfm = transpose(affineInv)  (scene/Instance.cpp:92-98)
      const float *m = r.xfm;
      float inv[9];
      if (!mat3Inverse(m, inv)) {
        dev->report(this, kind, VSR_SEVERITY_WARNING, VSR_ERROR_INVALID_ARGUMENT,
                    "singular instance transform; instance skipped");
        continue;
      }
      memcpy(di.affineInv, inv, sizeof(inv));
      for (int k = 0; k < 3; ++k) di.transInv[k] = -m[9 + k];
      for (int c = 0; c < 3; ++c)
        for (int rr = 0; rr < 3; ++rr) di.normalXfm[3 * c + rr] = inv[3 * rr + c];
      di.group = gidx[r.g];
      di.userID = r.userID;
      dinst.push_back(di);
      instAttrs.push_back(r.attr);
      for (Light *L : r.g->lights) {
        if (!L->valid) continue;
        // xfmLight (DeviceCopyableObjects.h:2398-2430): positions by the
        // instance's affine transform, directions by its linear part
        auto linear = [&](const float *v, float *o) {
          for (int k = 0; k < 3; ++k) o[k] = m[k] * v[0] + m[3 + k] * v[1] + m[6 + k] * v[2];
        };
        DLight dl{};
        dl.type = L->type;
        dl.visible = L->visible;
        if (L->type == LIGHT_DIRECTIONAL) {
          float d[3];
          linear(L->direction, d);
          float l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
          for (int k = 0; k < 3; ++k) {
            dl.dir[k] = -d[k] / l;
            dl.intensity[k] = L->color[k] * L->irradiance;
          }
          dl.cosHalfAngle = L->angularDiameter > 0.f ? std::cos(0.5f * L->angularDiameter) : 1.f;
        } else {
          linear(L->position, dl.pos);
          for (int k = 0; k < 3; ++k) {
            dl.pos[k] += m[9 + k];
            dl.intensity[k] = L->color[k] * L->intensity;
          }
          if (L->type == LIGHT_SPOT) linear(L->direction, dl.dir);
          dl.cosHalfAngle = 1.f;
          dl.cosOuter = L->cosOuter;
          dl.cosInner = L->cosInner;
          if (L->type == LIGHT_HDRI) {
            // xfmLight leaves HDRI lights untransformed (DeviceCopyableObjects.h
            // :2424-2426)
            dl.hdriTex = L->hdriTex.as<float4>();
            dl.hdriRows = L->hdriRows.as<float>();
            dl.hdriLastCol = L->hdriLastCol.as<float>();
            dl.hdriW = L->hdriW;
            dl.hdriH = L->hdriH;
            dl.scale = L->scale;
            memcpy(dl.toWorld, L->toWorld, sizeof(dl.toWorld));
            memcpy(dl.toLocal, L->toLocal, sizeof(dl.toLocal));
          }
          if (L->type == LIGHT_QUAD) {
            // the quad in world space (xfmLight); the areas and normal of
            // its tessellation (DeviceCopyableObjects.h:2191-2257)
            linear(L->edge1, dl.e1);
            linear(L->edge2, dl.e2);
            float d[3], c1[3], c2[3];
            for (int k = 0; k < 3; ++k) d[k] = dl.e1[k] + dl.e2[k];
            auto cross = [](const float *a, const float *b, float *o) {
              o[0] = a[1] * b[2] - a[2] * b[1];
              o[1] = a[2] * b[0] - a[0] * b[2];
              o[2] = a[0] * b[1] - a[1] * b[0];
            };
            cross(dl.e1, d, c1);
            cross(d, dl.e2, c2);
            const float n1 = std::sqrt(c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2]);
            const float n2 = std::sqrt(c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2]);
            dl.area1 = 0.5f * n1;
            dl.area2 = 0.5f * n2;
            for (int k = 0; k < 3; ++k) dl.normal[k] = c1[k] / n1;
          }
        }
        lights.push_back(dl);
      }
    }
    if (dInstances.upload(dinst.data(), dinst.size() * sizeof(DInstance), s) ||
        dGroups.upload(dgroups.data(), dgroups.size() * sizeof(DGroup), s) ||
        !assembleAttributes(mats, surfGeom, surfMat, instAttrs, s) ||
        dMaterials.upload(mats.data(), mats.size() * sizeof(DMaterial), s) ||
        dLights.upload(lights.data(), lights.size() * sizeof(DLight), s) ||
        dVolumes.upload(vols.data(), vols.size() * sizeof(DVolume), s) ||
        dGroupVolumes.upload(groupVols.data(), groupVols.size() * sizeof(int), s)) {
      dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY, "scene upload failed");
      return false;
    }
    cudaStreamSynchronize(s);
    volsHost = vols;
    scene = DScene{};
    scene.instances = dInstances.as<DInstance>();
    scene.groups = dGroups.as<DGroup>();
    scene.materials = dMaterials.as<DMaterial>();
    scene.lights = dLights.as<DLight>();
    scene.volumes = dVolumes.as<DVolume>();
    scene.groupVolumes = dGroupVolumes.as<int>();
    scene.numInstances = (int)dinst.size();
    scene.numGroups = (int)dgroups.size();
    scene.numLights = (int)lights.size();
    scene.positionalLights = 0;
    scene.areaLights = 0;
    for (const DLight &l : lights) {
      scene.positionalLights += l.type != LIGHT_DIRECTIONAL;
      scene.areaLights += l.type == LIGHT_QUAD || l.type == LIGHT_HDRI;
    }
    scene.numVolumes = (int)vols.size();
    scene.allOpaque = allOpaque ? 1 : 0;
    scene.hasSurfaces = anySurf ? 1 : 0;
    scene.numAnalytic = numAnalytic;
    scene.quadGroups = quadGroups;
    scene.numIso = numIso;
    scene.maxGroupWidth = 2;
    for (const DGroup &g : dgroups) scene.maxGroupWidth = std::max(scene.maxGroupWidth, g.width);
    scene.attributes = useAttributes ? 1 : 0;
    scene.surfAttr = useAttributes ? dSurfAttr.as<DSurfAttr>() : nullptr;
    scene.instAttr = useAttributes ? dInstAttr.as<DInstAttr>() : nullptr;
    scene.samplers = useAttributes ? dSamplers.as<DSampler>() : nullptr;
    builtStamp = deep;
    commitMs = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return true;
  }

  uint64_t deepStamp() override {
    uint64_t s = Object::deepStamp();
    return s;
  }

  // Attribute records per surface and instance, the samplers the materials
  // use, and the materials' parameter sources (a sampler's index in the
  // world's list); nothing when no geometry, material or instance uses
  // attributes, samplers or vertex normals.
  DevBuf dSurfAttr, dInstAttr, dSamplers;
  bool useAttributes = false;
  bool assembleAttributes(std::vector<DMaterial> &mats, const std::vector<Geometry *> &geoms,
                          const std::vector<Material *> &ms,
                          const std::vector<DInstAttr> &instAttrs, cudaStream_t s) {
    useAttributes = false;
    for (size_t i = 0; i < geoms.size(); ++i)
      useAttributes = useAttributes || geoms[i]->hasAttributes() || ms[i]->usesAttributes();
    for (const DInstAttr &a : instAttrs) useAttributes = useAttributes || a.mask != 0;
    if (!useAttributes) return true;
    std::vector<DSurfAttr> sattr;
    std::vector<DSampler> samplers;
    std::map<Sampler *, int> sidx;
    for (size_t i = 0; i < geoms.size(); ++i) {
      sattr.push_back(geoms[i]->attrRecord());
      for (int k = 0; k < 4; ++k) {
        Sampler *sp = ms[i]->samp[k];
        if (sp && sp->valid) {
          if (!sidx.count(sp)) {
            sidx[sp] = (int)samplers.size();
            samplers.push_back(sp->rec);
          }
          mats[i].src[k] = (short)(SRC_SAMPLER + sidx[sp]);
        } else {
          mats[i].src[k] = ms[i]->attrSrc[k];
        }
      }
    }
    return dSurfAttr.upload(sattr.data(), sattr.size() * sizeof(DSurfAttr), s) == cudaSuccess &&
           dInstAttr.upload(instAttrs.data(), instAttrs.size() * sizeof(DInstAttr), s) == cudaSuccess &&
           dSamplers.upload(samplers.data(), samplers.size() * sizeof(DSampler), s) == cudaSuccess;
  }
};

struct FrameObj : Object {
  Renderer *renderer = nullptr;
  Camera *camera = nullptr;
  World *world = nullptr;
  int width = 10, height = 10;
  VSRDataType colorType = VSR_UNKNOWN, depthType = VSR_UNKNOWN, normalType = VSR_UNKNOWN,
              albedoType = VSR_UNKNOWN, varianceType = VSR_UNKNOWN;
  DevBuf color, depth, normal, albedo, accum, errFlags, marchItems, marchGroups, marchCounters,
      unitGroup, segOut, groupDone;
  DevBuf variance, accumSq;                    // optional: variance of the mean (luminance)
  DevBuf denoiseIn, denoiseOut, denoiseCount;  // denoiser scratch, made on first use
  size_t marchPixels = 0;
  unsigned unitCap = 0;
  std::map<std::string, void *> pinned;
  uint32_t *errHost = nullptr;  // pinned: [0] error flags, [1] march work units the last frame needed
  cudaEvent_t evStart = nullptr, evRender = nullptr, evStop = nullptr;
  int accumID = 0;
  uint64_t lastStamp = 0;
  bool rendered = false;
  bool nextReset = true;
  bool countStats = false;
  DevBuf counters;
  unsigned long long countersHost[kStatCounters] = {0};
  // wavefront path-tracer state (allocated on first wavefront render)
  static constexpr int kWaveF4 = 15;
  DevBuf waveF4[kWaveF4], waveMeta, waveHit, waveQueue[2], waveCount;
  size_t wavePixels = 0;
  uint32_t *pinnedCount = nullptr;
  int lastIterations = 0;
  int batchTileW = 0, batchFetch = 0, batchTuned = 0;  // last batched render
  const uint8_t *sampleMask = nullptr;  // caller's device mask (vsrFrameSampleMask)
  DevBuf pixelFrames;  // frames per pixel, made by the first sample mask
  DevBuf chunkOut;     // per-chunk results of chunked path tracing (3 float4 per pixel and chunk)
  // TAA buffers (frame/Frame.cpp:535-540), zeroed when (re)made
  DevBuf taaCurr, taaPrev, taaCurrAlb, taaPrevAlb, motionVec;
  bool ensureTaa() {
    const size_t np = (size_t)width * height;
    if (taaCurr.bytes == np * sizeof(float4)) return true;
    bool ok = taaCurr.alloc(np * sizeof(float4)) == cudaSuccess &&
              taaPrev.alloc(np * sizeof(float4)) == cudaSuccess &&
              taaCurrAlb.alloc(np * 3 * sizeof(float)) == cudaSuccess &&
              taaPrevAlb.alloc(np * 3 * sizeof(float)) == cudaSuccess &&
              motionVec.alloc(np * sizeof(float2)) == cudaSuccess;
    if (ok) {
      for (DevBuf *b : {&taaCurr, &taaPrev, &taaCurrAlb, &taaPrevAlb, &motionVec})
        ok = ok && cudaMemset(b->p, 0, b->bytes) == cudaSuccess;
    }
    if (!ok) taaCurr.release();
    return ok;
  }
  bool ensureChunks(int chunks) {
    const size_t bytes = 3 * (size_t)chunks * width * height * sizeof(float4);
    if (chunkOut.bytes >= bytes) return true;
    return chunkOut.alloc(bytes) == cudaSuccess;
  }

  // scratch of the segmented volume marcher, made on first use: the ray list
  // (48 B per pixel), groups (16 B per 32 pixels) and work units for
  // 64 / VSR_SEG_SAMPLES segments per pixel (1 KiB per unit of 32 segments);
  // rays beyond that are marched whole by the combining warps, one ray at a
  // time per warp, which is slow for long rays. The set-up pass counts the
  // units a frame needs (copied to errHost[1] after the frame): when the
  // last frame needed more (large volumes filling the image), the unit list
  // grows to that count plus a quarter, up to kMaxMarchUnits, so later
  // frames of the same view are marched by segments.
  static constexpr size_t kMaxMarchUnits = size_t(1) << 22;  // 4 GiB of composites
  bool ensureMarch() {
    size_t np = (size_t)width * height;
    const size_t need = errHost[1];
    if (marchPixels == np && need > unitCap && unitCap < kMaxMarchUnits) {
      const size_t cap = std::min(need + need / 4, kMaxMarchUnits);
      if (unitGroup.alloc(cap * sizeof(int)) == cudaSuccess &&
          segOut.alloc(cap * 1024) == cudaSuccess) {
        unitCap = (unsigned)cap;
        return true;
      }
      marchPixels = 0;  // allocation failed: back to the default size below
    }
    if (marchPixels == np) return true;
    const size_t cap = std::max<size_t>(np * 2 / VSR_SEG_SAMPLES, 4096);
    const size_t numGroups = (np + 31) / 32;
    bool ok = marchItems.alloc(np * 48) == cudaSuccess &&
              marchGroups.alloc(numGroups * 16) == cudaSuccess &&
              marchCounters.alloc(4 * sizeof(unsigned)) == cudaSuccess &&
              unitGroup.alloc(cap * sizeof(int)) == cudaSuccess &&
              segOut.alloc(cap * 1024) == cudaSuccess &&
              groupDone.alloc(numGroups * sizeof(unsigned)) == cudaSuccess;
    unitCap = ok ? (unsigned)cap : 0;
    marchPixels = ok ? np : 0;
    return ok;
  }
  MarchScratch march() {
    return MarchScratch{marchItems.p, marchGroups.p, marchCounters.as<unsigned>(),
                        unitGroup.as<int>(), segOut.p, unitCap, groupDone.as<unsigned>()};
  }
  bool ensureWave() {
    size_t np = (size_t)width * height;
    if (wavePixels == np) return true;
    bool ok = true;
    for (auto &b : waveF4) ok = ok && b.alloc(np * sizeof(float4)) == cudaSuccess;
    ok = ok && waveMeta.alloc(np * sizeof(uint4)) == cudaSuccess &&
         waveHit.alloc(np * sizeof(int4)) == cudaSuccess &&
         waveQueue[0].alloc(np * sizeof(uint32_t)) == cudaSuccess &&
         waveQueue[1].alloc(np * sizeof(uint32_t)) == cudaSuccess &&
         waveCount.alloc(4 * sizeof(uint32_t)) == cudaSuccess;
    if (!pinnedCount) ok = ok && cudaMallocHost((void **)&pinnedCount, sizeof(uint32_t)) == cudaSuccess;
    wavePixels = ok ? np : 0;
    return ok;
  }
  DWave wave() {
    DWave w{};
    float4 **f[kWaveF4] = {&w.rayO, &w.rayD, &w.thr, &w.inten, &w.base, &w.shaded, &w.hpo, &w.sn,
                           &w.bdir, &w.bf, &w.acc, &w.pNg, &w.pAlb, &w.cNg, &w.cAlb};
    for (int i = 0; i < kWaveF4; ++i) *f[i] = waveF4[i].as<float4>();
    w.meta = waveMeta.as<uint4>();
    w.hit = waveHit.as<int4>();
    w.queue[0] = waveQueue[0].as<uint32_t>();
    w.queue[1] = waveQueue[1].as<uint32_t>();
    w.count = waveCount.as<uint32_t>();
    return w;
  }

  FrameObj(Device *d, VSRDataType k, std::string st) : Object(d, k, st) {
    cudaEventCreate(&evStart);
    cudaEventCreate(&evRender);
    cudaEventCreate(&evStop);
    cudaMallocHost((void **)&errHost, 2 * sizeof(uint32_t));
    errHost[0] = errHost[1] = 0;
  }
  ~FrameObj() override {
    if (evStart) cudaEventSynchronize(evStop);
    for (auto &kv : pinned) cudaFreeHost(kv.second);
    if (errHost) cudaFreeHost(errHost);
    if (pinnedCount) cudaFreeHost(pinnedCount);
    cudaEventDestroy(evStart);
    cudaEventDestroy(evRender);
    cudaEventDestroy(evStop);
  }
  // frame/Frame.cpp:75-160
  void commit() override {
    renderer = geto<Renderer>("renderer", VSR_RENDERER);
    camera = geto<Camera>("camera", VSR_CAMERA);
    world = geto<World>("world", VSR_WORLD);
    uint32_t sz[2] = {10, 10};
    if (const Param *p = find("size"))
      if (p->type == VSR_UINT32_VEC2 || p->type == VSR_INT32_VEC2) memcpy(sz, p->data.data(), 8);
    colorType = depthType = normalType = albedoType = varianceType = VSR_UNKNOWN;
    getType("channel.color", colorType);
    getType("channel.depth", depthType);
    getType("channel.normal", normalType);
    getType("channel.albedo", albedoType);
    // extension: variance of the accumulated mean's luminance (path tracer)
    getType("channel.variance", varianceType);
    if (varianceType != VSR_UNKNOWN && varianceType != VSR_FLOAT32) {
      warn("unsupported 'channel.variance' type");
      varianceType = VSR_UNKNOWN;
    }
    int cs = 0;
    countStats = geti("collectStatistics", cs) && cs;
    if (!renderer) warn("missing required parameter 'renderer' on frame");
    if (!camera) warn("missing required parameter 'camera' on frame");
    if (!world) warn("missing required parameter 'world' on frame");
    if (colorType != VSR_UNKNOWN && colorType != VSR_FLOAT32_VEC4 && colorType != VSR_UFIXED8_VEC4 &&
        colorType != VSR_UFIXED8_RGBA_SRGB) {
      warn("unsupported 'channel.color' type");
      colorType = VSR_UNKNOWN;
    }
    cudaEventSynchronize(evStop);
    width = (int)sz[0];
    height = (int)sz[1];
    size_t np = (size_t)width * height;
    if (pixelFrames.p && pixelFrames.bytes != np * sizeof(uint32_t)) {
      // a mask of the old size does not fit the new one
      pixelFrames.release();
      sampleMask = nullptr;
    }
    {
      bool ok = accum.alloc(np * sizeof(float4)) == cudaSuccess &&
                depth.alloc(np * sizeof(float)) == cudaSuccess &&
                normal.alloc(np * 3 * sizeof(float)) == cudaSuccess &&
                albedo.alloc(np * 3 * sizeof(float)) == cudaSuccess &&
                color.alloc(np * (colorType == VSR_FLOAT32_VEC4 ? 16 : 4)) == cudaSuccess &&
                errFlags.alloc(sizeof(uint32_t)) == cudaSuccess &&
                counters.alloc(kStatCounters * sizeof(unsigned long long)) == cudaSuccess;
      if (varianceType == VSR_FLOAT32) {
        ok = ok && variance.alloc(np * sizeof(float)) == cudaSuccess &&
             accumSq.alloc(np * sizeof(float)) == cudaSuccess;
        if (ok) {
          cudaMemset(variance.p, 0, np * sizeof(float));
          cudaMemset(accumSq.p, 0, np * sizeof(float));
        }
      } else {
        variance.release();
        accumSq.release();
      }
      for (auto &kv : pinned) cudaFreeHost(kv.second);
      pinned.clear();
      if (!ok) {
        dev->report(this, kind, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                    "frame buffer allocation failed");
        valid = false;
        return;
      }
      cudaMemset(errFlags.p, 0, sizeof(uint32_t));
    }
    nextReset = true;
    valid = renderer && renderer->valid && camera && camera->valid && world && world->valid;
  }
  DFrame record() {
    DFrame f{};
    f.width = width;
    f.height = height;
    f.accumID = accumID;
    f.colorType = colorType == VSR_FLOAT32_VEC4 ? COLOR_FLOAT4
                  : colorType == VSR_UFIXED8_VEC4 ? COLOR_UFIXED8
                  : colorType == VSR_UFIXED8_RGBA_SRGB ? COLOR_SRGB8 : COLOR_NONE;
    f.color = color.p;
    f.depth = depth.as<float>();
    f.normal = normal.as<float>();
    f.albedo = albedo.as<float>();
    f.accum = accum.as<float4>();
    f.errorFlags = errFlags.as<uint32_t>();
    f.counters = countStats ? counters.as<unsigned long long>() : nullptr;
    f.accumSq = accumSq.as<float>();
    f.variance = variance.as<float>();
    f.pixelSamples = renderer ? renderer->r.pixelSamples : 1;
    f.sampleMask = sampleMask;
    f.pixelFrames = pixelFrames.as<uint32_t>();
    f.chunkOut = chunkOut.as<float4>();
    f.taaCurr = taaCurr.as<float4>();
    f.taaPrev = taaPrev.as<float4>();
    f.taaCurrAlbedo = taaCurrAlb.as<float>();
    f.taaPrevAlbedo = taaPrevAlb.as<float>();
    f.motionVec = motionVec.as<float2>();
    return f;
  }
};

Object *asObj(VSRObject o) { return reinterpret_cast<Object *>(o); }
Device *asDev(VSRDevice d) { return reinterpret_cast<Device *>(d); }

VSRStatus renderFrame(Device *dev, FrameObj *F) {
  cudaStream_t s = dev->stream;
  cudaEventSynchronize(F->evStop);
  if (!F->valid) {
    dev->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_INCOMPLETE,
                "skipping render of incomplete frame object");
    return VSR_ERROR_INCOMPLETE;
  }
  World *W = F->world;
  uint64_t deep = W->deepStamp();
  if (deep > W->builtStamp) {
    if (!W->buildScene(deep)) return VSR_ERROR_CUDA;
  }
  // checkAccumulationReset, frame/Frame.cpp:499-513
  uint64_t stampAll = std::max({deep, F->stamp, F->renderer->deepStamp(), F->camera->stamp});
  if (stampAll > F->lastStamp) {
    F->lastStamp = stampAll;
    F->nextReset = true;
  }
  // host-side preparation first, so that the timed region between the
  // frame's events holds GPU work only
  const bool reset = F->nextReset;
  if (reset) {
    F->accumID = 0;
    F->nextReset = false;
  }
  const bool doRender = F->accumID < F->renderer->sampleLimit;
  const DRenderer &R = F->renderer->r;
  // the wavefront kernels have neither gradient shading nor spheres, cones,
  // cylinders, quads and iso-surfaces: the
  // megakernel takes such frames
  const bool wave = F->renderer->wavefront && !R.gradientShading && !W->scene.numAnalytic &&
                    !W->scene.quadGroups && !W->scene.numIso && R.sampleChunks <= 1 && !R.taa &&
                    !W->scene.areaLights && !W->scene.attributes;
  int stage = 0;
  MarchScratch ms{};
  bool segmented = false;
  if (doRender && R.type == REND_RAYCAST) {
    // stage the first volume's TF in shared memory when it fits (64 KB)
    if (!W->volsHost.empty() && W->volsHost[0].tfSize <= 4096) stage = W->volsHost[0].tfSize;
    // the segmented marcher composites unshaded samples; gradient shading
    // takes the per-pixel kernel
    segmented = !W->scene.hasSurfaces && R.pixelSamples == 1 && !R.gradientShading &&
                !W->scene.areaLights && !W->scene.attributes;
    if (segmented && !F->ensureMarch()) {
      dev->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                  "volume marcher scratch allocation failed");
      return VSR_ERROR_OUT_OF_MEMORY;
    }
    if (segmented) ms = F->march();
  } else if (doRender && wave && !F->ensureWave()) {
    dev->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                "wavefront state allocation failed");
    return VSR_ERROR_OUT_OF_MEMORY;
  } else if (doRender && !wave && R.sampleChunks > 1 && !F->ensureChunks(R.sampleChunks)) {
    dev->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                "sample-chunk buffer allocation failed");
    return VSR_ERROR_OUT_OF_MEMORY;
  }
  if (doRender && R.type == REND_PATHTRACE && R.taa && !F->ensureTaa()) {
    dev->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                "TAA buffer allocation failed");
    return VSR_ERROR_OUT_OF_MEMORY;
  }
  DFrame fr = F->record();
  if (doRender && R.type == REND_PATHTRACE) {
    // Frame.cpp:315-334: the current view-projection comes from the camera
    // (perspective and matrix cameras), the previous one is the last
    // frame's; after the render the current one becomes the previous one
    Renderer *rn = F->renderer;
    if (F->camera->hasMVP) memcpy(rn->currMVP, F->camera->mvp, sizeof(rn->currMVP));
    memcpy(fr.prevMVP, rn->prevMVP, sizeof(fr.prevMVP));
    memcpy(fr.currMVP, rn->currMVP, sizeof(fr.currMVP));
    memcpy(rn->prevMVP, rn->currMVP, sizeof(rn->prevMVP));
  }
  cudaEventRecord(F->evStart, s);
  if (reset) {
    launchFrameReset(F->accum.as<float4>(), F->depth.as<float>(), (size_t)F->width * F->height, s);
    if (F->pixelFrames.p) cudaMemsetAsync(F->pixelFrames.p, 0, (size_t)F->width * F->height * 4, s);
  }
  cudaMemsetAsync(F->errFlags.p, 0, sizeof(uint32_t), s);
  if (F->countStats)
    cudaMemsetAsync(F->counters.p, 0, kStatCounters * sizeof(unsigned long long), s);
  cudaEventRecord(F->evRender, s);
  cudaError_t e = cudaSuccess;
  if (doRender) {
    if (R.type == REND_RAYCAST) {
      e = launchRaycast(W->scene, F->camera->c, R, fr, stage, F->countStats,
                        segmented ? &ms : nullptr, s);
    } else if (wave) {
      e = launchPathtraceWavefront(W->scene, F->camera->c, R, fr, F->wave(), F->pinnedCount,
                                   F->countStats, s, &F->lastIterations);
    } else {
      e = launchPathtrace(W->scene, F->camera->c, R, fr, F->countStats, s);
    }
    F->accumID++;
  }
  cudaEventRecord(F->evStop, s);
  cudaMemcpyAsync(F->errHost, F->errFlags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  // the work units this frame needed (the set-up pass's unit counter), read
  // by the next frame's ensureMarch
  if (doRender && segmented)
    cudaMemcpyAsync(F->errHost + 1, ms.counters + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (F->countStats)
    cudaMemcpyAsync(F->countersHost, F->counters.p, kStatCounters * sizeof(unsigned long long),
                    cudaMemcpyDeviceToHost, s);
  F->rendered = true;
  if (e != cudaSuccess) {
    dev->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA, "render launch failed: %s",
                cudaGetErrorString(e));
    return VSR_ERROR_CUDA;
  }
  return VSR_OK;
}

// ------------------------------------------------------------ batching
// Work list of one kind: (job, tile) pairs, jobs ordered by cost per pixel,
// highest first (stable), all tiles of a job together. Longest-first order
// keeps the end of the persistent launch short.
size_t planItems(const uint32_t *w, const uint32_t *h, const float *cost, uint32_t n,
                 uint32_t tileW, std::vector<uint32_t> &out) {
  out.clear();
  if (tileW == 0 || tileW > 32 || 32 % tileW) return 0;
  const uint32_t tileH = 32 / tileW;
  std::vector<uint32_t> order(n);
  for (uint32_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
  for (uint32_t j : order) {
    const uint64_t tiles = (uint64_t)((w[j] + tileW - 1) / tileW) * ((h[j] + tileH - 1) / tileH);
    for (uint64_t t = 0; t < tiles; ++t) {
      out.push_back(j);
      out.push_back((uint32_t)t);
    }
  }
  return out.size() / 2;
}

// Tile shapes and items per fetch the autotuner tries, in this order.
struct BatchConfig {
  int tileW, fetch;
};
static const BatchConfig kBatchConfigs[] = {{8, 1}, {16, 1}, {32, 1}, {4, 1},
                                            {8, 4}, {16, 4}, {4, 4},  {8, 16}};
static const int kNumBatchConfigs = sizeof(kBatchConfigs) / sizeof(kBatchConfigs[0]);

// Online autotuner of one frame set: successive batches of the same set run
// the candidate configurations in turn (every configuration renders the same
// image); once each has been timed the fastest is kept.
struct BatchTuner {
  float ms[kNumBatchConfigs];
  int measured = 0;
  int best = -1;
  BatchTuner() {
    for (float &m : ms) m = -1.f;
  }
  int pick() const { return best >= 0 ? best : measured; }
  void record(int cfg, float t) {
    if (best >= 0 || cfg != measured) return;
    ms[cfg] = t;
    if (++measured == kNumBatchConfigs)
      best = (int)(std::min_element(ms, ms + kNumBatchConfigs) - ms);
  }
};

struct BatchState {
  std::vector<uint64_t> key;  // frame set and its work (sizes, kinds, sample counts)
  int config = -1;            // configuration of the items and the graph below
  DevBuf jobs, items[kJobKinds], counters;
  unsigned numItems[kJobKinds] = {};
  DJob *jobsHost = nullptr;  // pinned staging, read by the graph's copy
  size_t jobsCap = 0;
  int numJobs = 0;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool pending = false;  // a tuning measurement waits in ev0/ev1
  std::vector<uint64_t> pendingKey;
  int pendingConfig = -1;
  std::map<std::vector<uint64_t>, BatchTuner> tuners;
  ~BatchState() {
    if (graph) cudaGraphExecDestroy(graph);
    if (jobsHost) cudaFreeHost(jobsHost);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

void destroyBatch(BatchState *b) { delete b; }

static float jobCostPerPixel(const DRenderer &R, const DScene &S) {
  // path tracing: up to (maxBounce + 1) bounces of radiance + shadow + AO
  // rays per sample; raycast: one ray per sample
  const float spp = (float)std::max(R.pixelSamples, 1);
  const float vol = S.numVolumes > 0 ? 2.f : 1.f;
  if (R.type == REND_RAYCAST) return spp * vol;
  return spp * (float)(R.maxBounce + 1) * (2.f + (float)R.ambientSamples) * vol;
}

VSRStatus renderFrames(Device *dev, FrameObj *const *frames, uint32_t count) {
  cudaStream_t s = dev->stream;
  if (!dev->batch) dev->batch = new BatchState();
  BatchState &B = *dev->batch;
  if (!B.ev0 && (cudaEventCreate(&B.ev0) != cudaSuccess || cudaEventCreate(&B.ev1) != cudaSuccess))
    return VSR_ERROR_CUDA;
  // the previous batch: its timing feeds the tuner, and the staging buffer
  // is free again once it has run
  cudaEventSynchronize(B.ev1);
  if (B.pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, B.ev0, B.ev1) == cudaSuccess)
      B.tuners[B.pendingKey].record(B.pendingConfig, ms);
    B.pending = false;
  }
  VSRStatus status = VSR_OK;
  std::vector<FrameObj *> batched, single;
  std::vector<DJob> jobs;
  std::vector<uint64_t> key;
  for (uint32_t i = 0; i < count; ++i) {
    FrameObj *F = frames[i];
    cudaEventSynchronize(F->evStop);
    if (!F->valid) {
      dev->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_INCOMPLETE,
                  "skipping render of incomplete frame object");
      status = VSR_ERROR_INCOMPLETE;
      continue;
    }
    // statistics are collected by the per-frame kernels; chunked path tracing
    // and sample masks are per-frame launches too
    if (F->countStats || F->sampleMask ||
        (F->renderer->r.type == REND_PATHTRACE &&
         (F->renderer->r.sampleChunks > 1 || F->renderer->r.taa))) {
      single.push_back(F);
      continue;
    }
    World *W = F->world;
    uint64_t deep = W->deepStamp();
    if (deep > W->builtStamp && !W->buildScene(deep)) {
      status = VSR_ERROR_CUDA;
      continue;
    }
    uint64_t stampAll = std::max({deep, F->stamp, F->renderer->deepStamp(), F->camera->stamp});
    if (stampAll > F->lastStamp) {
      F->lastStamp = stampAll;
      F->nextReset = true;
    }
    DJob j{};
    j.S = W->scene;
    j.C = F->camera->c;
    j.R = F->renderer->r;
    j.reset = F->nextReset ? 1 : 0;
    if (F->nextReset) {
      F->accumID = 0;
      F->nextReset = false;
    }
    j.F = F->record();
    j.kind = j.R.type != REND_RAYCAST ? JOB_PATHTRACE
             : (j.R.gradientShading || j.S.areaLights || j.S.attributes ||
                (j.S.hasSurfaces &&
                 (j.S.positionalLights || j.S.numAnalytic || j.S.quadGroups || j.S.numIso)))
                 ? JOB_RAYCAST_FULL
             : j.S.hasSurfaces        ? JOB_RAYCAST_SURFACES
                                      : JOB_RAYCAST_VOLUME;
    // a frame past its sample limit only clears its error flags
    if (F->accumID >= F->renderer->sampleLimit) j.F.width = j.F.height = 0;
    jobs.push_back(j);
    batched.push_back(F);
    key.insert(key.end(), {(uint64_t)(uintptr_t)F, (uint64_t)j.F.width, (uint64_t)j.F.height,
                           (uint64_t)j.kind, (uint64_t)j.R.pixelSamples, (uint64_t)j.R.maxBounce,
                           (uint64_t)j.S.numVolumes, (uint64_t)j.R.gradientShading,
                           (uint64_t)j.S.positionalLights, (uint64_t)j.S.numAnalytic,
                           (uint64_t)j.S.quadGroups, (uint64_t)j.S.numIso});
  }
  if (!batched.empty()) {
    BatchTuner &tuner = B.tuners[key];
    const int cfg = tuner.pick();
    const BatchConfig C = kBatchConfigs[cfg];
    const int tileH = 32 / C.tileW;
    for (DJob &j : jobs) j.tilesX = (j.F.width + C.tileW - 1) / C.tileW;
    bool ok = true;
    if (key != B.key || cfg != B.config) {
      if (B.graph) cudaGraphExecDestroy(B.graph);
      B.graph = nullptr;
      B.key = key;
      B.config = cfg;
      std::vector<uint32_t> w, h, items;
      std::vector<float> cost;
      for (int k = 0; k < kJobKinds && ok; ++k) {
        w.clear(); h.clear(); cost.clear();
        for (const DJob &j : jobs) {
          const bool mine = j.kind == k;
          w.push_back(mine ? (uint32_t)j.F.width : 0u);
          h.push_back(mine ? (uint32_t)j.F.height : 0u);
          cost.push_back(jobCostPerPixel(j.R, j.S));
        }
        B.numItems[k] = (unsigned)planItems(w.data(), h.data(), cost.data(), (uint32_t)jobs.size(),
                                            (uint32_t)C.tileW, items);
        ok = B.items[k].alloc(std::max<size_t>(items.size(), 2) * sizeof(uint32_t)) == cudaSuccess &&
             (items.empty() || cudaMemcpy(B.items[k].p, items.data(), items.size() * 4,
                                          cudaMemcpyHostToDevice) == cudaSuccess);
      }
      ok = ok && B.counters.alloc(kJobKinds * sizeof(unsigned)) == cudaSuccess;
      if (jobs.size() > B.jobsCap) {
        if (B.jobsHost) cudaFreeHost(B.jobsHost);
        B.jobsHost = nullptr;
        B.jobsCap = 0;
        ok = ok && cudaMallocHost((void **)&B.jobsHost, jobs.size() * sizeof(DJob)) == cudaSuccess &&
             B.jobs.alloc(jobs.size() * sizeof(DJob)) == cudaSuccess;
        if (ok) B.jobsCap = jobs.size();
      }
      B.numJobs = (int)jobs.size();
      if (!ok) {
        B.key.clear();
        dev->report(nullptr, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                    "batch work list allocation failed");
        return VSR_ERROR_OUT_OF_MEMORY;
      }
    }
    (void)tileH;
    memcpy(B.jobsHost, jobs.data(), jobs.size() * sizeof(DJob));
    BatchLaunch L{};
    L.jobs = B.jobs.as<DJob>();
    L.numJobs = B.numJobs;
    for (int k = 0; k < kJobKinds; ++k) {
      L.items[k] = B.items[k].as<uint2>();
      L.numItems[k] = B.numItems[k];
    }
    L.counters = B.counters.as<unsigned>();
    L.tileW = C.tileW;
    L.fetch = C.fetch;
    for (const DJob &j : jobs)
      if (j.kind == JOB_PATHTRACE) {
        if (j.S.numVolumes > 0) L.pathtraceVariant |= 1;
        if (j.S.positionalLights || j.S.numAnalytic || j.S.quadGroups || j.S.numIso ||
            j.S.attributes || (j.S.numVolumes > 0 && j.R.gradientShading))
          L.pathtraceVariant |= 2;
      }
    // one CUDA graph per frame set and configuration: the job records are
    // copied from the pinned staging buffer when the graph runs
    if (!B.graph) {
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
        cudaMemcpyAsync(B.jobs.p, B.jobsHost, jobs.size() * sizeof(DJob), cudaMemcpyHostToDevice, s);
        cudaError_t le = launchBatch(L, s);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (le == cudaSuccess && ce == cudaSuccess && g &&
            cudaGraphInstantiate(&B.graph, g, 0) != cudaSuccess)
          B.graph = nullptr;
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();  // a failed capture falls back to direct launches
    }
    for (FrameObj *F : batched) {
      cudaEventRecord(F->evStart, s);
      cudaEventRecord(F->evRender, s);
    }
    cudaEventRecord(B.ev0, s);
    cudaError_t e;
    if (B.graph) {
      e = cudaGraphLaunch(B.graph, s);
    } else {
      e = cudaMemcpyAsync(B.jobs.p, B.jobsHost, jobs.size() * sizeof(DJob), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = launchBatch(L, s);
    }
    cudaEventRecord(B.ev1, s);
    if (tuner.best < 0) {
      B.pending = true;
      B.pendingKey = key;
      B.pendingConfig = cfg;
    }
    for (size_t i = 0; i < batched.size(); ++i) {
      FrameObj *F = batched[i];
      cudaEventRecord(F->evStop, s);
      cudaMemcpyAsync(F->errHost, F->errFlags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
      if (jobs[i].F.width) F->accumID++;
      F->rendered = true;
      F->batchTileW = C.tileW;
      F->batchFetch = C.fetch;
      F->batchTuned = tuner.best >= 0 ? 1 : 0;
    }
    if (e != cudaSuccess) {
      dev->report(nullptr, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA,
                  "batched render launch failed: %s", cudaGetErrorString(e));
      return VSR_ERROR_CUDA;
    }
  }
  for (FrameObj *F : single) {
    VSRStatus r = renderFrame(dev, F);
    if (r != VSR_OK) status = r;
  }
  return status;
}

} // namespace vsr

using namespace vsr;

static VSRArray newArray(VSRDevice dv, VSRDataType kind, const void *mem, VSRDataType type,
                         uint64_t n1, uint64_t n2, uint64_t n3) {
  Device *d = asDev(dv);
  if (!d) return nullptr;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  size_t es = isObjectType(type) ? sizeof(void *) : typeSize(type);
  if (es == 0) {
    d->report(nullptr, kind, VSR_SEVERITY_ERROR, VSR_ERROR_INVALID_ARGUMENT, "unsupported array element type");
    return nullptr;
  }
  auto *a = new Array(d, kind, type, n1, n2, n3);
  size_t bytes = es * n1 * n2 * n3;
  a->data.resize(bytes);
  if (mem) memcpy(a->data.data(), mem, bytes);
  if (isObjectType(type)) {
    const VSRObject *h = (const VSRObject *)mem;
    for (uint64_t i = 0; i < n1 * n2 * n3; ++i) {
      Object *o = h ? asObj(h[i]) : nullptr;
      if (o) retainObj(o);
      a->objs.push_back(o);
    }
  }
  return (VSRArray)a;
}

template <class T>
static VSRObject newObj(VSRDevice dv, VSRDataType kind, const char *subtype,
                        std::initializer_list<const char *> allowed) {
  Device *d = asDev(dv);
  if (!d) return nullptr;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  std::string st = subtype ? subtype : "";
  if (allowed.size()) {
    bool ok = false;
    for (const char *a : allowed) ok |= st == a;
    if (!ok) {
      d->report(nullptr, kind, VSR_SEVERITY_ERROR, VSR_ERROR_UNKNOWN_SUBTYPE,
                "unknown object subtype '%s'", st.c_str());
      return nullptr;
    }
  }
  if (kind == VSR_RENDERER && st == "default") st = "pathtrace";
  return (VSRObject) new T(d, kind, st);
}

static bool checkObj(Device *d, Object *o) {
  if (!d || !o || !d->live.count(o)) {
    if (d)
      d->report(nullptr, VSR_UNKNOWN, VSR_SEVERITY_ERROR, VSR_ERROR_INVALID_OBJECT,
                "invalid object handle");
    return false;
  }
  return true;
}

static bool channelBuf(FrameObj *F, const std::string &ch, void *&p, size_t &bytes,
                       VSRDataType &t) {
  size_t np = (size_t)F->width * F->height;
  if (ch == "channel.color" && F->colorType != VSR_UNKNOWN) {
    p = F->color.p;
    t = F->colorType;
    bytes = np * (t == VSR_FLOAT32_VEC4 ? 16 : 4);
  } else if (ch == "channel.depth" && F->depthType == VSR_FLOAT32) {
    p = F->depth.p;
    t = VSR_FLOAT32;
    bytes = np * 4;
  } else if (ch == "channel.normal" && F->normalType == VSR_FLOAT32_VEC3) {
    p = F->normal.p;
    t = VSR_FLOAT32_VEC3;
    bytes = np * 12;
  } else if (ch == "channel.albedo" && F->albedoType == VSR_FLOAT32_VEC3) {
    p = F->albedo.p;
    t = VSR_FLOAT32_VEC3;
    bytes = np * 12;
  } else if (ch == "channel.variance" && F->varianceType == VSR_FLOAT32) {
    p = F->variance.p;
    t = VSR_FLOAT32;
    bytes = np * 4;
  } else {
    return false;
  }
  return true;
}

// ---------------------------------------------------------------- C ABI
extern "C" {

VSRDevice vsrNewDevice(const char *subtype, VSRStatusCallback cb, const void *cbUserPtr) {
  if (subtype && strcmp(subtype, "default") != 0) {
    if (cb) cb(cbUserPtr, nullptr, nullptr, VSR_UNKNOWN, VSR_SEVERITY_ERROR, VSR_ERROR_UNKNOWN_SUBTYPE,
               "unknown device subtype");
    return nullptr;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    if (cb) cb(cbUserPtr, nullptr, nullptr, VSR_UNKNOWN, VSR_SEVERITY_FATAL_ERROR, VSR_ERROR_CUDA,
               "no CUDA device available: this renderer core has no CPU fallback");
    return nullptr;
  }
  auto *d = new Device;
  d->cb = cb;
  d->cbUser = cbUserPtr;
  // GPU selection as the reference's VISIONARAY_CUDA_DEVICE
  // (VisionarayDevice.cpp:373-380); default: the current CUDA device.
  cudaGetDevice(&d->cudaDevice);
  if (const char *env = getenv("VISIONARAY_CUDA_DEVICE")) d->cudaDevice = atoi(env);
  if (cudaSetDevice(d->cudaDevice) != cudaSuccess ||
      cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess) {
    if (cb) cb(cbUserPtr, nullptr, nullptr, VSR_UNKNOWN, VSR_SEVERITY_FATAL_ERROR, VSR_ERROR_CUDA,
               "CUDA device initialisation failed");
    delete d;
    return nullptr;
  }
  return (VSRDevice)d;
}

VSRStatus vsrReleaseDevice(VSRDevice dv) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  cudaStreamSynchronize(d->stream);
  destroyBatch(d->batch);
  d->batch = nullptr;
  for (Denoiser *n : d->denoisers) delete n;
  d->denoisers.clear();
  std::vector<Object *> left(d->live.begin(), d->live.end());
  if (!left.empty())
    d->report(nullptr, VSR_UNKNOWN, VSR_SEVERITY_WARNING, VSR_OK,
              "%zu objects still alive at device release", left.size());
  cudaStreamDestroy(d->stream);
  delete d;
  return VSR_OK;
}

VSRArray vsrNewArray1D(VSRDevice d, const void *m, VSRDataType t, uint64_t n1) {
  return newArray(d, VSR_ARRAY1D, m, t, n1, 1, 1);
}
VSRArray vsrNewArray2D(VSRDevice d, const void *m, VSRDataType t, uint64_t n1, uint64_t n2) {
  return newArray(d, VSR_ARRAY2D, m, t, n1, n2, 1);
}
VSRArray vsrNewArray3D(VSRDevice d, const void *m, VSRDataType t, uint64_t n1, uint64_t n2,
                       uint64_t n3) {
  return newArray(d, VSR_ARRAY3D, m, t, n1, n2, n3);
}

VSRObject vsrNewSpatialField(VSRDevice d, const char *s) {
  return newObj<SpatialField>(d, VSR_SPATIAL_FIELD, s, {"structuredRegular"});
}
VSRObject vsrNewVolume(VSRDevice d, const char *s) {
  return newObj<Volume>(d, VSR_VOLUME, s, {"transferFunction1D"});
}
VSRObject vsrNewGeometry(VSRDevice d, const char *s) {
  return newObj<Geometry>(d, VSR_GEOMETRY, s,
                         {"triangle", "quad", "sphere", "cone", "cylinder", "isosurface",
                          "bezierCurve"});
}
VSRObject vsrNewMaterial(VSRDevice d, const char *s) {
  return newObj<Material>(d, VSR_MATERIAL, s, {"matte", "physicallyBased"});
}
VSRObject vsrNewLight(VSRDevice d, const char *s) {
  return newObj<Light>(d, VSR_LIGHT, s, {"directional", "point", "spot", "quad", "hdri"});
}
VSRObject vsrNewSurface(VSRDevice d) { return newObj<Surface>(d, VSR_SURFACE, "", {}); }
VSRObject vsrNewGroup(VSRDevice d) { return newObj<Group>(d, VSR_GROUP, "", {}); }
VSRObject vsrNewInstance(VSRDevice d, const char *s) {
  return newObj<Instance>(d, VSR_INSTANCE, s, {"transform"});
}
VSRObject vsrNewWorld(VSRDevice d) { return newObj<World>(d, VSR_WORLD, "", {}); }
VSRObject vsrNewCamera(VSRDevice d, const char *s) {
  return newObj<Camera>(d, VSR_CAMERA, s, {"perspective", "matrix", "orthographic", "omnidirectional"});
}
VSRObject vsrNewSampler(VSRDevice d, const char *s) {
  return newObj<Sampler>(d, VSR_SAMPLER, s,
                         {"image1D", "image2D", "image3D", "transform", "primitive"});
}
VSRObject vsrNewRenderer(VSRDevice d, const char *s) {
  return newObj<Renderer>(d, VSR_RENDERER, s, {"raycast", "pathtrace", "default"});
}
VSRFrame vsrNewFrame(VSRDevice d) { return newObj<FrameObj>(d, VSR_FRAME, "", {}); }

VSRStatus vsrSetParameter(VSRDevice dv, VSRObject ov, const char *name, VSRDataType type,
                          const void *mem) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(ov);
  if (!checkObj(d, o)) return VSR_ERROR_INVALID_OBJECT;
  if (!name || !mem) return VSR_ERROR_INVALID_ARGUMENT;
  Param p;
  p.type = type;
  if (type == VSR_STRING) {
    p.str = (const char *)mem;
  } else if (isObjectType(type)) {
    Object *ref = asObj(*(const VSRObject *)mem);
    if (ref && !d->live.count(ref)) {
      d->report(o, o->kind, VSR_SEVERITY_ERROR, VSR_ERROR_INVALID_OBJECT,
                "parameter '%s' refers to an invalid object", name);
      return VSR_ERROR_INVALID_OBJECT;
    }
    p.obj = ref;
    if (ref) retainObj(ref);
  } else {
    size_t sz = typeSize(type);
    if (!sz) {
      d->report(o, o->kind, VSR_SEVERITY_ERROR, VSR_ERROR_INVALID_ARGUMENT,
                "parameter '%s' has an unsupported type", name);
      return VSR_ERROR_INVALID_ARGUMENT;
    }
    p.data.resize(sz);
    memcpy(p.data.data(), mem, sz);
  }
  auto it = o->params.find(name);
  if (it != o->params.end() && it->second.obj) releaseObj(it->second.obj);
  o->params[name] = std::move(p);
  return VSR_OK;
}

VSRStatus vsrUnsetParameter(VSRDevice dv, VSRObject ov, const char *name) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(ov);
  if (!checkObj(d, o)) return VSR_ERROR_INVALID_OBJECT;
  auto it = o->params.find(name);
  if (it != o->params.end()) {
    if (it->second.obj) releaseObj(it->second.obj);
    o->params.erase(it);
  }
  return VSR_OK;
}

VSRStatus vsrCommitParameters(VSRDevice dv, VSRObject ov) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(ov);
  if (!checkObj(d, o)) return VSR_ERROR_INVALID_OBJECT;
  o->commit();
  o->stamp = d->nextStamp();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    d->report(o, o->kind, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA, "CUDA error during commit: %s",
              cudaGetErrorString(e));
    return VSR_ERROR_CUDA;
  }
  return o->valid ? VSR_OK : VSR_ERROR_INVALID_ARGUMENT;
}

VSRStatus vsrRelease(VSRDevice dv, VSRObject ov) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(ov);
  if (!checkObj(d, o)) return VSR_ERROR_INVALID_OBJECT;
  releaseObj(o);
  return VSR_OK;
}

VSRStatus vsrRetain(VSRDevice dv, VSRObject ov) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(ov);
  if (!checkObj(d, o)) return VSR_ERROR_INVALID_OBJECT;
  retainObj(o);
  return VSR_OK;
}

int vsrGetProperty(VSRDevice dv, VSRObject ov, const char *name, VSRDataType type, void *mem,
                   uint64_t size, VSRWaitMask mask) {
  Device *d = asDev(dv);
  if (!d || !name || !mem) return 0;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(ov);
  if (!checkObj(d, o)) return 0;
  std::string n = name;
  if (o->kind == VSR_FRAME) {
    FrameObj *F = static_cast<FrameObj *>(o);
    if (mask == VSR_WAIT) cudaEventSynchronize(F->evStop);
    else if (cudaEventQuery(F->evStop) != cudaSuccess) return 0;
    if ((n == "duration" || n == "duration.render") && type == VSR_FLOAT32 && size >= 4) {
      if (!F->rendered) return 0;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, n == "duration" ? F->evStart : F->evRender, F->evStop);
      *(float *)mem = ms * 1e-3f;
      return 1;
    }
    if (n == "wavefrontIterations" && type == VSR_INT32 && size >= 4) {
      *(int32_t *)mem = F->lastIterations;
      return 1;
    }
    if ((n == "batch.tileWidth" || n == "batch.fetch" || n == "batch.tuned") &&
        type == VSR_INT32 && size >= 4) {
      *(int32_t *)mem = n == "batch.tileWidth" ? F->batchTileW
                        : n == "batch.fetch"   ? F->batchFetch
                                               : F->batchTuned;
      return 1;
    }
    if (n == "numSamples" && type == VSR_INT32 && size >= 4) {
      *(int32_t *)mem = F->accumID;
      return 1;
    }
    if (n == "errorFlags" && type == VSR_UINT32 && size >= 4) {
      *(uint32_t *)mem = *F->errHost;
      return 1;
    }
    // segmented volume marcher: the work units the last frame needed, and
    // how many the frame's unit list holds now
    if (n == "march.unitsNeeded" && type == VSR_UINT32 && size >= 4) {
      *(uint32_t *)mem = F->errHost[1];
      return 1;
    }
    if (n == "march.unitCapacity" && type == VSR_UINT32 && size >= 4) {
      *(uint32_t *)mem = F->unitCap;
      return 1;
    }
    if (n == "commitDuration" && type == VSR_FLOAT32 && size >= 4 && F->world) {
      *(float *)mem = F->world->commitMs * 1e-3f;
      return 1;
    }
    if (n == "statistics" && type == VSR_UINT64 && size >= 8 * sizeof(uint64_t)) {
      memcpy(mem, F->countersHost, std::min<size_t>(size, kStatCounters * sizeof(uint64_t)));
      return 1;
    }
  }
  if (o->kind == VSR_WORLD) {
    World *W = static_cast<World *>(o);
    if (n == "bvh.nodes" && type == VSR_UINT64 && size >= 8) { *(uint64_t *)mem = W->bvhNodes; return 1; }
    if (n == "bvh.triangles" && type == VSR_UINT64 && size >= 8) { *(uint64_t *)mem = W->bvhTris; return 1; }
    if (n == "bvh.buildDuration" && type == VSR_FLOAT32 && size >= 4) {
      float ms = 0.f;
      for (auto &g : W->groupsGPU) ms += g->buildMs;
      *(float *)mem = ms * 1e-3f;
      return 1;
    }
  }
  return 0;
}

VSRStatus vsrRenderFrames(VSRDevice dv, const VSRFrame *fv, uint32_t count) {
  Device *d = asDev(dv);
  if (!d || (!fv && count)) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  std::vector<FrameObj *> fs;
  for (uint32_t i = 0; i < count; ++i) {
    Object *o = asObj(fv[i]);
    if (!checkObj(d, o) || o->kind != VSR_FRAME) return VSR_ERROR_INVALID_OBJECT;
    FrameObj *F = static_cast<FrameObj *>(o);
    if (std::find(fs.begin(), fs.end(), F) != fs.end()) return VSR_ERROR_INVALID_ARGUMENT;
    fs.push_back(F);
  }
  if (fs.empty()) return VSR_OK;
  return renderFrames(d, fs.data(), (uint32_t)fs.size());
}

static Denoiser *asDenoiser(Device *d, VSRDenoiser n) {
  Denoiser *p = reinterpret_cast<Denoiser *>(n);
  return d && d->denoisers.count(p) ? p : nullptr;
}

static VSRStatus cudaStatus(Device *d, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return VSR_OK;
  const VSRStatus st = e == cudaErrorInvalidValue ? VSR_ERROR_INVALID_ARGUMENT
                       : e == cudaErrorMemoryAllocation ? VSR_ERROR_OUT_OF_MEMORY
                                                        : VSR_ERROR_CUDA;
  d->report(nullptr, VSR_UNKNOWN, VSR_SEVERITY_ERROR, st, "%s: %s", what, cudaGetErrorString(e));
  return st;
}

VSRDenoiser vsrNewDenoiser(VSRDevice dv, uint64_t seed) {
  Device *d = asDev(dv);
  if (!d) return nullptr;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = new Denoiser(seed);
  if (!n->ok()) {
    delete n;
    d->report(nullptr, VSR_UNKNOWN, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
              "denoiser allocation failed");
    return nullptr;
  }
  d->denoisers.insert(n);
  return reinterpret_cast<VSRDenoiser>(n);
}

VSRStatus vsrReleaseDenoiser(VSRDevice dv, VSRDenoiser nv) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  cudaStreamSynchronize(d->stream);
  d->denoisers.erase(n);
  delete n;
  return VSR_OK;
}

uint64_t vsrDenoiserParameterCount(VSRDevice dv, VSRDenoiser nv) {
  Device *d = asDev(dv);
  if (!d) return 0;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  return n ? n->numParams() : 0;
}

VSRStatus vsrDenoiserSetTensorPath(VSRDevice dv, VSRDenoiser nv, int path) {
  Device *d = asDev(dv);
  if (!d || path < 0 || path > 4) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  cudaStreamSynchronize(d->stream);
  n->setTensorPath(path);
  return VSR_OK;
}

uint32_t vsrDenoiserErrors(VSRDevice dv, VSRDenoiser nv) {
  Device *d = asDev(dv);
  if (!d) return 0;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return 0;
  uint32_t e = 0;
  if (cudaMemcpyAsync(&e, n->errorWord(), sizeof(e), cudaMemcpyDeviceToHost, d->stream) !=
          cudaSuccess ||
      cudaMemsetAsync(n->errorWord(), 0, sizeof(e), d->stream) != cudaSuccess ||
      cudaStreamSynchronize(d->stream) != cudaSuccess)
    return 0xffffffffu;
  return e;
}

VSRStatus vsrDenoiserTestWaitTimeout(VSRDevice dv, VSRDenoiser nv) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  n->armWaitTimeoutTest();
  return VSR_OK;
}

VSRStatus vsrDenoiserGetParameters(VSRDevice dv, VSRDenoiser nv, float *params, uint64_t count) {
  Device *d = asDev(dv);
  if (!d || !params) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  if (count != n->numParams()) return VSR_ERROR_INVALID_ARGUMENT;
  return cudaStatus(d, n->getParams(params, d->stream), "denoiser parameters");
}

VSRStatus vsrDenoiserSetParameters(VSRDevice dv, VSRDenoiser nv, const float *params,
                                   uint64_t count) {
  Device *d = asDev(dv);
  if (!d || !params) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  if (count != n->numParams()) return VSR_ERROR_INVALID_ARGUMENT;
  return cudaStatus(d, n->setParams(params, d->stream), "denoiser parameters");
}

VSRStatus vsrDenoiserForward(VSRDevice dv, VSRDenoiser nv, const void *input, uint32_t N,
                             uint32_t H, uint32_t W, float *output) {
  Device *d = asDev(dv);
  if (!d || !input || !output) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  return cudaStatus(
      d, n->forward((const __nv_bfloat16 *)input, (int)N, (int)H, (int)W, output, d->stream),
      "denoiser forward");
}

// forward + backward; the loss (if wanted) is copied to the host
static VSRStatus denoiserBackward(Device *d, Denoiser *n, const void *input, const float *target,
                                  uint32_t tC, uint32_t N, uint32_t H, uint32_t W, float *loss) {
  VSRStatus st = cudaStatus(d, n->backward((const __nv_bfloat16 *)input, target, (int)tC, (int)N,
                                           (int)H, (int)W, n->lossDevice(), d->stream),
                            "denoiser backward");
  if (st == VSR_OK && loss)
    st = cudaStatus(d, cudaMemcpyAsync(loss, n->lossDevice(), sizeof(float),
                                       cudaMemcpyDeviceToHost, d->stream),
                    "denoiser loss");
  return st;
}

VSRStatus vsrDenoiserGradients(VSRDevice dv, VSRDenoiser nv, const void *input, const float *target,
                               uint32_t tC, uint32_t N, uint32_t H, uint32_t W, float *grads,
                               uint64_t count, float *loss) {
  Device *d = asDev(dv);
  if (!d || !input || !target || !grads) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  if (count != n->numParams()) return VSR_ERROR_INVALID_ARGUMENT;
  VSRStatus st = denoiserBackward(d, n, input, target, tC, N, H, W, loss);
  if (st == VSR_OK)
    st = cudaStatus(d, cudaMemcpyAsync(grads, n->grad(), count * sizeof(float),
                                       cudaMemcpyDeviceToHost, d->stream),
                    "denoiser gradients");
  if (st == VSR_OK) st = cudaStatus(d, cudaStreamSynchronize(d->stream), "denoiser gradients");
  return st;
}

VSRStatus vsrDenoiserTrainStep(VSRDevice dv, VSRDenoiser nv, const void *input, const float *target,
                               uint32_t tC, uint32_t N, uint32_t H, uint32_t W, float lr,
                               float *loss) {
  Device *d = asDev(dv);
  if (!d || !input || !target) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  if (!n) return VSR_ERROR_INVALID_OBJECT;
  VSRStatus st = denoiserBackward(d, n, input, target, tC, N, H, W, loss);
  if (st == VSR_OK) st = cudaStatus(d, n->adam(lr, d->stream), "denoiser update");
  if (st == VSR_OK && loss) st = cudaStatus(d, cudaStreamSynchronize(d->stream), "denoiser step");
  return st;
}

// 1 / sqrt(samples per pixel accumulated in the frame), a network input
static float denoiseInvSqrtN(FrameObj *F) {
  const int spp = F->renderer ? F->renderer->r.pixelSamples : 1;
  const double n = (double)std::max(F->accumID, 1) * std::max(spp, 1);
  return (float)(1.0 / std::sqrt(n));
}

VSRStatus vsrDenoiserFrameInput(VSRDevice dv, VSRFrame fv, void *input) {
  Device *d = asDev(dv);
  if (!d || !input) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(fv);
  if (!checkObj(d, o) || o->kind != VSR_FRAME) return VSR_ERROR_INVALID_OBJECT;
  FrameObj *F = static_cast<FrameObj *>(o);
  if (!F->valid || !F->accum.p) return VSR_ERROR_INCOMPLETE;
  const int Wp = (F->width + 7) / 8 * 8, Hp = (F->height + 7) / 8 * 8;
  return cudaStatus(d, launchDenoiseInput(F->accum.as<float4>(), F->albedo.as<float>(),
                                          F->normal.as<float>(), F->depth.as<float>(),
                                          F->variance.as<float>(), denoiseInvSqrtN(F), F->width,
                                          F->height, Wp, Hp, (__nv_bfloat16 *)input,
                                          Denoiser::kInC, d->stream),
                    "denoiser input");
}

VSRStatus vsrDenoiseFrame(VSRDevice dv, VSRDenoiser nv, VSRFrame fv, float k, float floorAbs,
                          float *colorOut, uint8_t *retry, uint32_t *numRetry) {
  Device *d = asDev(dv);
  if (!d || !colorOut) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Denoiser *n = asDenoiser(d, nv);
  Object *o = asObj(fv);
  if (!n || !checkObj(d, o) || o->kind != VSR_FRAME) return VSR_ERROR_INVALID_OBJECT;
  FrameObj *F = static_cast<FrameObj *>(o);
  if (!F->valid || !F->accum.p) return VSR_ERROR_INCOMPLETE;
  const int Wp = (F->width + 7) / 8 * 8, Hp = (F->height + 7) / 8 * 8;
  const size_t np = (size_t)Wp * Hp;
  if (F->denoiseIn.bytes < np * Denoiser::kInC * 2 ||
      F->denoiseOut.bytes < np * Denoiser::kOutC * 4 || !F->denoiseCount.p) {
    if (F->denoiseIn.alloc(np * Denoiser::kInC * 2) != cudaSuccess ||
        F->denoiseOut.alloc(np * Denoiser::kOutC * 4) != cudaSuccess ||
        F->denoiseCount.alloc(sizeof(unsigned)) != cudaSuccess)
      return VSR_ERROR_OUT_OF_MEMORY;
  }
  cudaStream_t s = d->stream;
  const float4 *mean = F->accum.as<float4>();
  VSRStatus st = cudaStatus(
      d, launchDenoiseInput(mean, F->albedo.as<float>(), F->normal.as<float>(), F->depth.as<float>(),
                            F->variance.as<float>(), denoiseInvSqrtN(F), F->width, F->height, Wp,
                            Hp, F->denoiseIn.as<__nv_bfloat16>(), Denoiser::kInC, s),
      "denoiser input");
  if (st == VSR_OK)
    st = cudaStatus(d, n->forward(F->denoiseIn.as<__nv_bfloat16>(), 1, Hp, Wp,
                                  F->denoiseOut.as<float>(), s),
                    "denoiser forward");
  if (st == VSR_OK) cudaMemsetAsync(F->denoiseCount.p, 0, sizeof(unsigned), s);
  const float *var = F->variance.p ? F->variance.as<float>() : nullptr;
  if (st == VSR_OK)
    st = cudaStatus(d, launchDenoiseOutput(F->denoiseOut.as<float>(), Denoiser::kOutC, F->width,
                                           F->height, Wp, mean, var, k, floorAbs,
                                           (float4 *)colorOut, retry,
                                           F->denoiseCount.as<unsigned>(), s),
                    "denoiser output");
  if (st == VSR_OK && numRetry) {
    uint32_t word = 0;
    st = cudaStatus(d, cudaMemcpyAsync(numRetry, F->denoiseCount.p, sizeof(unsigned),
                                       cudaMemcpyDeviceToHost, s),
                    "denoiser retry count");
    if (st == VSR_OK)
      st = cudaStatus(d, cudaMemcpyAsync(&word, n->errorWord(), sizeof(word),
                                         cudaMemcpyDeviceToHost, s),
                      "denoiser error word");
    if (st == VSR_OK) st = cudaStatus(d, cudaStreamSynchronize(s), "denoiser");
    if (st == VSR_OK && word) {
      // a bounded wait of a tcgen05 convolution ran out: the image is not valid
      d->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_TIMEOUT,
                "denoiser: a tensor-core wait ran out (error word 0x%x)", word);
      st = VSR_ERROR_TIMEOUT;
    }
  }
  return st;
}

uint64_t vsrPlanBatch(const uint32_t *width, const uint32_t *height, const float *costPerPixel,
                      uint32_t numJobs, uint32_t tileWidth, uint32_t *items, uint64_t capacity) {
  if ((!width || !height || !costPerPixel) && numJobs) return 0;
  std::vector<uint32_t> out;
  const size_t n = planItems(width, height, costPerPixel, numJobs, tileWidth, out);
  if (items) memcpy(items, out.data(), std::min<uint64_t>(n, capacity) * 2 * sizeof(uint32_t));
  return n;
}

VSRStatus vsrRenderFrame(VSRDevice dv, VSRFrame fv) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(fv);
  if (!checkObj(d, o) || o->kind != VSR_FRAME) return VSR_ERROR_INVALID_OBJECT;
  return renderFrame(d, static_cast<FrameObj *>(o));
}

int vsrFrameReady(VSRDevice dv, VSRFrame fv, VSRWaitMask mask) {
  Device *d = asDev(dv);
  if (!d) return 0;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(fv);
  if (!checkObj(d, o) || o->kind != VSR_FRAME) return 0;
  FrameObj *F = static_cast<FrameObj *>(o);
  if (mask == VSR_WAIT) {
    cudaError_t e = cudaStreamSynchronize(d->stream);
    if (e != cudaSuccess) {
      d->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA, "render failed: %s",
                cudaGetErrorString(e));
      return 0;
    }
  } else if (cudaEventQuery(F->evStop) != cudaSuccess) {
    return 0;
  }
  if (*F->errHost)
    d->report(F, VSR_FRAME, VSR_SEVERITY_WARNING, VSR_OK, "device error flags 0x%x in last render",
              *F->errHost);
  return 1;
}

VSRStatus vsrFrameSampleMask(VSRDevice dv, VSRFrame fv, const uint8_t *mask) {
  Device *d = asDev(dv);
  if (!d) return VSR_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(fv);
  if (!checkObj(d, o) || o->kind != VSR_FRAME) return VSR_ERROR_INVALID_OBJECT;
  FrameObj *F = static_cast<FrameObj *>(o);
  if (mask && !F->pixelFrames.p) {
    // from now on each pixel counts its own frames, starting from the
    // frames accumulated so far
    const size_t np = (size_t)F->width * F->height;
    if (F->pixelFrames.alloc(np * sizeof(uint32_t)) != cudaSuccess) {
      d->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
                "sample mask: per-pixel frame counts could not be allocated");
      return VSR_ERROR_OUT_OF_MEMORY;
    }
    const uint32_t start = F->nextReset ? 0u : (uint32_t)F->accumID;
    if (launchFillU32(F->pixelFrames.as<uint32_t>(), start, np, d->stream) != cudaSuccess)
      return VSR_ERROR_CUDA;
  }
  F->sampleMask = mask;
  return VSR_OK;
}

VSRStatus vsrDiscardFrame(VSRDevice dv, VSRFrame fv) {
  (void)dv;
  (void)fv;
  return VSR_OK;
}

const void *vsrMapFrame(VSRDevice dv, VSRFrame fv, const char *channel, uint32_t *width,
                        uint32_t *height, VSRDataType *pixelType) {
  Device *d = asDev(dv);
  if (!d || !channel) return nullptr;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(fv);
  if (!checkObj(d, o) || o->kind != VSR_FRAME) return nullptr;
  FrameObj *F = static_cast<FrameObj *>(o);
  void *p;
  size_t bytes;
  VSRDataType t;
  if (!channelBuf(F, channel, p, bytes, t)) {
    d->report(F, VSR_FRAME, VSR_SEVERITY_WARNING, VSR_ERROR_INVALID_ARGUMENT,
              "channel '%s' is not enabled on this frame", channel);
    if (width) *width = 0;
    if (height) *height = 0;
    if (pixelType) *pixelType = VSR_UNKNOWN;
    return nullptr;
  }
  void *&host = F->pinned[channel];
  if (width) *width = 0;
  if (height) *height = 0;
  if (pixelType) *pixelType = VSR_UNKNOWN;
  if (!host && cudaMallocHost(&host, bytes) != cudaSuccess) {
    host = nullptr;
    d->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_OUT_OF_MEMORY,
              "map of channel '%s': no pinned host buffer of %zu bytes", channel, bytes);
    return nullptr;
  }
  // a failed copy must not hand back the previous frame's pixels
  cudaError_t e = cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, d->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) {
    d->report(F, VSR_FRAME, VSR_SEVERITY_ERROR, VSR_ERROR_CUDA, "map of channel '%s' failed: %s",
              channel, cudaGetErrorString(e));
    return nullptr;
  }
  if (width) *width = (uint32_t)F->width;
  if (height) *height = (uint32_t)F->height;
  if (pixelType) *pixelType = t;
  return host;
}

VSRStatus vsrUnmapFrame(VSRDevice dv, VSRFrame fv, const char *channel) {
  (void)dv;
  (void)fv;
  (void)channel;
  return VSR_OK;
}

const void *vsrMapFrameDevice(VSRDevice dv, VSRFrame fv, const char *channel, uint32_t *width,
                              uint32_t *height, VSRDataType *pixelType) {
  Device *d = asDev(dv);
  if (!d || !channel) return nullptr;
  std::lock_guard<std::recursive_mutex> lk(d->mtx);
  Object *o = asObj(fv);
  if (!checkObj(d, o) || o->kind != VSR_FRAME) return nullptr;
  FrameObj *F = static_cast<FrameObj *>(o);
  void *p;
  size_t bytes;
  VSRDataType t;
  if (!channelBuf(F, channel, p, bytes, t)) return nullptr;
  if (width) *width = (uint32_t)F->width;
  if (height) *height = (uint32_t)F->height;
  if (pixelType) *pixelType = t;
  return p;
}

void *vsrDeviceStream(VSRDevice dv) {
  Device *d = asDev(dv);
  return d ? (void *)d->stream : nullptr;
}

VSRStatus vsrBuildTriangleBVH(const float *v1, const float *e1, const float *e2, uint32_t n,
                              void *nodesOut, void *trisOut, void *stream) {
  if (n == 0) return VSR_OK;
  if (!v1 || !e1 || !e2 || !nodesOut || !trisOut || n >= (1u << 27))
    return VSR_ERROR_INVALID_ARGUMENT;
  cudaError_t e = buildGroupBVH(v1, e1, e2, (int)n, (float4 *)nodesOut, (float4 *)trisOut, nullptr,
                                (cudaStream_t)stream);
  return e == cudaSuccess ? VSR_OK : VSR_ERROR_CUDA;
}

} // extern "C"
