// Device-side scene, camera, renderer and frame records.
//
// These are the flat POD records the render kernels read. They are passed
// to each launch by value (kernel parameters), replacing the reference's
// per-frame DevicePointer copies of the object registry, renderer state,
// frame and camera (renderer/Renderer.cpp:19-22, DeviceArray.h:377-394).
//
// HBM layout per group (one BVH per group over all its triangle surfaces):
//   nodes : 4 x float4 per BVH2 node (64 B): child boxes interleaved
//           (lo0.x,hi0.x,lo0.y,hi0.y) (lo1.x,hi1.x,lo1.y,hi1.y)
//           (lo0.z,hi0.z,lo1.z,hi1.z) (child0,child1,-,-) as int bits.
//           child >= 0: inner node index; child < 0: leaf code ~(first |
//           (count-1) << 27) over the leaf-ordered triangle array.
//   tris  : 3 x float4 per triangle in leaf order (48 B):
//           (v1.xyz, local id), (e1.xyz, 0), (e2.xyz, 0)
//           with e1 = v2 - v1, e2 = v3 - v1 (scene/surface/geometry/Triangle.cpp:76-83).
//   triSurface : local triangle id -> global surface index (material).
//   triPrim    : local triangle id -> primitive id inside its geometry.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vsr {

enum { MAT_MATTE = 0, MAT_PBR = 1 };
enum { ALPHA_OPAQUE = 0, ALPHA_BLEND = 1, ALPHA_MASK = 2 };
enum { CAM_PERSPECTIVE = 0, CAM_MATRIX = 1, CAM_ORTHO = 2, CAM_OMNI = 3 };
enum { REND_RAYCAST = 0, REND_PATHTRACE = 1 };
enum { COLOR_FLOAT4 = 0, COLOR_UFIXED8 = 1, COLOR_SRGB8 = 2, COLOR_NONE = 3 };

// Device-side error bits, read back as frame property "errorFlags".
enum : uint32_t {
  ERR_STACK_OVERFLOW = 1u,   // BVH traversal stack full: traversal stopped
  ERR_DDA_LIMIT = 2u,        // DDA step limit reached
  ERR_TRACK_LIMIT = 4u,      // delta-tracking step limit reached
  ERR_PATH_LIMIT = 8u,       // path pass limit reached
  ERR_MARCH_LIMIT = 16u,     // ray-march step limit reached (dt too small for t)
  ERR_LAYER_LIMIT = 32u,     // transparent-surface loop limit reached
  ERR_NONFINITE = 64u,       // a path sample was NaN or infinite and was dropped
};

#ifdef __CUDACC__
// A path sample is dropped (counts as zero) when a component is NaN or
// infinite, so that one degenerate sample (e.g. a half vector of opposite
// directions) does not poison a pixel's running mean forever.
__device__ __forceinline__ bool finiteSample(const float4 &c) {
  return isfinite(c.x) && isfinite(c.y) && isfinite(c.z) && isfinite(c.w);
}
#endif

constexpr int kMaxMarchSteps = 1 << 20;
constexpr int kMaxSurfaceLayers = 1 << 12;

// Launch-bound tunables (minimum resident blocks per SM) of the path-tracer
// kernels; they trade registers for occupancy.
#ifndef VSR_MEGA_MIN_BLOCKS
#define VSR_MEGA_MIN_BLOCKS 16  // 32 registers, 64 warps per SM: latency hiding beats spill cost
#endif
#ifndef VSR_SMEM_STACK
#define VSR_SMEM_STACK 0  // BVH2 traversal: stack entries kept in shared memory (0: all local)
#endif
#ifndef VSR_MEGA_MIN_BLOCKS_VOLUMES
#define VSR_MEGA_MIN_BLOCKS_VOLUMES 8  // ~64 registers for worlds with volumes
#endif
#ifndef VSR_MEGA_BLOCK_Y
#define VSR_MEGA_BLOCK_Y 8  // path-tracer megakernel tile: 16 x VSR_MEGA_BLOCK_Y pixels
#endif
#ifndef VSR_MARCH_BATCH
#define VSR_MARCH_BATCH 4  // field fetches issued per thread before compositing
#endif
#ifndef VSR_RAYCAST_MIN_BLOCKS
#define VSR_RAYCAST_MIN_BLOCKS 1
#endif
#ifndef VSR_RAYCAST_FULL_MIN_BLOCKS
#define VSR_RAYCAST_FULL_MIN_BLOCKS 3  // the full-feature variant: at most 168 registers
#endif
#ifndef VSR_RAYCAST_BLOCK_X
#define VSR_RAYCAST_BLOCK_X 16  // raycast tile: VSR_RAYCAST_BLOCK_X x VSR_RAYCAST_BLOCK_Y pixels
#endif
#ifndef VSR_RAYCAST_BLOCK_Y
#define VSR_RAYCAST_BLOCK_Y 8
#endif
#ifndef VSR_WAVE_TRACE_MIN_BLOCKS
#define VSR_WAVE_TRACE_MIN_BLOCKS 1
#endif
#ifndef VSR_WAVE_SHADE_MIN_BLOCKS
#define VSR_WAVE_SHADE_MIN_BLOCKS 1
#endif
#ifndef VSR_WAVE_DYN_MIN_BLOCKS
#define VSR_WAVE_DYN_MIN_BLOCKS 8  // persistent traversal: 128-thread blocks, <= 64 registers
#endif

constexpr int kTraversalStack = 64;
// Frame statistics (frame property "statistics", uint64 each, filled by the
// counting kernel variants when "collectStatistics" is on):
//   0 rays traced, 1 BVH inner-node visits, 2 primitive tests, 3 ray-march
//   samples, 4 delta-tracking samples, 5 majorant cells visited,
//   8..23 histogram of inner-node visits per traversal (bins [2^k, 2^(k+1))),
//   path tracer only: 24 clock cycles per pixel thread from its start to
//   its frame write (summed over threads), 25 of them inside surface
//   traversal, 26 inside delta tracking; 27 warp iterations of the
//   traversal's inner-node loop x 65536 (each active lane adds
//   65536 / active lanes), 28 leaf-loop lane iterations, 29 leaf-loop warp
//   iterations x 65536. SIMT efficiency of the inner-node loop =
//   [1] / (32 [27] / 65536), of the leaf loop [28] / (32 [29] / 65536).
constexpr int kStatCounters = 32;
constexpr int kMaxClipPlanes = 8;
constexpr uint32_t kLeafCountShift = 27;
constexpr uint32_t kLeafFirstMask = (1u << kLeafCountShift) - 1u;

// Where a material parameter comes from (dco::MaterialParam*, renderer/
// common.h:593-640): its value, a geometry / hit attribute (ATTR_*), or a
// sampler (SRC_SAMPLER + the sampler's index in DScene::samplers).
enum { SRC_VALUE = -1, SRC_SAMPLER = 16 };
enum { MSRC_COLOR = 0, MSRC_OPACITY = 1, MSRC_METALLIC = 2, MSRC_ROUGHNESS = 3 };

struct DMaterial {
  float baseColor[3];
  int type;
  float metallic, roughness, ior, opacity;
  float clearcoat, clearcoatRoughness, transmission, sheenRoughness;
  float sheenColor[3];
  int alphaMode;
  float alphaCutoff;
  short src[4];  // MSRC_*: SRC_VALUE, an ATTR_* or SRC_SAMPLER + k
  int pad;
};

// Geometry and hit attributes (dco::Attribute, DeviceCopyableObjects.h
// :1626-1655): attribute0..3, color, then the hit's world position, world
// normal, object position and object normal.
enum { ATTR_0 = 0, ATTR_1, ATTR_2, ATTR_3, ATTR_COLOR, ATTR_WORLD_POS, ATTR_WORLD_NORMAL,
       ATTR_OBJECT_POS, ATTR_OBJECT_NORMAL, ATTR_NONE = 15 };

// One attribute array: `comps` components per element, float32 or unorm8
// / unorm16 (toRGBA, common.h:265-360); comps = 0: absent.
struct DAttr {
  const void *data;
  uint32_t len;
  uint16_t comps;
  uint16_t fixedBits;  // 0 = float32, 8 or 16 = unorm
};

// Per surface (indexed like DScene::materials): its geometry's attributes.
// Triangles: vertex and face-varying arrays interpolated with the hit's
// barycentrics (vertex indices from `index`, 3 per primitive, or
// consecutive), per-primitive arrays, then uniform values; other kinds use
// the per-primitive and uniform ones. vertexNormal: float3 per vertex
// (shading normals), fvNormal: the geometry has face-varying normals.
struct DSurfAttr {
  const uint32_t *index;
  const float *vertexNormal;
  uint32_t numVertexNormals;
  int fvNormal;
  DAttr vertex[5], faceVarying[5], primitive[5];
  float uniform[5][4];
  uint32_t uniformMask;
  int isTriangle;
};

// Per instance: its uniform attributes (Instance.cpp, "color",
// "attribute0..3").
struct DInstAttr {
  float v[5][4];
  uint32_t mask;
  int pad[3];
};

enum { SAMP_IMAGE1D = 0, SAMP_IMAGE2D = 1, SAMP_IMAGE3D = 2, SAMP_TRANSFORM = 3, SAMP_PRIMITIVE = 4 };
enum { WRAP_CLAMP = 0, WRAP_REPEAT = 1, WRAP_MIRROR = 2 };

// A sampler (scene/surface/material/sampler): image samplers hold RGBA8
// texels (every image format is converted to 8 bits per channel, as the
// reference's imageSamplerUpdateData does), dims[] texels per axis.
struct DSampler {
  int type;
  int inAttribute;
  int linear;       // filter "linear" (else nearest)
  int wrap[3];
  int dims[3];
  const uchar4 *texels;
  DAttr prim;       // primitive sampler: the array
  uint32_t primOffset;
  float inXfm[16], inOffset[4], outXfm[16], outOffset[4];  // column-major mat4
};

enum LightType { LIGHT_DIRECTIONAL = 0, LIGHT_POINT = 1, LIGHT_SPOT = 2, LIGHT_QUAD = 3, LIGHT_HDRI = 4 };

// One light in world space (instance transforms applied on the host).
struct DLight {
  float dir[3];        // directional: unit vector towards the light (-direction);
                       // spot: the cone axis (instance-transformed, normalised at use)
  float intensity[3];  // color * irradiance (directional) or color * intensity
  float cosHalfAngle;  // directional: cos(angularDiameter/2); 1 = delta light
  int type;            // LightType
  int visible;
  float pos[3];        // point / spot position
  float cosOuter;      // spot: cos(openingAngle)
  float cosInner;      // spot: cos(openingAngle - 2 falloffAngle)
  float pad[2];
  // quad: corner pos, edges e1, e2 (the parallelogram pos + a e1 + b e2,
  // tessellated as (pos, e1, e1 + e2) and (pos, e1 + e2, e2)), the two
  // triangles' areas and the unit normal of the first
  float e1[3], e2[3];
  float area1, area2;
  float normal[3];
  float pad2;
  // hdri: the radiance image (RGBA, row-major, hdriW x hdriH), its
  // row-wise normalised CDFs (hdriW x hdriH) and the normalised CDF of the
  // row sums (hdriH); scale; the image frame's rotation (column-major,
  // toWorld) and its inverse
  const float4 *hdriTex;
  const float *hdriRows;
  const float *hdriLastCol;
  int hdriW, hdriH;
  float scale;
  float toWorld[9], toLocal[9];
};

struct DVolume {
  cudaTextureObject_t tex;    // the same field as a 3D texture (linear, clamp, normalized)
  float vrScale;              // 1 / (vrMax - vrMin)
  const float *data;   // dims.x*dims.y*dims.z, x fastest
  const float4 *tf;    // transfer function table
  const float *majorant;  // gdims cells or null
  int dims[3];
  int tfSize;
  int gdims[3];
  float unitDistance;
  float boundsLo[3], boundsHi[3];
  float S[3], T[3];    // voxel space = S * (p + T)
  float cellSize;
  float vrMin, vrMax;
};

// BVH4 node (128 B, 8 x float4): child boxes as structure of arrays
//   [0] lo.x of children 0..3   [1] hi.x   [2] lo.y   [3] hi.y   [4] lo.z   [5] hi.z
//   [6] child codes (int bits): >= 0 inner node index, kEmptyChild = no child
//       (must be tested by code: its box bytes are meaningless), otherwise a
//       leaf code as for BVH2   [7] unused
constexpr int kEmptyChild = 0x7fffffff;

enum AnalyticKind { AP_SPHERE = 0, AP_CONE = 1, AP_CYLINDER = 2, AP_CURVE = 3 };
// float4 records per analytic primitive: sphere (center, r); cone /
// cylinder (v1, r1), (v2, r2); curve (w0, r), (w1, -), (w2, -), (w3, -)
constexpr int kApStride = 4;
constexpr int kApFloats = 4 * kApStride;

// An iso-surface of a structured field (ISOSurface.cpp): the field as a
// volume record (its TF fields unused), the iso values, the surface index.
struct DIso {
  DVolume field;
  const float *values;
  int numValues;
  uint32_t surface;
  float step;  // march step in world units: min(spacing) / 2
};
constexpr int kApKindShift = 28;
constexpr uint32_t kApLocalMask = (1u << kApKindShift) - 1u;

struct DGroup {
  const float4 *nodes;
  const float4 *tris;
  const uint32_t *triSurface;
  const uint32_t *triPrim;
  int numTris;
  int numNodes;
  int width;              // 2: BVH2 nodes (64 B), 4: BVH4 nodes (128 B)
  int volBegin, volEnd;   // range in DScene::groupVolumes
  float boundsLo[3], boundsHi[3];
  // analytic primitives (all sphere, cone and cylinder geometries of the
  // group) with their own BVH2: leaf i is apPrims[kApStride i ..]
  // (sphere: (center, radius), unused; cone / cylinder: (v1, r1), (v2, r2)),
  // apLocal[i] = the primitive's index in the group | kind << kApKindShift,
  // apSurface maps a group index to its surface. A hit on primitive k
  // carries Hit::tri = numTris + k.
  // per local triangle: an object-space shading normal (w = 1) that
  // replaces normalize(e1 x e2), set for quad geometries; null when the
  // group has none
  const float4 *triNormal;
  const float4 *apNodes;
  const float4 *apPrims;
  const uint32_t *apLocal;
  const uint32_t *apSurface;
  int numAP;
  int apNumNodes;
  // iso-surfaces of the group; a hit on iso-surface k carries
  // Hit::tri = numTris + numAP + k and Hit::leaf = k
  const DIso *isos;
  int numIso;
};

struct DInstance {
  float affineInv[9];  // column-major 3x3
  float transInv[3];
  float normalXfm[9];  // transpose(affineInv)
  int group;
  uint32_t userID;
};

struct DScene {
  const DInstance *instances;
  const DGroup *groups;
  const DMaterial *materials;
  const DLight *lights;
  const DVolume *volumes;
  const int *groupVolumes;
  int numInstances;
  int numGroups;
  int numLights;
  int positionalLights;  // point, spot and quad lights among them: the kernels' full variants
  int areaLights;        // quad and HDRI lights among them (hit by rays; no wavefront mode)
  int numAnalytic;       // spheres, cones, cylinders in all groups: the kernels' full variants
  int quadGroups;        // groups with quad geometry (triNormal set): the full variants
  int numIso;            // iso-surfaces in all groups: the full variants
  int numVolumes;
  int allOpaque;
  int hasSurfaces;
  int maxGroupWidth;  // widest group BVH (2 or 4)
  // attributes, samplers, shading normals (null / 0 when the world uses
  // none): the kernels' full variants resolve materials per hit
  const DSurfAttr *surfAttr;
  const DInstAttr *instAttr;
  const DSampler *samplers;
  int attributes;
};

struct DCamera {
  int type;
  float eye[3];
  float U[3], V[3], W[3];
  float dir[3];
  float lensRadius, focusDistance;
  float region[4];
  float shutter[2];
  float inv[16];       // matrix camera: inverse(proj * view), column-major
};

struct DRenderer {
  int type;
  float bg[4];
  float ambient[3];    // ambientColor * ambientRadiance
  float ambientColor[3];
  float ambientRadiance;
  float occlusionDistance;
  int ambientSamples;
  int maxBounce;
  int pixelSamples;
  // path tracer: a frame's pixelSamples are taken as sampleChunks streams of
  // pixelSamples / sampleChunks samples, defined as that many accumulated
  // sub-frames (accumulation IDs sampleChunks * accumID + c), rendered at
  // once; 1 = the reference's single stream per pixel and frame
  int sampleChunks;
  float samplingRateInv;
  int hwFilter;        // 1: field samples through the texture unit's trilinear filter
  int gradientShading; // volume samples lit along the normalised field gradient
  int numClipPlanes;
  float clip[kMaxClipPlanes][4];
  // temporal anti-aliasing of the path tracer (Pathtrace.cpp:24-37): a frame
  // writes its own mean colour and motion vectors, and a resolve pass
  // blends it with the reprojected previous result (weight taaAlpha)
  int taa;
  float taaAlpha;
};

struct DFrame {
  int width, height;
  int accumID;
  int colorType;
  void *color;
  float *depth;
  float *normal;   // float3 packed
  float *albedo;   // float3 packed
  float4 *accum;
  uint32_t *errorFlags;
  unsigned long long *counters;  // optional statistics (null = off)
  // optional (null = off): running mean over frames of the per-sample
  // squared luminance, and the variance of the accumulated mean's luminance
  float *accumSq;
  float *variance;
  int pixelSamples;  // samples per frame
  // optional (null = every pixel): one byte per pixel; the path tracer
  // leaves pixels whose byte is 0 untouched (no samples, no writes)
  const uint8_t *sampleMask;
  // optional (null = every pixel has accumID frames): frames accumulated
  // per pixel, kept once a frame has had a sample mask; the running mean
  // and the variance then weight each pixel by its own count
  uint32_t *pixelFrames;
  // per sample chunk and pixel, [3][chunks][pixels] (sampleChunks > 1):
  // the chunk's mean colour; (mean squared luminance, closest depth, Ng.xy);
  // (Ng.z, albedo)
  float4 *chunkOut;
  // temporal anti-aliasing (renderer taa): this frame's mean colour, the
  // albedo of its closest sample and its motion vector per pixel (the resolve
  // pass reads the previous frame's from taaPrev / taaPrevAlbedo), and the
  // previous and current view-projection matrices (column-major) that the
  // motion vectors are projected with
  float4 *taaCurr, *taaPrev;
  float *taaCurrAlbedo, *taaPrevAlbedo;  // float3 packed
  float2 *motionVec;
  float prevMVP[16], currMVP[16];
};

// Wavefront path-tracer state: one slot per pixel, structure of arrays
// (float4 / uint4 / int4 per pixel, so a warp working on consecutive queue
// entries reads consecutive 16-byte records), two pixel queues and their
// counts. Field packing (x,y,z | w):
//   rayO  : origin         | tmin        rayD  : direction     | tmax
//   thr   : throughput     | visLight    inten : intensity     | visAO
//   base  : baseColor      | aoWeights   shaded: shadedColor   | aoCount
//   hpo   : hitPosOff      | bsdf.pdf    sn    : shading normal| bsdf.cosT
//   bdir  : bsdf.dir       | tmin of the pass before opacity retraces
//   bf    : bsdf.f         | retrace count
//   acc   : sum of sample colours (rgba)
//   pNg   : sample Ng      | sample depth      pAlb : sample albedo | closest depth
//   cNg   : closest Ng     | -                 cAlb : closest albedo | -
//   meta  : rnd state, rng state, flags, passID
//           flags: rayType(2) firstHit(1) bounceID(9) aoSamples(9) sampleID(9) retrace(1)
//   hit   : t bits, instance (-1 = miss), local triangle, leaf index
struct DWave {
  float4 *rayO, *rayD, *thr, *inten, *base, *shaded, *hpo, *sn, *bdir, *bf, *acc, *pNg, *pAlb,
      *cNg, *cAlb;
  uint4 *meta;
  int4 *hit;
  uint32_t *queue[2];
  uint32_t *count;  // [0], [1] queue lengths; [2], [3] entries handed out by the traversal
};

} // namespace vsr
