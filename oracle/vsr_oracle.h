/* CPU oracle for the raycast / pathtrace hot path: C API.
 *
 * TEST INFRASTRUCTURE ONLY. This is a CPU restatement of the reference
 * anari-visionaray CPU device for the per-pixel hot path; it is the checker
 * used by tests/, the smoke check and the CPU-baseline leg of bench.py. The
 * product library never includes, links or calls it.
 *
 * The reference (Visionaray + ANARI-SDK based) cannot be compiled in this
 * environment, so parity is unpinned against the reference binary; each
 * function cites the reference source it restates.
 */
#ifndef VSR_ORACLE_H
#define VSR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_MATTE = 0, OR_PBR = 1 };
enum { OR_ALPHA_OPAQUE = 0, OR_ALPHA_BLEND = 1, OR_ALPHA_MASK = 2 };
enum { OR_CAM_PERSPECTIVE = 0, OR_CAM_MATRIX = 1, OR_CAM_ORTHO = 2, OR_CAM_OMNI = 3 };
enum { OR_RAYCAST = 0, OR_PATHTRACE = 1 };
enum { OR_GRID_NONE = 0, OR_GRID_REFERENCE = 1, OR_GRID_BRICK = 2 };
enum { OR_COLOR_FLOAT4 = 0, OR_COLOR_UFIXED8 = 1, OR_COLOR_SRGB8 = 2 };

/* dco::Material (DeviceCopyableObjects.h) with constant parameters. */
typedef struct OrMaterial {
  int32_t type;
  float baseColor[3];
  float opacity;
  float metallic, roughness, ior;
  float clearcoat, clearcoatRoughness, transmission;
  float sheenColor[3];
  float sheenRoughness;
  int32_t alphaMode;
  float alphaCutoff;
  int32_t src[4];           /* color, opacity, metallic, roughness: -1 the value,
                               0..8 an attribute (OR_ATTR_*), 16 + k sampler k */
} OrMaterial;

/* Attributes: attribute0..3, color, then the hit's world position, world
   normal, object position and object normal (dco::Attribute). */
enum { OR_ATTR_COLOR = 4, OR_ATTR_WORLD_POS = 5, OR_ATTR_WORLD_NORMAL = 6,
       OR_ATTR_OBJECT_POS = 7, OR_ATTR_OBJECT_NORMAL = 8, OR_ATTR_NONE = 15 };

typedef struct OrAttr {
  const void *data;         /* len elements of comps float32, or unorm (fixedBits 8 / 16) */
  uint32_t len;
  int32_t comps;            /* 0 = absent */
  int32_t fixedBits;
} OrAttr;

/* A surface's geometry attributes (triangles: vertex, face-varying and
   per-primitive arrays, vertex normals; every kind: uniform values). */
typedef struct OrSurfAttr {
  const uint32_t *index;    /* triangles: 3 vertex indices per primitive, or null */
  const float *vertexNormal;
  uint32_t numVertexNormals;
  int32_t fvNormal;         /* the geometry has face-varying normals */
  OrAttr vertex[5], faceVarying[5], primitive[5];
  float uniform[5][4];
  uint32_t uniformMask;
  int32_t isTriangle;
} OrSurfAttr;

enum { OR_SAMP_IMAGE1D = 0, OR_SAMP_IMAGE2D = 1, OR_SAMP_IMAGE3D = 2, OR_SAMP_TRANSFORM = 3,
       OR_SAMP_PRIMITIVE = 4 };
enum { OR_IMG_FLOAT = 0, OR_IMG_UNORM8 = 1, OR_IMG_SRGB8 = 2 };

typedef struct OrSampler {
  int32_t type, inAttribute, linear;
  int32_t wrap[3];          /* 0 clampToEdge, 1 repeat, 2 mirrorRepeat */
  int32_t dims[3];          /* texels per axis (1 past the image's dimension) */
  const void *image;        /* image samplers: dims[0] * dims[1] * dims[2] texels */
  int32_t imageType;        /* OR_IMG_* */
  int32_t imageComps;       /* 1..4 (sRGB: 4) */
  OrAttr prim;              /* primitive sampler */
  uint32_t primOffset;
  float inXfm[16], inOffset[4], outXfm[16], outOffset[4];
} OrSampler;

/* structuredRegular field + transferFunction1D volume. */
typedef struct OrVolume {
  const float *data;      /* dims.x*dims.y*dims.z floats, x fastest */
  int32_t dims[3];
  float origin[3];
  float spacing[3];
  const float *tf;        /* tfSize RGBA float4 entries */
  int32_t tfSize;
  float valueRange[2];
  float unitDistance;
  int32_t gridMethod;     /* OR_GRID_* : majorant grid for delta tracking */
  int32_t gridDims[3];    /* OR_GRID_REFERENCE: cell grid; OR_GRID_BRICK: ignored */
  int32_t brickSize;      /* OR_GRID_BRICK: voxels per brick edge */
} OrVolume;

typedef struct OrGroup {
  int32_t triBegin, triEnd; /* range in the scene's triangle array */
  int32_t volBegin, volEnd; /* range in the scene's volume array */
  int32_t apBegin, apEnd;   /* range in the scene's sphere / cone / cylinder array */
  int32_t isoBegin, isoEnd; /* range in the scene's iso-surface array */
} OrGroup;

typedef struct OrIso {
  int32_t field;            /* index into OrScene::isoFields (TF fields unused) */
  int32_t numValues;
  const float *values;
  uint32_t surface;         /* surface index */
} OrIso;

typedef struct OrInstance {
  float xfm[12];            /* column-major 3x4 affine: 3 columns + translation */
  int32_t group;
  uint32_t userID;
  float attr[5][4];         /* uniform attributes */
  uint32_t attrMask;
} OrInstance;

typedef struct OrLight {
  int32_t type;             /* 0 = directional, 1 = point, 2 = spot, 3 = quad,
                               4 = hdri */
  float direction[3];       /* directional: direction the light travels (ANARI
                               "direction"); spot: cone axis, world space */
  float color[3];
  float irradiance;
  float angularDiameter;
  int32_t visible;
  float position[3];        /* point / spot / quad, world space */
  float intensity;          /* point / spot / quad */
  float openingAngle;       /* spot */
  float falloffAngle;       /* spot */
  float edge1[3], edge2[3]; /* quad: the parallelogram position + a edge1 +
                               b edge2, world space */
  const float *radiance;    /* hdri: hdriH rows of hdriW RGB texels */
  int32_t hdriW, hdriH;
  float scale;              /* hdri */
  float up[3];              /* hdri: with 'direction', the image's frame */
} OrLight;

typedef struct OrScene {
  int32_t numTriangles;
  const float *triVerts;     /* 9 floats per triangle (object space) */
  const uint32_t *triSurface;/* surface index per triangle */
  const uint32_t *triPrimID; /* primitive index inside its geometry */
  int32_t numSurfaces;
  const OrMaterial *surfMaterial;
  const uint32_t *surfObjID;
  int32_t numVolumes;
  const OrVolume *volumes;
  int32_t numGroups;
  const OrGroup *groups;
  int32_t numInstances;
  const OrInstance *instances;
  int32_t numLights;
  const OrLight *lights;
  int32_t numPrims;              /* spheres, cones, cylinders, curves */
  const float *prims;            /* 16 floats each, object space: sphere (center, radius, -);
                                    cone / cylinder (v1, r1, v2, r2, -); curve (w0, r, w1, -,
                                    w2, -, w3, -) */
  const int32_t *primKind;       /* 0 sphere, 1 cone, 2 cylinder, 3 Bezier curve */
  const uint32_t *primSurface;   /* surface index per primitive */
  const int32_t *triNormalFrom;  /* per triangle: the triangle whose e1 x e2 is its shading
                                    normal (quads), -1 for its own; may be null */
  int32_t numIsos;
  const OrIso *isos;
  const OrVolume *isoFields;     /* one per iso-surface */
  const OrSurfAttr *surfAttr;    /* per surface, or null: no attributes in the scene */
  int32_t numSamplers;
  const OrSampler *samplers;
} OrScene;

typedef struct OrCamera {
  int32_t type;
  float position[3], direction[3], up[3];
  float fovy, aspect;
  float apertureRadius, focusDistance;
  float imageRegion[4];      /* min.x, min.y, max.x, max.y */
  float shutter[2];
  float height;              /* orthographic */
  float view[16], proj[16];  /* matrix camera, column-major */
} OrCamera;

typedef struct OrRenderer {
  int32_t type;
  float background[4];
  float ambientColor[3];
  float ambientRadiance;
  float occlusionDistance;
  int32_t ambientSamples;
  int32_t maxBounce;
  int32_t pixelSamples;
  float volumeSamplingRate;
  int32_t numClipPlanes;
  const float *clipPlanes;   /* float4 (n.xyz, d) each */
  int32_t gradientShading;   /* volume samples lit along the field gradient */
  int32_t taa;               /* temporal anti-aliasing (path tracer) */
  float taaAlpha;            /* weight of the new frame in the TAA blend */
} OrRenderer;

typedef struct OrFrame {
  int32_t width, height;
  int32_t accumID;           /* in/out: incremented by or_render_frame */
  int32_t colorType;         /* OR_COLOR_* */
  void *color;               /* float4 or uint32 per pixel */
  float *depth;
  float *normal;             /* float3 */
  float *albedo;             /* float3 */
  float *accum;              /* float4 accumulation buffer */
  double *sampleSum;         /* optional: per-pixel sum of sample rgb (3 doubles) */
  double *sampleSumSq;       /* optional: per-pixel sum of squares (3 doubles) */
  int32_t rowBegin, rowEnd;  /* render rows [rowBegin,rowEnd) only (0,0 = all) */
  int32_t tileSize;          /* square pixel tiles handed to the threads (0 = 64, as
                                the reference CPU device); results do not depend on it */
  /* TAA (renderer taa): this frame's colour, the previous resolved image,
     the closest samples' albedo (float3) now and before, motion vectors
     (float2) per pixel; the previous and current view-projection matrices
     (column-major, in/out: the current one becomes the previous one after
     each frame; identity at first) */
  float *taaCurr, *taaPrev, *taaCurrAlbedo, *taaPrevAlbedo, *motionVec;
  float prevMVP[16], currMVP[16];
} OrFrame;

typedef struct OrStats {
  uint64_t rays;             /* traversals started */
  uint64_t nodeVisits;       /* BVH inner-node visits */
  uint64_t triTests;         /* ray/triangle tests */
  uint64_t marchSamples;     /* rayMarchVolume samples taken */
  uint64_t trackingSamples;  /* delta-tracking tentative collisions */
  uint64_t cellsVisited;     /* DDA cells visited */
} OrStats;

/* Build the per-group BVHs and majorant grids; arrays must outlive the handle. */
void *or_scene_commit(const OrScene *scene);
void or_scene_release(void *handle);

/* Clear the accumulation buffer and set depth to 1e31, accumID = 0
   (frame/Frame.cpp:287-312). */
void or_frame_reset(OrFrame *frame);

/* Render one frame (frame/Frame.cpp:215-397 minus the device plumbing).
   numThreads <= 0 uses std::thread::hardware_concurrency(). */
int or_render_frame(void *scene, const OrCamera *cam, const OrRenderer *rend,
                    OrFrame *frame, int numThreads, OrStats *stats);

/* ---- unit-level entry points used by the oracle's own tests ---- */
void or_lcg_sequence(uint32_t v0, uint32_t v1, int n, float *out);
float or_sample_field(const OrVolume *vol, float px, float py, float pz);
void or_tf_lookup(const OrVolume *vol, float v, float *rgba);
void or_primary_ray(const OrCamera *cam, float x, float y, float w, float h,
                    uint32_t seed0, uint32_t seed1, float *ori, float *dir);
void or_eval_material(const OrMaterial *mat, const float *Ng, const float *Ns,
                      const float *viewDir, const float *lightDir, float *out);
/* Draws from an LCG seeded (seed0,seed1); writes dir[3], f[3], pdf, cosT. */
void or_sample_material(const OrMaterial *mat, const float *Ng, const float *Ns,
                        const float *viewDir, uint32_t seed0, uint32_t seed1,
                        float *dir, float *f, float *pdf, float *cosT);
/* Majorant grid of volume `vol` of a committed scene: writes dims and up to
   maxCells floats; returns the cell count. */
int or_majorants(void *scene, int vol, int32_t *dims, float *out, int maxCells);
/* DDA over a grid: writes visited cell ids and [t0,t1] pairs; returns count. */
int or_dda(const float *ori, const float *dir, float tmin, float tmax,
           const int32_t *dims, const float *boundsLo, const float *boundsHi,
           int32_t *cells, float *t01, int maxCells);
/* Colour conversion of n float4 colours to packed RGBA8 (srgb != 0: the
   sRGB-encoded variant), as the frame's UFIXED8 / sRGB8 colour formats. */
void or_cvt(const float *rgba, int n, int srgb, uint32_t *out);
/* Closest hit through the committed scene: returns 1 on hit. */
int or_trace(void *scene, const float *ori, const float *dir, float tmin, float tmax,
             float *t, uint32_t *inst, uint32_t *tri, float *uv);

#ifdef __cplusplus
}
#endif

#endif
