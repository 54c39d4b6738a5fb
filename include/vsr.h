/* vsr.h — C ABI of the GB300 renderer core behind the anari-visionaray
 * "raycast" and "pathtracer" per-pixel hot path.
 *
 * Each entry point is the counterpart of one call of the ANARI API that the
 * reference device implements; the reference site it replaces is cited
 * beside it. Object model, parameter names and channel names follow the
 * reference device (VisionarayDevice.cpp:59-214, frame/Frame.cpp:75-94).
 * The ANARI SDK headers are not part of this build, so data-type values are
 * this library's own (VSR_*), named after the ANARI_* type they stand for.
 *
 * Errors: every call returns a VSRStatus (0 = success) and reports problems
 * through the device's status callback with a severity, as the reference
 * reports them through reportMessage (e.g. frame/Frame.cpp:98-110).
 * Rendering is asynchronous on one CUDA stream; vsrFrameReady waits on the
 * frame's completion event (frame/Frame.cpp:474-497).
 */
#ifndef VSR_H
#define VSR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define VSR_API __declspec(dllexport)
#else
#define VSR_API __attribute__((visibility("default")))
#endif

typedef struct VSRDevice_ *VSRDevice;
typedef struct VSRObject_ *VSRObject;
typedef VSRObject VSRArray;
typedef VSRObject VSRFrame;

typedef enum VSRStatus {
  VSR_OK = 0,
  VSR_ERROR_INVALID_ARGUMENT = 1,
  VSR_ERROR_INVALID_OBJECT = 2,
  VSR_ERROR_UNKNOWN_SUBTYPE = 3,
  VSR_ERROR_OUT_OF_MEMORY = 4,
  VSR_ERROR_CUDA = 5,
  VSR_ERROR_INCOMPLETE = 6,
  VSR_ERROR_TIMEOUT = 7,
  VSR_ERROR_LIMIT_EXCEEDED = 8
} VSRStatus;

typedef enum VSRSeverity {
  VSR_SEVERITY_FATAL_ERROR = 1,
  VSR_SEVERITY_ERROR = 2,
  VSR_SEVERITY_WARNING = 3,
  VSR_SEVERITY_PERFORMANCE_WARNING = 4,
  VSR_SEVERITY_INFO = 5,
  VSR_SEVERITY_DEBUG = 6
} VSRSeverity;

typedef enum VSRDataType {
  VSR_UNKNOWN = 0,
  VSR_STRING = 1,
  VSR_OBJECT = 2,
  VSR_ARRAY1D = 3,
  VSR_ARRAY2D = 4,
  VSR_ARRAY3D = 5,
  VSR_CAMERA = 6,
  VSR_FRAME = 7,
  VSR_GEOMETRY = 8,
  VSR_GROUP = 9,
  VSR_INSTANCE = 10,
  VSR_LIGHT = 11,
  VSR_MATERIAL = 12,
  VSR_RENDERER = 13,
  VSR_SURFACE = 14,
  VSR_SPATIAL_FIELD = 15,
  VSR_VOLUME = 16,
  VSR_WORLD = 17,
  VSR_DATA_TYPE = 18,      /* a VSRDataType value, e.g. for "channel.color" */
  VSR_BOOL = 19,
  VSR_INT32 = 20,
  VSR_UINT32 = 21,
  VSR_INT32_VEC2 = 22,
  VSR_UINT32_VEC2 = 23,
  VSR_UINT32_VEC3 = 24,
  VSR_FLOAT32 = 25,
  VSR_FLOAT32_VEC2 = 26,
  VSR_FLOAT32_VEC3 = 27,
  VSR_FLOAT32_VEC4 = 28,
  VSR_FLOAT32_BOX1 = 29,
  VSR_FLOAT32_MAT4 = 30,   /* column-major 4x4 */
  VSR_FLOAT32_MAT3x4 = 31, /* column-major 3x4 affine */
  VSR_UFIXED8 = 32,
  VSR_UFIXED8_VEC4 = 33,
  VSR_UFIXED8_RGBA_SRGB = 34,
  VSR_UFIXED16 = 35,
  VSR_FLOAT64_BOX1 = 36,
  VSR_UINT64 = 37,
  VSR_FLOAT64 = 38,
  VSR_UINT32_VEC4 = 39,
  VSR_SAMPLER = 40,
  VSR_UFIXED8_VEC2 = 41,
  VSR_UFIXED8_VEC3 = 42
} VSRDataType;

typedef enum VSRWaitMask { VSR_NO_WAIT = 0, VSR_WAIT = 1 } VSRWaitMask;

typedef void (*VSRStatusCallback)(const void *userPtr, VSRDevice device, VSRObject source,
                                  VSRDataType sourceType, VSRSeverity severity,
                                  VSRStatus code, const char *message);

/* Device creation; replaces anariNewVisionarayDevice (VisionarayLibrary.cpp:69-73)
   and the device-level parameters of deviceCommitParameters
   (VisionarayDevice.cpp:354-391). subtype "default" selects the current
   CUDA device, or the one named by the VISIONARAY_CUDA_DEVICE environment
   variable as in the reference (VisionarayDevice.cpp:373-380). Returns NULL
   (and reports VSR_ERROR_CUDA) when no CUDA device is present: there is no
   CPU fallback. */
VSR_API VSRDevice vsrNewDevice(const char *subtype, VSRStatusCallback cb, const void *cbUserPtr);
VSR_API VSRStatus vsrReleaseDevice(VSRDevice device);

/* Arrays; replace newArray1D/2D/3D (VisionarayDevice.cpp:59-122). The data is
   copied at creation (the reference copies into HostDeviceArrays on commit). */
VSR_API VSRArray vsrNewArray1D(VSRDevice d, const void *appMemory, VSRDataType type, uint64_t n1);
VSR_API VSRArray vsrNewArray2D(VSRDevice d, const void *appMemory, VSRDataType type, uint64_t n1,
                               uint64_t n2);
VSR_API VSRArray vsrNewArray3D(VSRDevice d, const void *appMemory, VSRDataType type, uint64_t n1,
                               uint64_t n2, uint64_t n3);

/* Object factories; replace newSpatialField/newVolume/newGeometry/newMaterial/
   newLight/newSurface/newGroup/newInstance/newWorld/newCamera/newRenderer/
   newFrame (VisionarayDevice.cpp:125-214). Supported subtypes:
   spatial field "structuredRegular"; volume "transferFunction1D";
   geometry "triangle", "quad", "sphere", "cone", "cylinder", "isosurface",
   "bezierCurve";
   material "matte", "physicallyBased"; light "directional", "point",
   "spot", "quad", "hdri"; instance "transform"; camera "perspective",
   "matrix", "orthographic", "omnidirectional"; renderer "raycast",
   "pathtrace", "default" (= pathtrace, renderer/Renderer.cpp:144-152).
   Unknown subtypes return NULL and report VSR_ERROR_UNKNOWN_SUBTYPE. */
VSR_API VSRObject vsrNewSpatialField(VSRDevice d, const char *subtype);
VSR_API VSRObject vsrNewVolume(VSRDevice d, const char *subtype);
VSR_API VSRObject vsrNewGeometry(VSRDevice d, const char *subtype);
VSR_API VSRObject vsrNewMaterial(VSRDevice d, const char *subtype);
VSR_API VSRObject vsrNewLight(VSRDevice d, const char *subtype);
VSR_API VSRObject vsrNewSurface(VSRDevice d);
VSR_API VSRObject vsrNewGroup(VSRDevice d);
VSR_API VSRObject vsrNewInstance(VSRDevice d, const char *subtype);
VSR_API VSRObject vsrNewWorld(VSRDevice d);
VSR_API VSRObject vsrNewCamera(VSRDevice d, const char *subtype);
VSR_API VSRObject vsrNewRenderer(VSRDevice d, const char *subtype);
/* Samplers (newSampler, VisionarayDevice.cpp:125-214; scene/surface/
   material/sampler): "image1D", "image2D", "image3D" (image: Array1D / 2D /
   3D of FLOAT32 (VEC2/3/4) or UFIXED8 (VEC2/3/4, RGBA_SRGB) texels, stored
   as RGBA8; inAttribute, filter "linear" | "nearest", wrapMode1..3
   "clampToEdge" | "repeat" | "mirrorRepeat", inTransform / outTransform
   (FLOAT32_MAT4), inOffset / outOffset (FLOAT32_VEC4)), "transform"
   (inAttribute, outTransform, outOffset) and "primitive" (array, offset).
   A material's color / baseColor, opacity, metallic and roughness take a
   sampler object, an attribute name (STRING: "attribute0".."attribute3",
   "color", "worldPosition", "worldNormal", "objectPosition",
   "objectNormal") or a value. */
VSR_API VSRObject vsrNewSampler(VSRDevice d, const char *subtype);
VSR_API VSRFrame vsrNewFrame(VSRDevice d);

/* Parameters; replace anariSetParameter/anariUnsetParameter/
   anariCommitParameters (helium BaseObject, used by every commitParameters()
   in the reference). Object-valued parameters pass a pointer to the handle;
   VSR_STRING passes the C string itself. Parameter names and defaults are
   the reference's (e.g. renderer/Pathtrace.cpp:16-28, renderer/Raycast.cpp:16-20,
   renderer/Renderer.cpp:34-45, camera/Camera.cpp:30-36). */
VSR_API VSRStatus vsrSetParameter(VSRDevice d, VSRObject o, const char *name, VSRDataType type,
                                  const void *mem);
VSR_API VSRStatus vsrUnsetParameter(VSRDevice d, VSRObject o, const char *name);
VSR_API VSRStatus vsrCommitParameters(VSRDevice d, VSRObject o);
VSR_API VSRStatus vsrRelease(VSRDevice d, VSRObject o);
VSR_API VSRStatus vsrRetain(VSRDevice d, VSRObject o);

/* Properties; replace anariGetProperty (frame/Frame.cpp:171-213): frame
   "duration" (FLOAT32, seconds of GPU time of the last render),
   "duration.render" (FLOAT32, render kernel only), "numSamples" (INT32),
   "commitDuration" (FLOAT32, seconds of the last scene update incl. BVH
   build), "errorFlags" (UINT32, device-side error bits of the last render:
   1 traversal stack full, 2 DDA step limit, 4 delta-tracking step limit,
   8 path pass limit, 16 ray-march step limit, 32 transparent-layer limit,
   64 a NaN or infinite path sample was dropped), "march.unitsNeeded" and
   "march.unitCapacity" (UINT32, volume-only raycast frames: the work units
   of 32 ray segments the last frame needed, and the frame's unit list
   size, which grows to the need of the frame before); world "bvh.nodes" /
   "bvh.triangles" (UINT64). Frame channel "channel.variance" (FLOAT32, an
   extension) holds the path tracer's variance of each pixel's accumulated
   mean luminance. Returns 1 if found. */
VSR_API int vsrGetProperty(VSRDevice d, VSRObject o, const char *name, VSRDataType type,
                           void *mem, uint64_t size, VSRWaitMask mask);

/* Rendering; replaces anariRenderFrame / anariFrameReady / anariDiscardFrame
   (Frame::renderFrame frame/Frame.cpp:215-397, Frame::wait :474-497). */
VSR_API VSRStatus vsrRenderFrame(VSRDevice d, VSRFrame f);
VSR_API int vsrFrameReady(VSRDevice d, VSRFrame f, VSRWaitMask mask);
VSR_API VSRStatus vsrDiscardFrame(VSRDevice d, VSRFrame f);

/* vsrRenderFrames has no counterpart in the reference (which renders one
   frame per anariRenderFrame call). It renders `count` distinct frames, of
   any scenes, cameras, renderers and sizes, as one batch: each frame gets
   what vsrRenderFrame would do to it (accumulation reset after commits,
   sampleLimit, one more accumulated frame) and the same image, but all
   frames' pixels are drawn from shared work lists by persistent kernels,
   replayed as one CUDA graph per frame set. Successive batches of the same
   frame set try the tile shapes and fetch sizes of a built-in autotuner and
   then keep the fastest (frame properties batch.tileWidth, batch.fetch,
   batch.tuned). Frames collecting statistics are rendered one by one.
   Completion: vsrFrameReady on any of the frames. */
VSR_API VSRStatus vsrRenderFrames(VSRDevice d, const VSRFrame *frames, uint32_t count);

/* Learned denoiser (no counterpart in the reference): a 4-level U-Net of
   3x3 convolutions (32/64/128/256 channels, ~1.9M parameters), bf16
   weights and activations with fp32 accumulation, trained and run by this
   library's own kernels. Network images are N x H x W pixels, H and W
   multiples of 8, NHWC: input 16 bf16 channels (log(1 + colour), albedo,
   normal, depth / (1 + depth), log(1 + standard error of the mean
   luminance) from the variance channel, 1 / sqrt(samples per pixel), four
   zeros), output 16 fp32 channels whose
   first three are log(1 + colour): the input's plus a learned correction. Pointers to images are device pointers;
   work runs on the device's stream (vsrDeviceStream). */
typedef struct VSRDenoiser_ *VSRDenoiser;
VSR_API VSRDenoiser vsrNewDenoiser(VSRDevice d, uint64_t seed);
VSR_API VSRStatus vsrReleaseDenoiser(VSRDevice d, VSRDenoiser n);
VSR_API uint64_t vsrDenoiserParameterCount(VSRDevice d, VSRDenoiser n);
/* Parameters in layer order (weights [cout][3][3][cin], then bias), as fp32
   host arrays of vsrDenoiserParameterCount floats; setting them restarts
   the optimiser. */
VSR_API VSRStatus vsrDenoiserGetParameters(VSRDevice d, VSRDenoiser n, float *params,
                                           uint64_t count);
/* Which tensor-core path the convolutions take: 0 warp-level mma.sync,
   1 tcgen05 with the accumulators in tensor memory, on a persistent
   warp-specialised kernel with TMA loads, for levels at least 128 pixels
   wide (mma.sync below), 2 (default) the same kernel at every width, 3 as
   1 on a kernel that stages one tile per CTA with cp.async, 4 as 2 with
   the training's weight gradients on tcgen05 too (accumulated in tensor
   memory over pixel ranges, summed without atomics; slower than the
   mma.sync weight gradient at the training's crop sizes). On the
   tcgen05 path the forward reads each decoder's upsampled input and skip
   connection in place instead of writing their concatenation.
   vsrDenoiserErrors returns the device error word of the tcgen05 path
   (value 1: a bounded wait on the tensor core, a load or another role ran
   out; that launch ended early and its layer's output is undefined), 0
   when all is well, and clears it (0xffffffff if it cannot be read).
   vsrDenoiserTestWaitTimeout arms a test of that failure path for the next
   tcgen05 convolution launch only: the MMA thread of each CTA first waits
   on a barrier that nothing completes, its wait runs out after one second,
   and the launch ends early with error word 1 (no GPU fault; the device
   stays usable). Not in the reference (it has no denoiser). */
VSR_API VSRStatus vsrDenoiserSetTensorPath(VSRDevice d, VSRDenoiser n, int path);
VSR_API uint32_t vsrDenoiserErrors(VSRDevice d, VSRDenoiser n);
VSR_API VSRStatus vsrDenoiserTestWaitTimeout(VSRDevice d, VSRDenoiser n);
VSR_API VSRStatus vsrDenoiserSetParameters(VSRDevice d, VSRDenoiser n, const float *params,
                                           uint64_t count);
VSR_API VSRStatus vsrDenoiserForward(VSRDevice d, VSRDenoiser n, const void *input, uint32_t N,
                                     uint32_t H, uint32_t W, float *output);
/* L1 loss of log(1 + colour) against a linear target colour (targetStride
   floats per pixel, first three used). vsrDenoiserGradients returns the
   loss and the fp32 parameter gradients (host, `count` floats) without
   changing the network; vsrDenoiserTrainStep applies one Adam step (beta
   0.9 / 0.999, eps 1e-8) at the given learning rate. loss may be null. */
VSR_API VSRStatus vsrDenoiserGradients(VSRDevice d, VSRDenoiser n, const void *input,
                                       const float *target, uint32_t targetStride, uint32_t N,
                                       uint32_t H, uint32_t W, float *grads, uint64_t count,
                                       float *loss);
VSR_API VSRStatus vsrDenoiserTrainStep(VSRDevice d, VSRDenoiser n, const void *input,
                                       const float *target, uint32_t targetStride, uint32_t N,
                                       uint32_t H, uint32_t W, float learningRate, float *loss);
/* The network input of a frame (its accumulated colour, albedo, normal and
   depth channels; absent channels read as zero), W8 x H8 pixels with W8, H8
   the frame size rounded up to multiples of 8. */
VSR_API VSRStatus vsrDenoiserFrameInput(VSRDevice d, VSRFrame f, void *input);
/* Denoise a frame: the network on its accumulated image, then the variance
   gate: a pixel keeps the denoised colour when |lum(denoised) - lum(mean)|
   <= k * sqrt(variance of the mean) + floorAbs, else the accumulated mean,
   and is marked for more samples (retry: one byte per pixel, device, may be
   null). Without a variance channel on the frame every pixel takes the
   denoised colour. colorOut: device float4 per pixel; numRetry: host, may be
   null. With numRetry the call waits for the pass and returns
   VSR_ERROR_TIMEOUT (also through the status callback) when a bounded wait
   of a tcgen05 convolution ran out (vsrDenoiserErrors); without it the call
   returns once the work is enqueued. */
VSR_API VSRStatus vsrDenoiseFrame(VSRDevice d, VSRDenoiser n, VSRFrame f, float k,
                                  float floorAbs, float *colorOut, uint8_t *retry,
                                  uint32_t *numRetry);

/* Per-pixel sample mask of a frame's path tracer (no counterpart in the
   reference): one byte per pixel in device memory (the caller's, e.g. the
   retry mask of vsrDenoiseFrame), null for every pixel. Following renders
   of the path tracer take samples only for pixels whose byte is nonzero;
   the others keep their colour, accumulation and G-buffer. Setting it does
   not restart accumulation. From the first mask on, the frame counts the
   frames accumulated in each pixel (starting from those accumulated so
   far), and each pixel's running mean and variance weight its own count,
   so masks may change between renders. A committed frame size change drops
   the mask. The denoiser's 1/sqrt(samples) input stays the frame-wide
   value. The raycast renderer ignores the mask. The buffer must stay valid
   while renders that use it run. */
VSR_API VSRStatus vsrFrameSampleMask(VSRDevice d, VSRFrame f, const uint8_t *mask);

/* Work list of a batch, without a device (vsrPlanBatch has no counterpart in
   the reference): tiles of tileWidth x (32 / tileWidth) pixels for jobs of
   the given sizes, as (job, tile) uint32 pairs ordered by cost per pixel,
   highest first, all tiles of a job together. Writes at most `capacity`
   pairs to `items` (may be null) and returns the number of pairs; 0 for a
   tileWidth that does not divide 32. */
VSR_API uint64_t vsrPlanBatch(const uint32_t *width, const uint32_t *height,
                              const float *costPerPixel, uint32_t numJobs, uint32_t tileWidth,
                              uint32_t *items, uint64_t capacity);

/* Mapping; replaces anariMapFrame / anariUnmapFrame (frame/Frame.cpp:399-447).
   Channels: "channel.color", "channel.depth", "channel.normal",
   "channel.albedo". Returns a host pointer valid until the next render or
   unmap; the copy from device memory happens inside this call. On failure
   (channel not enabled, no pinned host buffer, a failed copy) returns NULL
   with width = height = 0, reported through the status callback
   (VSR_ERROR_INVALID_ARGUMENT, VSR_ERROR_OUT_OF_MEMORY, VSR_ERROR_CUDA). */
VSR_API const void *vsrMapFrame(VSRDevice d, VSRFrame f, const char *channel, uint32_t *width,
                                uint32_t *height, VSRDataType *pixelType);
VSR_API VSRStatus vsrUnmapFrame(VSRDevice d, VSRFrame f, const char *channel);

/* Device-resident view of a channel (no copy): the CUDA device pointer of
   the frame buffer, for consumers that stay on the GPU. Same channels as
   vsrMapFrame. Not in the reference (its frame buffers are pinned host
   memory, DeviceArray.h:50). */
VSR_API const void *vsrMapFrameDevice(VSRDevice d, VSRFrame f, const char *channel,
                                      uint32_t *width, uint32_t *height, VSRDataType *pixelType);

/* The CUDA stream the device renders on (cudaStream_t), so that callers can
   order their own GPU work against frames. */
VSR_API void *vsrDeviceStream(VSRDevice d);

/* Device-side BVH build for a triangle set whose data already lives in GPU
   memory; replaces DeviceBVH<basic_triangle>::update + deviceIndexBVH2
   (DeviceBVH.h:51-55, :266-335), which the reference's Triangle::finalize
   calls (scene/surface/geometry/Triangle.cpp:200-206).
     v1, e1, e2 : device pointers, n packed float3 each (e1 = v2-v1,
                  e2 = v3-v1, Triangle.cpp:76-83)
     nodesOut   : device pointer, 4*max(n-1,1) float4 (64-byte BVH2 nodes)
     trisOut    : device pointer, 3*n float4 (leaf-ordered triangles)
     stream     : cudaStream_t to run on (NULL = legacy default stream)
   Temporary device memory is taken from the stream-ordered allocator and
   returned before the call completes on the stream. The call returns once
   the work is enqueued. Returns VSR_OK, VSR_ERROR_INVALID_ARGUMENT or
   VSR_ERROR_CUDA. Requires n < 2^27. */
VSR_API VSRStatus vsrBuildTriangleBVH(const float *v1, const float *e1, const float *e2,
                                      uint32_t n, void *nodesOut, void *trisOut, void *stream);

/* vsrBuildTriangleBVHNoAlloc has no counterpart in the reference. It is the
   same device BVH build as vsrBuildTriangleBVH (same arguments, bit-identical
   output) for callers that cannot let a library allocate GPU memory: a host
   application that owns a fixed GPU memory budget and only passes in buffers
   it allocated itself, or a per-frame loop that must not risk an allocation
   or a free (a free can synchronize the whole device) mid-frame. It calls no
   cudaMalloc, cudaFree or other allocating routine.
   Limit: n <= VSR_BVH_NOALLOC_MAX_TRIANGLES; a larger n returns
   VSR_ERROR_LIMIT_EXCEEDED and does nothing.
   Temporaries live in one 8 MiB buffer in the library's device data, held by
   every GPU that loads the library until the process exits. All calls on a
   device share it and it keeps the last call's contents (each call clears
   what must start at zero). Calls that overlap on the GPU race on the buffer
   and corrupt each other's result: order them (one stream, or events).
   The first call on each device, made with that device current, looks up
   the buffer's device address; make that first call before any stream
   capture. Every later call made outside stream capture looks the address
   up again (a lookup, no allocation), so a cudaDeviceReset or a re-created
   primary context between calls does not leave a stale address. */
#define VSR_BVH_NOALLOC_MAX_TRIANGLES 65536u
VSR_API VSRStatus vsrBuildTriangleBVHNoAlloc(const float *v1, const float *e1, const float *e2,
                                             uint32_t n, void *nodesOut, void *trisOut,
                                             void *stream);

#ifdef __cplusplus
}
#endif

#endif
