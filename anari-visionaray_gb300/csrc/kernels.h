// Host-side launch entry points of the CUDA kernels (called by runtime.cpp).
#pragma once

#include "vsr_device.h"
#include <cuda_runtime.h>
#include <stddef.h>

namespace vsr {

// Device scratch of the segmented marcher for volume-only raycast worlds at
// one sample per pixel (k_volume_march.cu): items 48 B per pixel, groups
// 16 B per 32 pixels, counters 4 uint, and unitCap work units of 32
// segments (unitGroup 4 B and segOut 1 KiB per unit).
struct MarchScratch {
  void *items;
  void *groups;
  unsigned *counters;
  int *unitGroup;
  void *segOut;
  unsigned unitCap;
};
// scratch null selects the per-pixel kernel for volume-only worlds too
cudaError_t launchRaycast(const DScene &S, const DCamera &C, const DRenderer &R, const DFrame &F,
                          int stageTFSize, bool count, const MarchScratch *scratch,
                          cudaStream_t stream);
cudaError_t launchVolumeMarch(const DScene &S, const DCamera &C, const DRenderer &R,
                              const DFrame &F, int stageTFSize, bool count,
                              const MarchScratch &M, cudaStream_t stream);
cudaError_t launchPathtrace(const DScene &S, const DCamera &C, const DRenderer &R, const DFrame &F,
                            bool count, cudaStream_t stream);

// Wavefront path tracer (same per-pixel random stream as launchPathtrace):
// init + iterations of trace/shade over compacted pixel queues until every
// pixel has finished its pixelSamples samples. pinnedCount is a host-pinned
// uint32 used to poll the queue size between batches of iterations.
cudaError_t launchPathtraceWavefront(const DScene &S, const DCamera &C, const DRenderer &R,
                                     const DFrame &F, const DWave &Wv, uint32_t *pinnedCount,
                                     bool count, cudaStream_t stream, int *iterations);

// Batched rendering (k_batch.cu). A job is one frame's records; kinds are
// rendered by separate persistent kernels, each over its own work list of
// (job, tile) items with tiles of tileW x (32 / tileW) pixels.
enum JobKind { JOB_PATHTRACE = 0, JOB_RAYCAST_SURFACES = 1, JOB_RAYCAST_VOLUME = 2, kJobKinds = 3 };
struct DJob {
  DScene S;
  DCamera C;
  DRenderer R;
  DFrame F;
  int kind;
  int tilesX;
  int reset;  // restart accumulation before rendering
  int pad;
};
struct BatchLaunch {
  const DJob *jobs;
  int numJobs;
  const uint2 *items[kJobKinds];
  unsigned numItems[kJobKinds];
  unsigned *counters;  // kJobKinds work counters
  int tileW;           // 1..32, a divisor of 32
  int fetch;           // items per atomic
};
cudaError_t launchBatch(const BatchLaunch &L, cudaStream_t stream);

// Accumulation reset: accum = 0, depth = 1e31 (frame/Frame.cpp:287-312).
cudaError_t launchFrameReset(float4 *accum, float *depth, size_t numPixels, cudaStream_t stream);

// Brick majorant grid of a structured volume: one cell per brick of
// `brick` voxels per edge; majorant = max TF alpha over the TF bins that the
// brick's texel value range can reach under trilinear + linear TF filtering.
cudaError_t launchBrickMajorants(const float *field, const int dims[3], int brick,
                                 const float4 *tf, int tfSize, float vrMin, float vrMax,
                                 float *outMajorant, const int gdims[3], cudaStream_t stream);

// On-device LBVH build (63-bit Morton codes, Karras-style hierarchy,
// bottom-up refit) for one group's triangles.
//   v1/e1/e2 : device float3-packed arrays, n triangles (local order)
//   nodesOut : 4*max(n-1,1) float4 (BVH2 node layout of vsr_device.h)
//   trisOut  : 3*n float4 in leaf order
// Temporary device memory is allocated internally. Returns cudaSuccess or
// the first CUDA error.
struct BvhBuildStats {
  int numNodes;
  float buildMs;
};
cudaError_t buildGroupBVH(const float *v1, const float *e1, const float *e2, int n,
                          float4 *nodesOut, float4 *trisOut, BvhBuildStats *stats,
                          cudaStream_t stream);

// Collapse a BVH2 (traversal layout, root 0) into a BVH4 (layout above):
// each BVH4 node opens the largest-area inner child until it holds four
// children. nodes4Out needs room for numNodes2 BVH4 nodes. Leaf codes and
// the leaf-ordered triangles are unchanged. Returns the BVH4 node count in
// *numNodes4 (synchronizes the stream).
cudaError_t collapseBVH4(const float4 *nodes2, int numNodes2, float4 *nodes4Out, int *numNodes4,
                         cudaStream_t stream);

// Same inputs/outputs, PLOC clustering instead of the Karras hierarchy:
// tighter boxes (close to a greedy SAH build), a few ms more per 1M
// triangles. Used for world commits unless the world asks for "fast".
cudaError_t buildGroupBVHQuality(const float *v1, const float *e1, const float *e2, int n,
                                 float4 *nodesOut, float4 *trisOut, BvhBuildStats *stats,
                                 cudaStream_t stream);

} // namespace vsr
