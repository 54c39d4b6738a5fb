// Host-side launch entry points of the CUDA kernels (called by runtime.cpp).
#pragma once

#include "vsr_device.h"
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stddef.h>

namespace vsr {

// Device scratch of the segmented marcher for volume-only raycast worlds at
// one sample per pixel (k_volume_march.cu): items 48 B per pixel, groups
// 16 B per 32 pixels, counters 4 uint, and unitCap work units of 32
// segments (unitGroup 4 B and segOut 1 KiB per unit).
// samples per segment of the segmented volume marcher (k_volume_march.cu);
// the work-unit capacity of MarchScratch scales with it
#ifndef VSR_SEG_SAMPLES
#define VSR_SEG_SAMPLES 12
#endif
struct MarchScratch {
  void *items;
  void *groups;
  unsigned *counters;
  int *unitGroup;
  void *segOut;
  unsigned unitCap;
  unsigned *groupDone;  // per group: its work units finished (fused combination)
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
enum JobKind {
  JOB_PATHTRACE = 0,
  JOB_RAYCAST_SURFACES = 1,
  JOB_RAYCAST_VOLUME = 2,
  JOB_RAYCAST_FULL = 3,  // raycast with gradient shading or point / spot lights
  kJobKinds = 4
};
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
  int pathtraceVariant;  // bit 0: a path-traced job's world has volumes (the 64-register
                         // kernel); bit 1: a job uses gradient shading or point / spot lights
};
cudaError_t launchBatch(const BatchLaunch &L, cudaStream_t stream);

// Denoiser kernels (k_denoise.cu). Activations are bf16 in channel-blocked
// planes: element (pixel p, channel c) of a tensor of P pixels (N x H x W,
// row-major) is at ((c / 8) P + p) 8 + c % 8, so that 8 channels of a pixel
// are 16 contiguous bytes and a row of pixels of one 8-channel block is
// contiguous. A tensor view is (pointer, channels of the buffer, first
// channel), both multiples of 8; the pixel count is that of the resolution
// the view is used at. Convolution weights are [Cout][9][Cin] bf16 (tap =
// 3 (dy + 1) + dx + 1), biases fp32.
__host__ __device__ inline size_t actAt(size_t P, size_t p, int c) {
  return ((size_t)(c >> 3) * P + p) * 8 + (size_t)(c & 7);
}
struct ConvArgs {
  const __nv_bfloat16 *x;
  int xC, xOff, Cin;  // Cin a multiple of 16
  const __nv_bfloat16 *w;
  const float *bias;  // or null
  int Cout;
  __nv_bfloat16 *y;   // bf16 output, or
  float *yf;          // fp32 output
  int yC, yOff;
  const __nv_bfloat16 *mask;  // zero outputs where mask <= 0 (a ReLU's backward), or null
  int maskC, maskOff;
  int relu;
  int N, H, W;
  const __nv_bfloat16 *resid;  // added to output channels [0, residN), or null
  int residC, residN;
  // tcgen05 path only: input channels [split, Cin) come from x2 (x2C
  // channels per pixel, from x2Off), channels [0, split) from x; with up, x
  // is at half resolution and is read at (y / 2, x / 2) (nearest 2x
  // upsampling). split a multiple of 32; 0: every channel from x.
  const __nv_bfloat16 *x2;
  int x2C, x2Off, split, up;
  // the weights packed for kConv3x3Ws (packConvWeights), or null
  const __nv_bfloat16 *wPacked;
  // tcgen05 kernels, for tests of the timeout path only (0 otherwise): the
  // MMA role of every CTA first waits on a barrier that nothing completes,
  // so that its bounded wait runs out and the launch ends early with error
  // word 1 and no output
  int testStall;
};
struct WgradArgs {
  const __nv_bfloat16 *dy;  // output gradient (after the ReLU mask)
  int dyC, dyOff, Cout;     // Cout a multiple of 8
  const __nv_bfloat16 *x;   // layer input
  int xC, xOff, Cin;        // Cin a multiple of 8
  float *dw;                // [Cout][9][Cin], accumulated
  int N, H, W;
  int chunk;                // pixels per CTA
};
cudaError_t launchConv3x3(const ConvArgs &a, cudaStream_t s);
// the same convolution on tcgen05 (k_denoise_tc.cu); error: a device word
// that gets bit 1 if a bounded wait ran out
cudaError_t launchConv3x3Tc(const ConvArgs &a, unsigned *error, cudaStream_t s);
// the same on a persistent warp-specialised kernel with TMA loads
// (k_denoise_ws.cu); split requires up
cudaError_t launchConv3x3Ws(const ConvArgs &a, unsigned *error, cudaStream_t s);
cudaError_t launchConvWgrad(const WgradArgs &a, cudaStream_t s);
// the weight gradient on tcgen05 (k_denoise_wg.cu): per-CTA partial sums in
// `part` (wgradPartFloats floats), then added into dw in a fixed order;
// error: a device word that gets bit 1 if a bounded wait ran out
cudaError_t launchConvWgradTc(const WgradArgs &a, float *part, unsigned *error, cudaStream_t s);
size_t wgradPartFloats(int Cout, int Cin, int P);
cudaError_t launchBiasGrad(const __nv_bfloat16 *dy, int dyC, int dyOff, int C, int P, float *db,
                           cudaStream_t s);
cudaError_t launchMaxPool(const __nv_bfloat16 *x, int C, int N, int H, int W, __nv_bfloat16 *y,
                          cudaStream_t s);
cudaError_t launchMaxPoolGrad(const __nv_bfloat16 *x, const __nv_bfloat16 *dy, int C, int N, int H,
                              int W, const __nv_bfloat16 *mask, __nv_bfloat16 *dx, cudaStream_t s);
cudaError_t launchUpsample(const __nv_bfloat16 *x, int C, int N, int H, int W, __nv_bfloat16 *y,
                           int yC, int yOff, cudaStream_t s);
cudaError_t launchUpsampleGrad(const __nv_bfloat16 *dy, int dyC, int dyOff, int C, int N, int H,
                               int W, const __nv_bfloat16 *mask, __nv_bfloat16 *dx, cudaStream_t s);
cudaError_t launchCopyChannels(const __nv_bfloat16 *x, int xC, int xOff, __nv_bfloat16 *y, int yC,
                               int yOff, int C, size_t P, int add, cudaStream_t s);
cudaError_t launchReluMask(__nv_bfloat16 *d, int dC, int dOff, const __nv_bfloat16 *post, int pC,
                           int pOff, int C, size_t P, cudaStream_t s);
cudaError_t launchL1(const float *out, int oC, const float *target, int tC, int C, size_t P,
                     __nv_bfloat16 *grad, int gC, float *loss, cudaStream_t s);
cudaError_t launchAdam(float *w, float *m, float *v, const float *g, size_t n, float lr, float b1,
                       float b2, float eps, int step, __nv_bfloat16 *wb, __nv_bfloat16 *wt, int Cin,
                       int CoutT, cudaStream_t s);
// NHWC bf16 (C channels per pixel, a multiple of 8) -> channel-blocked planes
cudaError_t launchToBlocked(const __nv_bfloat16 *x, int C, size_t P, __nv_bfloat16 *y,
                            cudaStream_t s);
// Weights of one layer packed for kConv3x3Ws: per block of N output channels
// (N = 32 if Cout <= 32, else 64) and stage of 32 input channels, the nine
// taps' [tap][chunk 0..3][N][8] image of shared memory, zero-padded; from
// w [Cout][9][Cin]. packedConvWeights gives the element count.
size_t packedConvWeights(int Cin, int Cout);
cudaError_t launchPackConvWeights(const __nv_bfloat16 *w, int Cin, int Cout, __nv_bfloat16 *packed,
                                  cudaStream_t s);
cudaError_t launchDenoiseInput(const float4 *color, const float *albedo, const float *normal,
                               const float *depth, const float *var, float invSqrtN, int W, int H,
                               int Wp, int Hp, __nv_bfloat16 *x, int xC, cudaStream_t s);
cudaError_t launchDenoiseOutput(const float *out, int oC, int W, int H, int Wp, const float4 *mean,
                                const float *var, float k, float floorAbs, float4 *result,
                                uint8_t *retry, unsigned *numRetry, cudaStream_t s);

// Accumulation reset: accum = 0, depth = 1e31 (frame/Frame.cpp:287-312).
cudaError_t launchFrameReset(float4 *accum, float *depth, size_t numPixels, cudaStream_t stream);
// p[0 .. n) = value
cudaError_t launchFillU32(uint32_t *p, uint32_t value, size_t n, cudaStream_t stream);

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
// Spheres, cones, cylinders and curves in BVH leaf order: for leaf i with
// group index k (the w of the leaf's first float4), the kApStride records
// primsOut[kApStride i ..] = src[kApStride k ..] and localOut[i] =
// k | kinds[k] << kApKindShift.
cudaError_t launchGatherAnalytic(const float4 *leafTris, const float4 *src, const uint32_t *kinds,
                                 int n, float4 *primsOut, uint32_t *localOut,
                                 cudaStream_t stream);

cudaError_t collapseBVH4(const float4 *nodes2, int numNodes2, float4 *nodes4Out, int *numNodes4,
                         cudaStream_t stream);

// Turns small subtrees of a one-triangle-per-leaf BVH2 (traversal layout,
// root 0, numInner = n - 1 inner nodes) into leaves of up to maxLeaf
// triangles where the surface-area heuristic expects fewer node visits,
// reorders tris (n triangles, 3 float4 each) depth first and rewrites the
// nodes in place, the remaining ones in depth-first order (k_bvh_leaves.cu;
// *numNodesOut: the nodes kept; synchronizes the stream). maxLeaf <= 1
// leaves the BVH as it is.
cudaError_t collapseLeaves(float4 *nodes, int numInner, float4 *tris, int n, int maxLeaf,
                           int *numNodesOut, cudaStream_t stream);

// Same inputs/outputs, PLOC clustering instead of the Karras hierarchy:
// tighter boxes (close to a greedy SAH build), a few ms more per 1M
// triangles. Used for world commits unless the world asks for "fast".
cudaError_t buildGroupBVHQuality(const float *v1, const float *e1, const float *e2, int n,
                                 float4 *nodesOut, float4 *trisOut, BvhBuildStats *stats,
                                 cudaStream_t stream);

} // namespace vsr
