// Batched rendering: the frames of many scenes, cameras and image sizes in
// one persistent launch per renderer kind. Every frame is cut into tiles of
// 32 pixels (one warp); all tiles of all frames of a kind form one shared
// work list, ordered by estimated cost (longest first), and warps take items
// from it with an atomic counter. A warp keeps its current frame's scene,
// camera, renderer and frame records in shared memory. Pixels are rendered
// by the same per-pixel bodies as the per-frame kernels (render_pixel.cuh),
// with the same per-pixel random streams, so a batched frame is bit-identical
// to the same frame rendered alone.
#include "render_pixel.cuh"
#include "kernels.h"

namespace vsr {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// Per-frame preparation for the batch: the accumulation reset of frames
// whose accumulation restarts (frame/Frame.cpp:287-312), and the error flags.
__global__ void kBatchPrepare(const DJob *jobs, int numJobs) {
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int j = 0; j < numJobs; ++j) {
    const DJob &J = jobs[j];
    if (tid == 0) *J.F.errorFlags = 0u;
    if (!J.reset) continue;
    const size_t n = (size_t)J.F.width * J.F.height;
    for (size_t i = tid; i < n; i += stride) {
      J.F.accum[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (J.F.depth) J.F.depth[i] = 1e31f;
    }
  }
}

template <int Kind, bool Full>
__device__ __forceinline__ void renderItem(const DJob &J, int x, int y) {
  if (Kind == JOB_PATHTRACE) pathtracePixel<false, Full>(J.S, J.C, J.R, J.F, x, y);
  else if (Kind == JOB_RAYCAST_SURFACES) raycastPixel<false, true>(J.S, J.C, J.R, J.F, x, y, nullptr);
  else if (Kind == JOB_RAYCAST_FULL)
    raycastPixel<false, true, true>(J.S, J.C, J.R, J.F, x, y, nullptr);
  else raycastPixel<false, false>(J.S, J.C, J.R, J.F, x, y, nullptr);
}

// Items are (job, tile) pairs; a tile is tileW x (32 / tileW) pixels. A warp
// takes `fetch` consecutive items per atomic.
template <int Kind, bool Full = false>
__device__ __forceinline__ void batchLoop(const DJob *jobs, const uint2 *items, unsigned numItems,
                                          unsigned *next, int tileW, int fetch, DJob *sJob) {
  const int lane = threadIdx.x & 31;
  const int tileH = 32 / tileW;
  const int px = lane % tileW, py = lane / tileW;
  int cur = -1;
  for (;;) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(next, (unsigned)fetch);
    base = __shfl_sync(kFull, base, 0);
    if (base >= numItems) break;
    const unsigned end = min(base + (unsigned)fetch, numItems);
    for (unsigned k = base; k < end; ++k) {
      const uint2 it = items[k];
      if ((int)it.x != cur) {  // warp-uniform: stage the job's records
        __syncwarp();
        const int *src = reinterpret_cast<const int *>(jobs + it.x);
        int *dst = reinterpret_cast<int *>(sJob);
        for (int w = lane; w < (int)(sizeof(DJob) / 4); w += 32) dst[w] = src[w];
        __syncwarp();
        cur = (int)it.x;
      }
      const int tx = (int)it.y % sJob->tilesX, ty = (int)it.y / sJob->tilesX;
      const int x = tx * tileW + px, y = ty * tileH + py;
      if (x < sJob->F.width && y < sJob->F.height) renderItem<Kind, Full>(*sJob, x, y);
    }
  }
}

// the register budgets of kPathtrace: 64 registers when worlds have volumes;
// Full: a job uses gradient shading or point / spot lights
template <bool Volumes, bool Full>
__global__ void __launch_bounds__(128, Volumes ? VSR_MEGA_MIN_BLOCKS_VOLUMES : VSR_MEGA_MIN_BLOCKS)
    kBatchPathtrace(const DJob *jobs, const uint2 *items, unsigned numItems, unsigned *next,
                    int tileW, int fetch) {
  __shared__ __align__(16) DJob sJob[4];
  batchLoop<JOB_PATHTRACE, Full>(jobs, items, numItems, next, tileW, fetch,
                                 &sJob[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(128)
    kBatchRaycastSurfaces(const DJob *jobs, const uint2 *items, unsigned numItems, unsigned *next,
                          int tileW, int fetch) {
  __shared__ __align__(16) DJob sJob[4];
  batchLoop<JOB_RAYCAST_SURFACES>(jobs, items, numItems, next, tileW, fetch,
                                  &sJob[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(128)
    kBatchRaycastVolume(const DJob *jobs, const uint2 *items, unsigned numItems, unsigned *next,
                        int tileW, int fetch) {
  __shared__ __align__(16) DJob sJob[4];
  batchLoop<JOB_RAYCAST_VOLUME>(jobs, items, numItems, next, tileW, fetch,
                                &sJob[threadIdx.x >> 5]);
}

// raycast frames with gradient shading or point / spot lights, any world
__global__ void __launch_bounds__(128)
    kBatchRaycastFull(const DJob *jobs, const uint2 *items, unsigned numItems, unsigned *next,
                      int tileW, int fetch) {
  __shared__ __align__(16) DJob sJob[4];
  batchLoop<JOB_RAYCAST_FULL>(jobs, items, numItems, next, tileW, fetch,
                              &sJob[threadIdx.x >> 5]);
}

int smCount() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  return sms;
}

template <typename K>
cudaError_t launchPersistent(K kernel, const BatchLaunch &L, int kind, cudaStream_t stream) {
  const unsigned n = L.numItems[kind];
  if (!n) return cudaSuccess;
  int perSM = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, 128, 0);
  const unsigned warps = (unsigned)(smCount() * (perSM > 0 ? perSM : 1) * 4);
  // no more warps than item fetches
  const unsigned fetches = (n + (unsigned)L.fetch - 1) / (unsigned)L.fetch;
  const unsigned blocks = (min(warps, fetches) + 3) / 4;
  kernel<<<blocks, 128, 0, stream>>>(L.jobs, L.items[kind], n, L.counters + kind, L.tileW,
                                     L.fetch);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launchBatch(const BatchLaunch &L, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(L.counters, 0, kJobKinds * sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  kBatchPrepare<<<smCount() * 4, 256, 0, stream>>>(L.jobs, L.numJobs);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  switch (L.pathtraceVariant) {
    case 3: e = launchPersistent(kBatchPathtrace<true, true>, L, JOB_PATHTRACE, stream); break;
    case 2: e = launchPersistent(kBatchPathtrace<false, true>, L, JOB_PATHTRACE, stream); break;
    case 1: e = launchPersistent(kBatchPathtrace<true, false>, L, JOB_PATHTRACE, stream); break;
    default: e = launchPersistent(kBatchPathtrace<false, false>, L, JOB_PATHTRACE, stream);
  }
  if (e != cudaSuccess) return e;
  if ((e = launchPersistent(kBatchRaycastSurfaces, L, JOB_RAYCAST_SURFACES, stream)) != cudaSuccess)
    return e;
  if ((e = launchPersistent(kBatchRaycastVolume, L, JOB_RAYCAST_VOLUME, stream)) != cudaSuccess)
    return e;
  return launchPersistent(kBatchRaycastFull, L, JOB_RAYCAST_FULL, stream);
}

}  // namespace vsr
