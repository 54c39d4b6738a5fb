// vsrBuildTriangleBVHNoAlloc: the device BVH build without any GPU memory
// allocation.
//
// The regular build (vsrBuildTriangleBVH) takes its temporary buffers from
// the stream-ordered allocator. Some callers cannot let a library allocate
// GPU memory: a host application that owns a fixed GPU memory budget and
// hands plugins only the buffers it allocated itself, or a latency-critical
// per-frame loop that must not risk an allocation (or a free, which can
// synchronize the whole device) in the middle of a frame. For them this
// entry point runs the same kernels with all temporaries carved out of one
// statically sized buffer in the library's device data.
//
// The buffer (kScratchBytes) exists once per GPU that loads the library and
// stays until the process exits. Every call on a device shares it and leaves
// its contents behind; the parts that must start at zero (bounds, refit
// counters) are cleared by each call. Calls that overlap on the GPU race on
// the buffer, so callers must order them (one stream, or events).
#include "bvh_kernels.cuh"
#include "vsr.h"

#include <cub/device/device_radix_sort.cuh>

#include <mutex>

namespace vsr {
namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;  // 8 MiB per device
static_assert(VSR_BVH_NOALLOC_MAX_TRIANGLES == 65536u, "limit documented in vsr.h");

static __device__ __align__(256) unsigned char g_bvhScratch[kScratchBytes];

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct ScratchLayout {
  size_t bounds, keys, keys2, vals, vals2, childL, childR, parentInner, parentLeaf, flags,
      innerBox, cubTemp, cubBytes, total;
};

cudaError_t layoutFor(uint32_t n, cudaStream_t stream, ScratchLayout &L) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t at = off;
    off = align256(off + bytes);
    return at;
  };
  L.bounds = take(6 * sizeof(uint32_t));
  L.keys = take(n * sizeof(uint64_t));
  L.keys2 = take(n * sizeof(uint64_t));
  L.vals = take(n * sizeof(uint32_t));
  L.vals2 = take(n * sizeof(uint32_t));
  L.childL = take((n - 1) * sizeof(int));
  L.childR = take((n - 1) * sizeof(int));
  L.parentInner = take((n - 1) * sizeof(int));
  L.parentLeaf = take(n * sizeof(int));
  L.flags = take((n - 1) * sizeof(int));
  L.innerBox = take((n - 1) * sizeof(Aabb));
  L.cubBytes = 0;
  // size query only: no memory is touched or allocated
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, L.cubBytes, (uint64_t *)nullptr,
                                                  (uint64_t *)nullptr, (uint32_t *)nullptr,
                                                  (uint32_t *)nullptr, (int)n, 0, 63, stream);
  L.cubTemp = take(L.cubBytes);
  L.total = off;
  return e;
}

// Reset what the build expects to start at zero / empty.
__global__ void kClearScratch(uint32_t *bounds, int *flags, int numFlags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 6) bounds[i] = i < 3 ? 0xffffffffu : 0u;
  for (int k = i; k < numFlags; k += gridDim.x * blockDim.x) flags[k] = 0;
}

std::mutex g_setupMutex;
void *g_scratch[256] = {};

// The device address of the static buffer on the current device. The
// address belongs to the device's current context: a cudaDeviceReset (or a
// released and re-created primary context) reloads the module and may move
// it. So every call made outside stream capture looks it up again (a
// lookup, no allocation) and refreshes the per-device copy; while `stream`
// is being captured the copy from the device's last uncaptured call is
// used (the first lookup may load the module, so the first call on a
// device must come before any capture; without a copy the call fails).
cudaError_t scratchOfCurrentDevice(cudaStream_t stream, void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_setupMutex);
  if (cap == cudaStreamCaptureStatusNone) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress((void **)&ptr, g_bvhScratch);
    if (e != cudaSuccess) return e;
    g_scratch[dev] = ptr;
  } else if (!g_scratch[dev]) {
    return cudaErrorStreamCaptureUnsupported;
  }
  *out = g_scratch[dev];
  return cudaSuccess;
}

} // namespace
} // namespace vsr

using namespace vsr;

extern "C" VSRStatus vsrBuildTriangleBVHNoAlloc(const float *v1, const float *e1, const float *e2,
                                                uint32_t n, void *nodesOut, void *trisOut,
                                                void *streamPtr) {
  if (n == 0) return VSR_OK;
  if (!v1 || !e1 || !e2 || !nodesOut || !trisOut) return VSR_ERROR_INVALID_ARGUMENT;
  if (n > VSR_BVH_NOALLOC_MAX_TRIANGLES) return VSR_ERROR_LIMIT_EXCEEDED;
  cudaStream_t stream = (cudaStream_t)streamPtr;
  float4 *nodes = (float4 *)nodesOut;
  float4 *tris = (float4 *)trisOut;
  if (n == 1) {
    kSingle<<<1, 1, 0, stream>>>(v1, e1, e2, nodes, tris);
    return cudaGetLastError() == cudaSuccess ? VSR_OK : VSR_ERROR_CUDA;
  }
  void *base = nullptr;
  if (scratchOfCurrentDevice(stream, &base) != cudaSuccess) return VSR_ERROR_CUDA;
  ScratchLayout L;
  if (layoutFor(n, stream, L) != cudaSuccess) return VSR_ERROR_CUDA;
  if (L.total > kScratchBytes) return VSR_ERROR_LIMIT_EXCEEDED;
  unsigned char *s = (unsigned char *)base;
  uint32_t *bounds = (uint32_t *)(s + L.bounds);
  uint64_t *keys = (uint64_t *)(s + L.keys), *keys2 = (uint64_t *)(s + L.keys2);
  uint32_t *vals = (uint32_t *)(s + L.vals), *vals2 = (uint32_t *)(s + L.vals2);
  int *childL = (int *)(s + L.childL), *childR = (int *)(s + L.childR);
  int *parentInner = (int *)(s + L.parentInner), *parentLeaf = (int *)(s + L.parentLeaf);
  int *flags = (int *)(s + L.flags);
  Aabb *innerBox = (Aabb *)(s + L.innerBox);
  void *tmp = s + L.cubTemp;
  size_t tmpBytes = L.cubBytes;

  const int B = 256;
  const int grid = (int)((n + B - 1) / B);
  kClearScratch<<<min(grid, 1024), B, 0, stream>>>(bounds, flags, (int)n - 1);
  kCentroidBounds<<<min(grid, 1024), B, 0, stream>>>(v1, e1, e2, (int)n, bounds);
  kMorton<<<grid, B, 0, stream>>>(v1, e1, e2, (int)n, bounds, keys, vals);
  if (cudaGetLastError() != cudaSuccess) return VSR_ERROR_CUDA;
  if (cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, keys, keys2, vals, vals2, (int)n, 0, 63,
                                      stream) != cudaSuccess)
    return VSR_ERROR_CUDA;
  kHierarchy<<<(int)((n - 1 + B - 1) / B), B, 0, stream>>>(keys2, (int)n, childL, childR,
                                                          parentInner, parentLeaf);
  kRefit<<<grid, B, 0, stream>>>(v1, e1, e2, vals2, (int)n, childL, childR, parentInner,
                                 parentLeaf, flags, innerBox, nodes);
  kReorder<<<grid, B, 0, stream>>>(v1, e1, e2, vals2, (int)n, tris);
  return cudaGetLastError() == cudaSuccess ? VSR_OK : VSR_ERROR_CUDA;
}
