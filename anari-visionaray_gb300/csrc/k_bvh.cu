// On-device BVH build per commit: Morton codes (21 bits per axis) over the
// triangle centroids, a radix sort, the parallel hierarchy construction of
// Karras (HPG 2012), and a bottom-up refit that writes the traversal layout
// (child boxes stored in the parent, vsr_device.h) directly.
//
// Replaces DeviceBVH's host binned-SAH/spatial-split build plus upload for
// triangle BLSs (DeviceBVH.h:174-237, :350-377) and the device LBVH used
// for TLSs (DeviceBVH.h:300-309). The BVH shape affects speed only: the
// traversal resolves closest hits by (t, instance, triangle).
#include "bvh_kernels.cuh"

#include <cub/device/device_radix_sort.cuh>

namespace vsr {


#define VSR_TRY(x)                     \
  do {                                 \
    cudaError_t e_ = (x);              \
    if (e_ != cudaSuccess) {           \
      err = e_;                        \
      goto cleanup;                    \
    }                                  \
  } while (0)

cudaError_t buildGroupBVH(const float *v1, const float *e1, const float *e2, int n,
                          float4 *nodesOut, float4 *trisOut, BvhBuildStats *stats,
                          cudaStream_t stream) {
  if (n <= 0) {
    if (stats) { stats->numNodes = 0; stats->buildMs = 0.f; }
    return cudaSuccess;
  }
  if (n == 1) {
    kSingle<<<1, 1, 0, stream>>>(v1, e1, e2, nodesOut, trisOut);
    if (stats) { stats->numNodes = 1; stats->buildMs = 0.f; }
    return cudaGetLastError();
  }
  cudaError_t err = cudaSuccess;
  uint32_t *bounds = nullptr;
  uint64_t *keys = nullptr, *keys2 = nullptr;
  uint32_t *vals = nullptr, *vals2 = nullptr;
  int *childL = nullptr, *childR = nullptr, *parentInner = nullptr, *parentLeaf = nullptr;
  int *flags = nullptr;
  Aabb *innerBox = nullptr;
  void *tmp = nullptr;
  size_t tmpBytes = 0;
  cudaEvent_t e0 = nullptr, e1ev = nullptr;
  const int B = 256;
  const int grid = (n + B - 1) / B;
  const uint32_t initBounds[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  VSR_TRY(cudaEventCreate(&e0));
  VSR_TRY(cudaEventCreate(&e1ev));
  VSR_TRY(cudaEventRecord(e0, stream));
  VSR_TRY(cudaMallocAsync((void **)&bounds, 6 * sizeof(uint32_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&keys, n * sizeof(uint64_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&keys2, n * sizeof(uint64_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&vals, n * sizeof(uint32_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&vals2, n * sizeof(uint32_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&childL, (n - 1) * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&childR, (n - 1) * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&parentInner, (n - 1) * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&parentLeaf, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&flags, (n - 1) * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&innerBox, (n - 1) * sizeof(Aabb), stream));
  VSR_TRY(cudaMemcpyAsync(bounds, initBounds, sizeof(initBounds), cudaMemcpyHostToDevice, stream));
  VSR_TRY(cudaMemsetAsync(flags, 0, (n - 1) * sizeof(int), stream));
  kCentroidBounds<<<min(grid, 1024), B, 0, stream>>>(v1, e1, e2, n, bounds);
  VSR_TRY(cudaGetLastError());
  kMorton<<<grid, B, 0, stream>>>(v1, e1, e2, n, bounds, keys, vals);
  VSR_TRY(cudaGetLastError());
  VSR_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, keys, keys2, vals, vals2, n, 0, 63,
                                          stream));
  VSR_TRY(cudaMallocAsync(&tmp, tmpBytes, stream));
  VSR_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, keys, keys2, vals, vals2, n, 0, 63,
                                          stream));
  kHierarchy<<<(n - 1 + B - 1) / B, B, 0, stream>>>(keys2, n, childL, childR, parentInner,
                                                    parentLeaf);
  VSR_TRY(cudaGetLastError());
  kRefit<<<grid, B, 0, stream>>>(v1, e1, e2, vals2, n, childL, childR, parentInner, parentLeaf,
                                 flags, innerBox, nodesOut);
  VSR_TRY(cudaGetLastError());
  kReorder<<<grid, B, 0, stream>>>(v1, e1, e2, vals2, n, trisOut);
  VSR_TRY(cudaGetLastError());
  VSR_TRY(cudaEventRecord(e1ev, stream));
  if (stats) {
    stats->numNodes = n - 1;
    VSR_TRY(cudaEventSynchronize(e1ev));
    VSR_TRY(cudaEventElapsedTime(&stats->buildMs, e0, e1ev));
  }
cleanup:
  if (bounds) cudaFreeAsync(bounds, stream);
  if (keys) cudaFreeAsync(keys, stream);
  if (keys2) cudaFreeAsync(keys2, stream);
  if (vals) cudaFreeAsync(vals, stream);
  if (vals2) cudaFreeAsync(vals2, stream);
  if (childL) cudaFreeAsync(childL, stream);
  if (childR) cudaFreeAsync(childR, stream);
  if (parentInner) cudaFreeAsync(parentInner, stream);
  if (parentLeaf) cudaFreeAsync(parentLeaf, stream);
  if (flags) cudaFreeAsync(flags, stream);
  if (innerBox) cudaFreeAsync(innerBox, stream);
  if (tmp) cudaFreeAsync(tmp, stream);
  if (e0) cudaEventDestroy(e0);
  if (e1ev) cudaEventDestroy(e1ev);
  return err;
}

// Analytic-primitive leaves: the builder ran over each primitive's
// bounding triangle and wrote the leaf-ordered triangles with the group
// index in the first float4's w; the primitive records follow that order.
__global__ void kGatherAnalytic(const float4 *leafTris, const float4 *src, const uint32_t *kinds,
                                int n, float4 *primsOut, uint32_t *localOut) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = __float_as_int(leafTris[3 * (size_t)i].w);
  if (k < 0 || k >= n) {  // not a valid group index: a sphere that is never hit
    primsOut[kApStride * (size_t)i] = make_float4(__int_as_float(0x7fffffff), 0.f, 0.f, 0.f);
    for (int c = 1; c < kApStride; ++c)
      primsOut[kApStride * (size_t)i + c] = make_float4(0.f, 0.f, 0.f, 0.f);
    localOut[i] = 0;
    return;
  }
  for (int c = 0; c < kApStride; ++c)
    primsOut[kApStride * (size_t)i + c] = src[kApStride * (size_t)k + c];
  localOut[i] = (uint32_t)k | (kinds[k] << kApKindShift);
}

cudaError_t launchGatherAnalytic(const float4 *leafTris, const float4 *src, const uint32_t *kinds,
                                 int n, float4 *primsOut, uint32_t *localOut,
                                 cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  kGatherAnalytic<<<(n + 255) / 256, 256, 0, stream>>>(leafTris, src, kinds, n, primsOut,
                                                       localOut);
  return cudaGetLastError();
}

} // namespace vsr
