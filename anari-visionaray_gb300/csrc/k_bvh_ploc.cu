// Higher-quality device BVH build for world commits: PLOC (parallel locally
// ordered clustering, Meister & Bittner, TVCG 2018) over the Morton-sorted
// triangles. Every round, each cluster looks for the neighbour within
// +-kRadius positions whose union box has the smallest surface area; mutual
// nearest neighbours merge into a new inner node; survivors are compacted in
// order. This approximates a greedy SAH agglomerative build and gives far
// tighter boxes than the spatial-median splits of the LBVH, which matters
// for the divergent secondary rays of the path tracer.
//
// The node layout written is the traversal layout of vsr_device.h: inner
// node ids are assigned in creation order and stored reversed, so the root
// (created last) is node 0. Node ids come from prefix sums, so the output is
// deterministic.
#include "bvh_kernels.cuh"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

namespace vsr {
namespace {

// neighbours searched on either side of a cluster (measured on the 1M-
// triangle sphere scene, ms per 64-spp frame at radius 8 / 16 / 32 / 64 /
// 96 / 128 / 192: 207.8 / 198.7 / 191.5 / 184.3 / 180.5 / 178.6 / 178.6,
// build 7.2 ms at 16 and 8.7 ms at 128)
constexpr int kRadius = 128;
constexpr int kBlock = 256;

__device__ __forceinline__ float halfArea(const Aabb &b) {
  const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ Aabb unite(const Aabb &a, const Aabb &b) {
  Aabb u;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    u.lo[k] = fminf(a.lo[k], b.lo[k]);
    u.hi[k] = fmaxf(a.hi[k], b.hi[k]);
  }
  return u;
}

__global__ void kInitClusters(const float *v1, const float *e1, const float *e2,
                              const uint32_t *order, int n, int *cluster, Aabb *box) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cluster[i] = ~i;  // leaf: position in the sorted (leaf) order
  box[i] = triBox(v1, e1, e2, (int)order[i]);
}

__global__ void kNearest(const Aabb *box, int count, int *nn) {
  __shared__ Aabb sbox[kBlock + 2 * kRadius];
  const int start = blockIdx.x * blockDim.x;
  for (int k = threadIdx.x; k < kBlock + 2 * kRadius; k += blockDim.x) {
    const int g = start - kRadius + k;
    if (g >= 0 && g < count) sbox[k] = box[g];
  }
  __syncthreads();
  const int i = start + threadIdx.x;
  if (i >= count) return;
  const Aabb me = sbox[threadIdx.x + kRadius];
  float best = FLT_MAX;
  int bj = -1;
  for (int o = -kRadius; o <= kRadius; ++o) {
    const int j = i + o;
    if (o == 0 || j < 0 || j >= count) continue;
    const float a = halfArea(unite(me, sbox[threadIdx.x + kRadius + o]));
    if (a < best) {  // o ascends, so ties keep the smaller index
      best = a;
      bj = j;
    }
  }
  nn[i] = bj;
}

// leader[i] = 1 if i merges with its mutual neighbour j > i;
// keep[i] = 0 if i is absorbed by a mutual neighbour j < i.
__global__ void kMergeFlags(const int *nn, int count, int *leader, int *keep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int j = nn[i];
  const bool mutual = j >= 0 && nn[j] == i;
  leader[i] = (mutual && i < j) ? 1 : 0;
  keep[i] = (mutual && j < i) ? 0 : 1;
}

__global__ void kMergeApply(const int *nn, const int *leader, const int *leaderScan, int count,
                            int nodeBase, int numInner, int *cluster, Aabb *box,
                            float4 *nodes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count || !leader[i]) return;
  const int j = nn[i];
  const int id = nodeBase + leaderScan[i];   // creation order
  const int slot = numInner - 1 - id;        // root (created last) -> 0
  const Aabb a = box[i], b = box[j];
  float4 *N = nodes + 4 * (size_t)slot;
  N[0] = make_float4(a.lo[0], a.hi[0], a.lo[1], a.hi[1]);
  N[1] = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
  N[2] = make_float4(a.lo[2], a.hi[2], b.lo[2], b.hi[2]);
  N[3] = make_float4(__int_as_float(cluster[i]), __int_as_float(cluster[j]), 0.f, 0.f);
  cluster[i] = slot;
  box[i] = unite(a, b);
}

__global__ void kCompact(const int *keep, const int *keepScan, int count, const int *cluster,
                         const Aabb *box, int *cluster2, Aabb *box2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count || !keep[i]) return;
  const int k = keepScan[i];
  cluster2[k] = cluster[i];
  box2[k] = box[i];
}

} // namespace

#define VSR_TRY(x)        \
  do {                    \
    cudaError_t e_ = (x); \
    if (e_ != cudaSuccess) { \
      err = e_;           \
      goto cleanup;       \
    }                     \
  } while (0)

cudaError_t buildGroupBVHQuality(const float *v1, const float *e1, const float *e2, int n,
                                 float4 *nodesOut, float4 *trisOut, BvhBuildStats *stats,
                                 cudaStream_t stream) {
  if (n <= 1) return buildGroupBVH(v1, e1, e2, n, nodesOut, trisOut, stats, stream);
  cudaError_t err = cudaSuccess;
  uint32_t *bounds = nullptr, *vals = nullptr, *vals2 = nullptr, *host = nullptr;
  uint64_t *keys = nullptr, *keys2 = nullptr;
  int *cluster = nullptr, *cluster2 = nullptr, *nn = nullptr, *leader = nullptr, *keep = nullptr,
      *leaderScan = nullptr, *keepScan = nullptr;
  Aabb *box = nullptr, *box2 = nullptr;
  void *tmp = nullptr;
  size_t tmpBytes = 0, sortBytes = 0, scanBytes = 0;
  cudaEvent_t e0 = nullptr, e1ev = nullptr;
  int count = n, nodeBase = 0, rounds = 0;
  const int numInner = n - 1;
  const int grid = (n + kBlock - 1) / kBlock;
  const uint32_t initBounds[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  VSR_TRY(cudaEventCreate(&e0));
  VSR_TRY(cudaEventCreate(&e1ev));
  VSR_TRY(cudaEventRecord(e0, stream));
  VSR_TRY(cudaMallocHost((void **)&host, 4 * sizeof(uint32_t)));
  VSR_TRY(cudaMallocAsync((void **)&bounds, 6 * sizeof(uint32_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&keys, n * sizeof(uint64_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&keys2, n * sizeof(uint64_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&vals, n * sizeof(uint32_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&vals2, n * sizeof(uint32_t), stream));
  VSR_TRY(cudaMallocAsync((void **)&cluster, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&cluster2, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&nn, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&leader, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&keep, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&leaderScan, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&keepScan, n * sizeof(int), stream));
  VSR_TRY(cudaMallocAsync((void **)&box, n * sizeof(Aabb), stream));
  VSR_TRY(cudaMallocAsync((void **)&box2, n * sizeof(Aabb), stream));
  VSR_TRY(cudaMemcpyAsync(bounds, initBounds, sizeof(initBounds), cudaMemcpyHostToDevice, stream));
  kCentroidBounds<<<min(grid, 1024), kBlock, 0, stream>>>(v1, e1, e2, n, bounds);
  kMorton<<<grid, kBlock, 0, stream>>>(v1, e1, e2, n, bounds, keys, vals);
  VSR_TRY(cudaGetLastError());
  VSR_TRY(cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, keys, keys2, vals, vals2, n, 0, 63,
                                          stream));
  VSR_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, leader, leaderScan, n, stream));
  tmpBytes = sortBytes > scanBytes ? sortBytes : scanBytes;
  VSR_TRY(cudaMallocAsync(&tmp, tmpBytes, stream));
  VSR_TRY(cub::DeviceRadixSort::SortPairs(tmp, sortBytes, keys, keys2, vals, vals2, n, 0, 63,
                                          stream));
  kInitClusters<<<grid, kBlock, 0, stream>>>(v1, e1, e2, vals2, n, cluster, box);
  VSR_TRY(cudaGetLastError());
  while (count > 1) {
    const int g = (count + kBlock - 1) / kBlock;
    kNearest<<<g, kBlock, 0, stream>>>(box, count, nn);
    kMergeFlags<<<g, kBlock, 0, stream>>>(nn, count, leader, keep);
    VSR_TRY(cudaGetLastError());
    size_t sb = scanBytes;
    VSR_TRY(cub::DeviceScan::ExclusiveSum(tmp, sb, leader, leaderScan, count, stream));
    sb = scanBytes;
    VSR_TRY(cub::DeviceScan::ExclusiveSum(tmp, sb, keep, keepScan, count, stream));
    kMergeApply<<<g, kBlock, 0, stream>>>(nn, leader, leaderScan, count, nodeBase, numInner,
                                          cluster, box, nodesOut);
    kCompact<<<g, kBlock, 0, stream>>>(keep, keepScan, count, cluster, box, cluster2, box2);
    VSR_TRY(cudaGetLastError());
    // merges this round = leaderScan[last] + leader[last]
    VSR_TRY(cudaMemcpyAsync(host, leaderScan + count - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
    VSR_TRY(cudaMemcpyAsync(host + 1, leader + count - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
    VSR_TRY(cudaStreamSynchronize(stream));
    const int merges = (int)host[0] + (int)host[1];
    if (merges == 0 || ++rounds > 4096) {
      err = cudaErrorUnknown;  // no mutual pair: cannot happen for finite boxes
      goto cleanup;
    }
    nodeBase += merges;
    count -= merges;
    int *ct = cluster; cluster = cluster2; cluster2 = ct;
    Aabb *bt = box; box = box2; box2 = bt;
  }
  kReorder<<<grid, kBlock, 0, stream>>>(v1, e1, e2, vals2, n, trisOut);
  VSR_TRY(cudaGetLastError());
  VSR_TRY(cudaEventRecord(e1ev, stream));
  if (stats) {
    stats->numNodes = numInner;
    VSR_TRY(cudaEventSynchronize(e1ev));
    VSR_TRY(cudaEventElapsedTime(&stats->buildMs, e0, e1ev));
  }
cleanup:
  for (void *p : {(void *)bounds, (void *)keys, (void *)keys2, (void *)vals, (void *)vals2,
                  (void *)cluster, (void *)cluster2, (void *)nn, (void *)leader, (void *)keep,
                  (void *)leaderScan, (void *)keepScan, (void *)box, (void *)box2, tmp})
    if (p) cudaFreeAsync(p, stream);
  if (host) {
    cudaStreamSynchronize(stream);
    cudaFreeHost(host);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1ev) cudaEventDestroy(e1ev);
  return err;
}

} // namespace vsr
