// BVH2 -> BVH4 collapse on the device, level by level. A BVH4 node starts
// from the two children of a BVH2 node and repeatedly opens the inner child
// with the largest box surface area until it has four children; every inner
// child left becomes a BVH4 node of the next level. Four-wide nodes halve
// the depth of the traversal loop and let one 128-byte fetch test four
// boxes, which shortens the chain of dependent node loads per ray.
#include "kernels.h"

#include <float.h>

namespace vsr {
namespace {

struct Cand {
  float lo[3], hi[3];
  int code;
};

__device__ __forceinline__ float halfArea(const Cand &c) {
  const float dx = c.hi[0] - c.lo[0], dy = c.hi[1] - c.lo[1], dz = c.hi[2] - c.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void childrenOf(const float4 *nodes2, int n, Cand &a, Cand &b) {
  const float4 n0 = nodes2[4 * (size_t)n], n1 = nodes2[4 * (size_t)n + 1],
               n2 = nodes2[4 * (size_t)n + 2];
  const int4 n3 = reinterpret_cast<const int4 *>(nodes2)[4 * (size_t)n + 3];
  a.lo[0] = n0.x; a.hi[0] = n0.y; a.lo[1] = n0.z; a.hi[1] = n0.w; a.lo[2] = n2.x; a.hi[2] = n2.y;
  b.lo[0] = n1.x; b.hi[0] = n1.y; b.lo[1] = n1.z; b.hi[1] = n1.w; b.lo[2] = n2.z; b.hi[2] = n2.w;
  a.code = n3.x;
  b.code = n3.y;
}

// queue items: (BVH2 node, BVH4 slot)
__global__ void kCollapse(const float4 *nodes2, const int2 *qin, const int *countIn, int2 *qout,
                          int *countOut, int *nodeCounter, float4 *nodes4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *countIn) return;
  const int2 item = qin[i];
  Cand c[4];
  int k = 2;
  childrenOf(nodes2, item.x, c[0], c[1]);
  while (k < 4) {
    int best = -1;
    float ba = -1.f;
    for (int j = 0; j < k; ++j)
      if (c[j].code >= 0) {
        const float a = halfArea(c[j]);
        if (a > ba) { ba = a; best = j; }
      }
    if (best < 0) break;
    Cand a, b;
    childrenOf(nodes2, c[best].code, a, b);
    c[best] = a;
    c[k++] = b;
  }
  int inner = 0;
  for (int j = 0; j < k; ++j) inner += c[j].code >= 0;
  int base = inner ? atomicAdd(nodeCounter, inner) : 0;
  int qbase = inner ? atomicAdd(countOut, inner) : 0;
  float lo[3][4], hi[3][4];
  int codes[4];
  for (int j = 0; j < 4; ++j) {
    if (j < k) {
      for (int a = 0; a < 3; ++a) { lo[a][j] = c[j].lo[a]; hi[a][j] = c[j].hi[a]; }
      if (c[j].code >= 0) {
        codes[j] = base;
        qout[qbase++] = make_int2(c[j].code, base);
        ++base;
      } else {
        codes[j] = c[j].code;
      }
    } else {
      // empty slot: the traversal skips kEmptyChild by its code
      for (int a = 0; a < 3; ++a) { lo[a][j] = 0.f; hi[a][j] = 0.f; }
      codes[j] = kEmptyChild;
    }
  }
  float4 *N = nodes4 + 8 * (size_t)item.y;
  N[0] = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
  N[1] = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
  N[2] = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
  N[3] = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
  N[4] = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
  N[5] = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
  N[6] = make_float4(__int_as_float(codes[0]), __int_as_float(codes[1]),
                     __int_as_float(codes[2]), __int_as_float(codes[3]));
  N[7] = make_float4(0.f, 0.f, 0.f, 0.f);
}

} // namespace

cudaError_t collapseBVH4(const float4 *nodes2, int numNodes2, float4 *nodes4Out, int *numNodes4,
                         cudaStream_t stream) {
  cudaError_t err = cudaSuccess;
  int2 *q[2] = {nullptr, nullptr};
  int *counts = nullptr, *host = nullptr;
  int cur = 0, levels = 0;
  const int2 root = make_int2(0, 0);
  const int init[3] = {1, 0, 1};  // count q0, count q1, nodes allocated (root)
  if (numNodes2 <= 0) {
    *numNodes4 = 0;
    return cudaSuccess;
  }
  if ((err = cudaMallocAsync((void **)&q[0], numNodes2 * sizeof(int2), stream)) ||
      (err = cudaMallocAsync((void **)&q[1], numNodes2 * sizeof(int2), stream)) ||
      (err = cudaMallocAsync((void **)&counts, 3 * sizeof(int), stream)) ||
      (err = cudaMallocHost((void **)&host, 3 * sizeof(int))))
    goto cleanup;
  if ((err = cudaMemcpyAsync(q[0], &root, sizeof(int2), cudaMemcpyHostToDevice, stream)) ||
      (err = cudaMemcpyAsync(counts, init, sizeof(init), cudaMemcpyHostToDevice, stream)))
    goto cleanup;
  host[0] = 1;
  while (host[cur] > 0 && levels < 256) {
    const int n = host[cur];
    if ((err = cudaMemsetAsync(counts + (cur ^ 1), 0, sizeof(int), stream))) goto cleanup;
    kCollapse<<<(n + 127) / 128, 128, 0, stream>>>(nodes2, q[cur], counts + cur, q[cur ^ 1],
                                                    counts + (cur ^ 1), counts + 2, nodes4Out);
    if ((err = cudaGetLastError()) ||
        (err = cudaMemcpyAsync(host, counts, 3 * sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
        (err = cudaStreamSynchronize(stream)))
      goto cleanup;
    cur ^= 1;
    ++levels;
  }
  *numNodes4 = host[2];
cleanup:
  if (q[0]) cudaFreeAsync(q[0], stream);
  if (q[1]) cudaFreeAsync(q[1], stream);
  if (counts) cudaFreeAsync(counts, stream);
  if (host) {
    cudaStreamSynchronize(stream);
    cudaFreeHost(host);
  }
  return err;
}

} // namespace vsr
