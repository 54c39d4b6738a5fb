// LBVH build kernels shared by the BVH entry points: centroid bounds,
// 63-bit Morton codes, the Karras (HPG 2012) hierarchy, the bottom-up refit
// that writes the traversal node layout of vsr_device.h, and the leaf-order
// triangle copy. Internal linkage: each including translation unit gets its
// own instances.
#pragma once

#include "kernels.h"

#include <float.h>
#include <stdint.h>

namespace vsr {
namespace {

__device__ __forceinline__ uint32_t floatToOrdered(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float orderedToFloat(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

struct Aabb {
  float lo[3], hi[3];
};

__device__ __forceinline__ Aabb triBox(const float *v1, const float *e1, const float *e2, int i) {
  Aabb b;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float p0 = v1[3 * i + a];
    float p1 = p0 + e1[3 * i + a];
    float p2 = p0 + e2[3 * i + a];
    float lo = fminf(p0, fminf(p1, p2)), hi = fmaxf(p0, fmaxf(p1, p2));
    // pad by a relative 1e-6 so rounding in the slab test cannot cull a
    // triangle that touches its box
    float pad = fmaxf(fabsf(lo), fabsf(hi)) * 1e-6f + 1e-30f;
    b.lo[a] = lo - pad;
    b.hi[a] = hi + pad;
  }
  return b;
}

__global__ void kCentroidBounds(const float *v1, const float *e1, const float *e2, int n,
                                uint32_t *bounds /* 6: lo xyz, hi xyz ordered */) {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float p0 = v1[3 * i + a];
      float c = p0 + (e1[3 * i + a] + e2[3 * i + a]) * (1.f / 3.f);
      lo[a] = fminf(lo[a], c);
      hi[a] = fmaxf(hi[a], c);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
      hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(&bounds[a], floatToOrdered(lo[a]));
      atomicMax(&bounds[3 + a], floatToOrdered(hi[a]));
    }
  }
}

__device__ __forceinline__ uint64_t expandBits21(uint32_t v) {
  uint64_t x = v & 0x1fffff;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

// Sort key: a 3-bit size class above 60 bits of Morton code (20 bits per
// axis). Triangles whose extent is a large fraction of the scene get the
// smallest classes, so the hierarchy separates them near the root instead of
// inflating the boxes of a deep chain of ancestors in the Morton order.
__global__ void kMorton(const float *v1, const float *e1, const float *e2, int n,
                        const uint32_t *bounds, uint64_t *keys, uint32_t *vals) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t q[3];
  float triExt = 0.f, sceneExt = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float lo = orderedToFloat(bounds[a]), hi = orderedToFloat(bounds[3 + a]);
    float p0 = v1[3 * i + a], p1 = p0 + e1[3 * i + a], p2 = p0 + e2[3 * i + a];
    float c = p0 + (e1[3 * i + a] + e2[3 * i + a]) * (1.f / 3.f);
    float ext = hi - lo;
    float u = ext > 0.f ? (c - lo) / ext : 0.5f;
    u = fminf(fmaxf(u, 0.f), 1.f);
    q[a] = (uint32_t)fminf(u * 1048576.f, 1048575.f);
    triExt = fmaxf(triExt, fmaxf(p0, fmaxf(p1, p2)) - fminf(p0, fminf(p1, p2)));
    sceneExt = fmaxf(sceneExt, ext);
  }
  // class 0: triangle spans >= 1/4 of the centroid extent ... class 7: < 1/512
  const float rel = sceneExt > 0.f ? triExt / sceneExt : 0.f;
  int cls = rel > 0.f ? (int)floorf(-log2f(rel)) - 1 : 7;
  cls = min(max(cls, 0), 7);
  keys[i] = ((uint64_t)cls << 60) |
            (((expandBits21(q[0]) << 2) | (expandBits21(q[1]) << 1) | expandBits21(q[2])));
  vals[i] = (uint32_t)i;
}

__device__ __forceinline__ int delta(const uint64_t *k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint64_t a = k[i], b = k[j];
  if (a == b) return 64 + __clz((uint32_t)(i ^ j));
  return __clzll((long long)(a ^ b));
}

// Karras 2012: internal node i spans a key range; children are either
// internal nodes or leaves (encoded ~leaf).
__global__ void kHierarchy(const uint64_t *k, int n, int *childL, int *childR, int *parentInner,
                           int *parentLeaf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(k, n, i, i - d);
  int lmax = 2;
  while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(k, n, i, j);
  int s = 0;
  int div = 2;
  int t = (l + div - 1) / div;
  while (true) {
    if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
    div <<= 1;
    t = (l + div - 1) / div;
  }
  int gamma = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  int left = (lo == gamma) ? ~gamma : gamma;
  int right = (hi == gamma + 1) ? ~(gamma + 1) : (gamma + 1);
  childL[i] = left;
  childR[i] = right;
  if (left >= 0) parentInner[left] = i; else parentLeaf[~left] = i;
  if (right >= 0) parentInner[right] = i; else parentLeaf[~right] = i;
}

// Bottom-up refit: the second thread to arrive at a node writes it.
__global__ void kRefit(const float *v1, const float *e1, const float *e2, const uint32_t *order,
                       int n, const int *childL, const int *childR, const int *parentInner,
                       const int *parentLeaf, int *flags, Aabb *innerBox, float4 *nodes) {
  int leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  int p = parentLeaf[leaf];
  while (p >= 0) {
    __threadfence();
    if (atomicAdd(&flags[p], 1) == 0) return;  // sibling not done yet
    __threadfence();
    int c[2] = {childL[p], childR[p]};
    Aabb b[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (c[s] < 0) {
        b[s] = triBox(v1, e1, e2, (int)order[~c[s]]);
      } else {
        volatile const float *vb = reinterpret_cast<volatile const float *>(&innerBox[c[s]]);
#pragma unroll
        for (int a = 0; a < 3; ++a) { b[s].lo[a] = vb[a]; b[s].hi[a] = vb[3 + a]; }
      }
    }
    Aabb u;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      u.lo[a] = fminf(b[0].lo[a], b[1].lo[a]);
      u.hi[a] = fmaxf(b[0].hi[a], b[1].hi[a]);
    }
    innerBox[p] = u;
    float4 *N = nodes + 4 * (size_t)p;
    N[0] = make_float4(b[0].lo[0], b[0].hi[0], b[0].lo[1], b[0].hi[1]);
    N[1] = make_float4(b[1].lo[0], b[1].hi[0], b[1].lo[1], b[1].hi[1]);
    N[2] = make_float4(b[0].lo[2], b[0].hi[2], b[1].lo[2], b[1].hi[2]);
    N[3] = make_float4(__int_as_float(c[0]), __int_as_float(c[1]), 0.f, 0.f);
    p = (p == 0) ? -1 : parentInner[p];
  }
}

__global__ void kReorder(const float *v1, const float *e1, const float *e2, const uint32_t *order,
                         int n, float4 *tris) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int i = (int)order[j];
  tris[3 * (size_t)j] = make_float4(v1[3 * i], v1[3 * i + 1], v1[3 * i + 2], __int_as_float(i));
  tris[3 * (size_t)j + 1] = make_float4(e1[3 * i], e1[3 * i + 1], e1[3 * i + 2], 0.f);
  tris[3 * (size_t)j + 2] = make_float4(e2[3 * i], e2[3 * i + 1], e2[3 * i + 2], 0.f);
}

__global__ void kSingle(const float *v1, const float *e1, const float *e2, float4 *nodes,
                        float4 *tris) {
  Aabb b = triBox(v1, e1, e2, 0);
  nodes[0] = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
  nodes[1] = nodes[0];
  nodes[2] = make_float4(b.lo[2], b.hi[2], b.lo[2], b.hi[2]);
  nodes[3] = make_float4(__int_as_float(~0), __int_as_float(~0), 0.f, 0.f);
  tris[0] = make_float4(v1[0], v1[1], v1[2], __int_as_float(0));
  tris[1] = make_float4(e1[0], e1[1], e1[2], 0.f);
  tris[2] = make_float4(e2[0], e2[1], e2[2], 0.f);
}

} // namespace

} // namespace vsr
