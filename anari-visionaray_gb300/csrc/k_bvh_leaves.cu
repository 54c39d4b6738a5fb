// Leaf collapse for the triangle BVHs of world commits. Both builders make
// one triangle per leaf. A bottom-up surface-area-heuristic pass turns small
// subtrees into leaves of up to maxLeaf triangles where that lowers the
// expected cost of a ray (an inner-node visit tests both child boxes; a
// triangle test is priced at three quarters of one), so rays visit fewer
// inner nodes. The triangles are then put in depth-first leaf order, which makes
// every subtree's triangles contiguous, and the child links of the nodes
// that remain are rewritten to the (first, count) leaf codes of
// vsr_device.h. The remaining inner nodes are then stored in depth-first
// order (a node's left child right after it, its subtree contiguous), which
// drops the collapsed subtrees' nodes. Closest hits are ordered by (t,
// instance, triangle), so the collapsed tree gives the same hits as the one
// it came from.
#include "bvh_kernels.cuh"

namespace vsr {
namespace {

// relative costs (measured on the 1M-triangle sphere scene with a PLOC
// search radius of 16: a triangle test priced at 0.5 / 0.75 / 1 inner-node
// visits gave 202.4 / 200.0 / 200.9 ms per frame)
constexpr float kCostInner = 1.f;  // one inner-node visit (both child boxes)
constexpr float kCostTri = 0.75f;  // one triangle test
constexpr int kBlock = 256;

__device__ __forceinline__ float halfArea(float lx, float hx, float ly, float hy, float lz,
                                          float hz) {
  const float dx = hx - lx, dy = hy - ly, dz = hz - lz;
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int2 childLinks(const float4 *nodes, int p) {
  const int4 c = *reinterpret_cast<const int4 *>(nodes + 4 * (size_t)p + 3);
  return make_int2(c.x, c.y);
}

// Parent links, 2 p + side (side 1: the right child); -1 above the root.
// The builders' leaves hold one triangle each (code ~i, count bits 0).
// Links out of range (only in a malformed tree) are skipped; the walks below
// then end early and report it.
__global__ void kLinks(const float4 *nodes, int numInner, int *parentInner, int *parentLeaf) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= numInner) return;
  const int2 c = childLinks(nodes, p);
  const int ch[2] = {c.x, c.y};
  for (int s = 0; s < 2; ++s) {
    if (ch[s] > 0 && ch[s] < numInner) parentInner[ch[s]] = 2 * p + s;
    else if (ch[s] < 0 && ~ch[s] <= numInner) parentLeaf[~ch[s]] = 2 * p + s;
  }
  if (p == 0) parentInner[0] = -1;
}

// Bottom-up, one thread per triangle walking to the root; the second thread
// to reach a node evaluates it: its triangle count, its cheaper cost
// (cost x half area of the box), and whether it becomes a leaf (never the
// root). Children's results are read from L2: other SMs wrote them.
__global__ void kLeafCost(const float4 *nodes, int n, const int *parentInner,
                          const int *parentLeaf, int maxLeaf, int *flags, int *count, float *cost,
                          int *collapse, int *inner, int *bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int q = parentLeaf[i] >> 1;
  for (int steps = 0; q >= 0; ++steps) {
    if (q >= n - 1 || steps >= n) {  // not a tree: give up, reported to the host
      atomicOr(bad, 1);
      return;
    }
    __threadfence();
    if (atomicAdd(&flags[q], 1) == 0) return;  // the sibling's subtree is not done yet
    __threadfence();
    const float4 *N = nodes + 4 * (size_t)q;
    const float4 n0 = N[0], n1 = N[1], n2 = N[2];
    const int2 c = childLinks(nodes, q);
    const float a0 = halfArea(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y);
    const float a1 = halfArea(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w);
    const float A = halfArea(fminf(n0.x, n1.x), fmaxf(n0.y, n1.y), fminf(n0.z, n1.z),
                             fmaxf(n0.w, n1.w), fminf(n2.x, n2.z), fmaxf(n2.y, n2.w));
    const int k0 = c.x < 0 ? 1 : __ldcg(count + c.x);
    const int k1 = c.y < 0 ? 1 : __ldcg(count + c.y);
    const float c0 = c.x < 0 ? kCostTri * a0 : __ldcg(cost + c.x);
    const float c1 = c.y < 0 ? kCostTri * a1 : __ldcg(cost + c.y);
    const int k = k0 + k1;
    const float split = kCostInner * A + c0 + c1;
    const float leaf = kCostTri * (float)k * A;
    const bool col = q != 0 && k <= maxLeaf && leaf <= split;
    count[q] = k;
    cost[q] = col ? leaf : split;
    collapse[q] = col ? 1 : 0;
    // inner nodes that stay in q's subtree (none if q becomes a leaf)
    inner[q] = col ? 0
                   : 1 + (c.x < 0 ? 0 : __ldcg(inner + c.x)) + (c.y < 0 ? 0 : __ldcg(inner + c.y));
    const int up = parentInner[q];
    q = up >= 0 ? up >> 1 : -1;
  }
}

// Position in depth-first leaf order of the first triangle under the link
// `link` (2 p + side of the element's parent), found by walking to the
// root and adding the triangle count of every left sibling passed; `top`
// gets the topmost collapsed node on the way (-1 if none).
__device__ __forceinline__ int dfsFirst(const float4 *nodes, int numInner,
                                        const int *parentInner, const int *count,
                                        const int *collapse, int link, int &top, int *bad) {
  int off = 0;
  top = -1;
  for (int steps = 0; link >= 0; ++steps) {
    const int p = link >> 1;
    if (p >= numInner || steps >= numInner) {
      atomicOr(bad, 1);
      return 0;
    }
    if (link & 1) {
      const int left = childLinks(nodes, p).x;
      off += left < 0 ? 1 : count[left];
    }
    if (collapse[p]) top = p;
    link = parentInner[p];
  }
  return off;
}

// Per inner node: its first triangle's depth-first position, and whether it
// stays an inner node (neither it nor an ancestor collapsed).
__global__ void kNodeOrder(const float4 *nodes, int numInner, const int *parentInner,
                           const int *count, const int *collapse, int *first, int *alive,
                           int *bad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= numInner) return;
  int top;
  first[p] = dfsFirst(nodes, numInner, parentInner, count, collapse, parentInner[p], top, bad);
  alive[p] = (top < 0 && !collapse[p]) ? 1 : 0;
}

__global__ void kTriOrder(const float4 *nodes, int n, const int *parentInner,
                          const int *parentLeaf, const int *count, const int *collapse,
                          int *pos, int *bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int top;
  pos[i] = dfsFirst(nodes, n - 1, parentInner, count, collapse, parentLeaf[i], top, bad);
  if (pos[i] < 0 || pos[i] >= n) {  // only for a malformed tree; the scatter skips it
    atomicOr(bad, 1);
    pos[i] = -1;
  }
}

// The remaining inner nodes' child links: a triangle's new position, a
// collapsed child's (first, count) leaf code, or the inner child as it was.
__global__ void kRelink(float4 *nodes, int numInner, const int *alive, const int *collapse,
                        const int *count, const int *first, const int *pos) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= numInner || !alive[p]) return;
  const int2 c = childLinks(nodes, p);
  int out[2] = {c.x, c.y};
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int ch = out[s];
    if (ch < 0)
      out[s] = ~ch <= numInner ? ~pos[~ch] : ch;  // n = numInner + 1 triangles
    else if (ch < numInner && collapse[ch])
      out[s] = ~(int)((uint32_t)first[ch] | ((uint32_t)(count[ch] - 1) << kLeafCountShift));
  }
  nodes[4 * (size_t)p + 3] = make_float4(__int_as_float(out[0]), __int_as_float(out[1]), 0.f, 0.f);
}

// Depth-first (preorder) position of every remaining inner node: one for
// each ancestor, plus the remaining inner nodes of the left subtree of every
// ancestor whose right subtree holds the node (the links are the relinked
// ones: collapsed and triangle children are negative and count none).
__global__ void kNodePreorder(const float4 *nodes, int numInner, const int *parentInner,
                              const int *alive, const int *inner, int *pre, int *bad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= numInner || !alive[p]) return;
  int off = 0;
  for (int link = parentInner[p], steps = 0; link >= 0; ++steps) {
    const int q = link >> 1;
    if (q >= numInner || steps >= numInner) {
      atomicOr(bad, 1);
      break;
    }
    ++off;
    if (link & 1) {
      const int left = childLinks(nodes, q).x;
      if (left >= 0) off += inner[left];
    }
    link = parentInner[q];
  }
  pre[p] = off;
}

__global__ void kNodeScatter(const float4 *nodes, int numInner, const int *alive, const int *pre,
                             const int *kept, float4 *out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= numInner || !alive[p] || pre[p] < 0 || pre[p] >= *kept) return;
  const float4 *N = nodes + 4 * (size_t)p;
  float4 *O = out + 4 * (size_t)pre[p];
  O[0] = N[0];
  O[1] = N[1];
  O[2] = N[2];
  const int2 c = childLinks(nodes, p);
  O[3] = make_float4(__int_as_float(c.x >= 0 ? pre[c.x] : c.x),
                     __int_as_float(c.y >= 0 ? pre[c.y] : c.y), 0.f, 0.f);
}

__global__ void kScatterTris(const float4 *in, int n, const int *pos, float4 *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || pos[i] < 0) return;
  const size_t j = (size_t)pos[i];
  out[3 * j] = in[3 * (size_t)i];
  out[3 * j + 1] = in[3 * (size_t)i + 1];
  out[3 * j + 2] = in[3 * (size_t)i + 2];
}

} // namespace

cudaError_t collapseLeaves(float4 *nodes, int numInner, float4 *tris, int n, int maxLeaf,
                           int *numNodesOut, cudaStream_t stream) {
  *numNodesOut = numInner;
  if (maxLeaf <= 1 || n < 3 || numInner != n - 1) return cudaSuccess;
  if (maxLeaf > (1 << (32 - kLeafCountShift))) maxLeaf = 1 << (32 - kLeafCountShift);
  if ((uint32_t)n > kLeafFirstMask) return cudaErrorInvalidValue;
  cudaError_t err = cudaSuccess;
  int *ints = nullptr;
  float *cost = nullptr;
  float4 *trisIn = nullptr, *nodesOut = nullptr;
  int kept = 0, badHost = 0;
  // parentInner, flags, count, collapse, first, alive, inner, pre: numInner
  // each; parentLeaf, pos: n each; the malformed-tree flag
  const size_t ni = (size_t)numInner, nt = (size_t)n;
  const int gi = (numInner + kBlock - 1) / kBlock, gt = (n + kBlock - 1) / kBlock;
  int *parentInner, *flags, *count, *collapse, *first, *alive, *inner, *pre, *parentLeaf, *pos,
      *bad;
  if ((err = cudaMallocAsync((void **)&ints, (8 * ni + 2 * nt + 1) * sizeof(int), stream)) !=
      cudaSuccess)
    return err;
  parentInner = ints;
  flags = parentInner + ni;
  count = flags + ni;
  collapse = count + ni;
  first = collapse + ni;
  alive = first + ni;
  inner = alive + ni;
  pre = inner + ni;
  parentLeaf = pre + ni;
  pos = parentLeaf + nt;
  bad = pos + nt;
  if ((err = cudaMallocAsync((void **)&cost, ni * sizeof(float), stream)) != cudaSuccess) goto done;
  if ((err = cudaMallocAsync((void **)&trisIn, 3 * nt * sizeof(float4), stream)) != cudaSuccess)
    goto done;
  if ((err = cudaMallocAsync((void **)&nodesOut, 4 * ni * sizeof(float4), stream)) != cudaSuccess)
    goto done;
  // links not set by kLinks (only in a malformed tree) read -1: walks end there
  if ((err = cudaMemsetAsync(ints, 0xff, (8 * ni + 2 * nt) * sizeof(int), stream)) != cudaSuccess)
    goto done;
  if ((err = cudaMemsetAsync(flags, 0, ni * sizeof(int), stream)) != cudaSuccess) goto done;
  if ((err = cudaMemsetAsync(bad, 0, sizeof(int), stream)) != cudaSuccess) goto done;
  if ((err = cudaMemcpyAsync(trisIn, tris, 3 * nt * sizeof(float4), cudaMemcpyDeviceToDevice,
                             stream)) != cudaSuccess)
    goto done;
  kLinks<<<gi, kBlock, 0, stream>>>(nodes, numInner, parentInner, parentLeaf);
  kLeafCost<<<gt, kBlock, 0, stream>>>(nodes, n, parentInner, parentLeaf, maxLeaf, flags, count,
                                       cost, collapse, inner, bad);
  kNodeOrder<<<gi, kBlock, 0, stream>>>(nodes, numInner, parentInner, count, collapse, first,
                                        alive, bad);
  kTriOrder<<<gt, kBlock, 0, stream>>>(nodes, n, parentInner, parentLeaf, count, collapse, pos,
                                       bad);
  kRelink<<<gi, kBlock, 0, stream>>>(nodes, numInner, alive, collapse, count, first, pos);
  kScatterTris<<<gt, kBlock, 0, stream>>>(trisIn, n, pos, tris);
  kNodePreorder<<<gi, kBlock, 0, stream>>>(nodes, numInner, parentInner, alive, inner, pre, bad);
  // inner[0], the root's count, is the number of nodes kept
  kNodeScatter<<<gi, kBlock, 0, stream>>>(nodes, numInner, alive, pre, inner, nodesOut);
  if ((err = cudaGetLastError()) != cudaSuccess) goto done;
  if ((err = cudaMemcpyAsync(&kept, inner, sizeof(int), cudaMemcpyDeviceToHost, stream)) !=
      cudaSuccess)
    goto done;
  if ((err = cudaMemcpyAsync(&badHost, bad, sizeof(int), cudaMemcpyDeviceToHost, stream)) !=
      cudaSuccess)
    goto done;
  if ((err = cudaStreamSynchronize(stream)) != cudaSuccess) goto done;
  if (badHost || kept < 1 || kept > numInner) {
    err = cudaErrorUnknown;
    goto done;
  }
  if ((err = cudaMemcpyAsync(nodes, nodesOut, 4 * (size_t)kept * sizeof(float4),
                             cudaMemcpyDeviceToDevice, stream)) != cudaSuccess)
    goto done;
  *numNodesOut = kept;
done:
  if (nodesOut) cudaFreeAsync(nodesOut, stream);
  if (trisIn) cudaFreeAsync(trisIn, stream);
  if (cost) cudaFreeAsync(cost, stream);
  cudaFreeAsync(ints, stream);
  return err;
}

} // namespace vsr
