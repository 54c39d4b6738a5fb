// Volume-only raycast worlds at one sample per pixel: rayMarchVolume<0>
// (renderer/VolumeIntegration.h:374-468) split into three passes so that
// every lane of every warp marches samples:
//
//  1. kVolumeSetup, one thread per pixel: camera ray, clip planes, closest
//     volume box entry. Pixels with nothing to march are written at once.
//     The rays of each warp (up to 32 neighbouring pixels of a row) form a
//     group and are appended to a compact ray list; each ray is cut into
//     segments of kSegSamples consecutive samples, and the group gets one
//     work unit per segment index of its longest ray.
//  2. kVolumeSegments, one warp per work unit: lane i marches segment j of
//     the group's ray i. Neighbouring pixels at the same depth keep the
//     texture fetches of a warp coherent. Each segment is composited front
//     to back in the reference's order, from (C, A, T) = (0, 0, 1).
//  3. kVolumeCombine, one warp per group, one lane per ray (or, compiled
//     with VSR_SEG_FUSE, done by the warp that finishes a group's last work
//     unit, which a per-group counter incremented after a memory fence
//     tells; slower, see there): the segment composites are combined in
//     order with the front-to-back operator
//       (C, A, T)front o (C, A, T)back = (Cf + Tf Cb, Af + Tf Ab, Tf Tb).
//     A segment after which the accumulated alpha reaches 0.99, and any part
//     of a ray the segments did not cover, is marched again by the whole warp
//     in chunks of 64 samples, with the reference's test (alpha < 0.99 and
//     t <= tmax) before every sample.
//
// Sample positions are bit-identical to the reference's sequential t += dt
// and every sample's value and step opacity are the reference's; only the
// association of the compositing sums differs.
#include "render_common.cuh"
#include "kernels.h"

#include <mutex>

namespace vsr {
namespace {

#ifndef VSR_SEG_MIN_BLOCKS
#define VSR_SEG_MIN_BLOCKS 1
#endif
#ifndef VSR_SETUP_MIN_BLOCKS
// 8 blocks of 256 per SM (32 registers): a 512x512 frame's set-up grid is
// resident in one wave (a 128^3 blob volume at 512x512: 0.0658 ms per
// frame against 0.0665 at 4 blocks and 0.0673 at 6)
#define VSR_SETUP_MIN_BLOCKS 8
#endif
#ifndef VSR_COMBINE_PREFETCH
#define VSR_COMBINE_PREFETCH 8
#endif
#ifndef VSR_VOLUME_REFILL
// 1: the one-pass marcher (kVolumeRefill): measured 0.21-0.24 ms per frame
// of a 128^3 blob volume at 512x512 (refill every 8 / 12 / 16 samples, 3 or
// 4 blocks per SM) against 0.066 ms for the three passes
#define VSR_VOLUME_REFILL 0
#endif
#ifndef VSR_REFILL_SAMPLES
#define VSR_REFILL_SAMPLES 8
#endif
#ifndef VSR_REFILL_MIN_BLOCKS
#define VSR_REFILL_MIN_BLOCKS 4
#endif
#ifndef VSR_SEG_FUSE
// 1: the combination inside the segments pass (measured 0.125 ms per frame
// of the same volume against 0.067 ms with its own pass: the last groups'
// combinations run at the end with few warps, and the fused kernel spills
// at the segments pass's 64 registers)
#define VSR_SEG_FUSE 0
#endif
#ifndef VSR_SEG_FUSED_MIN_BLOCKS
#define VSR_SEG_FUSED_MIN_BLOCKS 4  // 64 registers, as the segments pass alone
#endif
#ifndef VSR_SEG_FUSED_PREFETCH
#define VSR_SEG_FUSED_PREFETCH 4
#endif
#ifndef VSR_SEG_DYNAMIC
#define VSR_SEG_DYNAMIC 0
#endif
constexpr int kSegSamples = VSR_SEG_SAMPLES;
constexpr unsigned kFull = 0xffffffffu;

struct MarchItem {
  float4 o;   // voxel-space origin, tmin
  float4 d;   // voxel-space direction, tmax
  int4 info;  // pixel, volume index, -, segment count
};

// a group: the rays one setup warp appended, and its work units
struct MarchGroup {
  int itemBase, numRays, unitBase, numUnits;
};

// composite of one segment: (C.rgb, A), (T, t of its first sample, t after
// its last sample inside [tmin, tmax], sample count)
struct SegOut {
  float4 c;
  float4 m;
};

// zeroes the set-up pass's counters; the set-up pass is its programmatic
// dependent and computes its rays before it waits for this grid
__global__ void kMarchReset(unsigned *counters) {
  if (threadIdx.x < 4) counters[threadIdx.x] = 0u;
  asm volatile("griddepcontrol.launch_dependents;\n" ::);
}

__global__ void __launch_bounds__(256, VSR_SETUP_MIN_BLOCKS) kVolumeSetup(DScene S, DCamera C, DRenderer R, DFrame F,
                                                    MarchScratch M) {
  // the segments pass may launch now; it waits for this grid's results
  asm volatile("griddepcontrol.launch_dependents;\n" ::);
  MarchItem *items = reinterpret_cast<MarchItem *>(M.items);
  MarchGroup *groups = reinterpret_cast<MarchGroup *>(M.groups);
  const int numPix = F.width * F.height;
  const int lane = threadIdx.x & 31;
  const float4 bg = make_float4(R.bg[0], R.bg[1], R.bg[2], R.bg[3]);
  Rng none;
  none.state = 0;
  // block-uniform loop: the block synchronises once per iteration
  for (int blockBase = blockIdx.x * blockDim.x; blockBase < numPix;
       blockBase += gridDim.x * blockDim.x) {
    const int p = blockBase + (int)threadIdx.x;
    bool march = false;
    MarchItem it;
    int nseg = 0;
    if (p < numPix) {
      const int x = p % F.width, y = p / F.width;
      Ray ray = primaryRay<false>(C, none, (float)x, (float)y, (float)F.width, (float)F.height);
      clipRay(ray, R);
      int vIdx = -1;
      float vT = FLT_MAX, vFar = 0.f;
      float3 vlo = f3(0.f), vld = f3(0.f);
      for (int i = 0; i < S.numInstances; ++i) {
        const DInstance &I = S.instances[i];
        const DGroup &G = S.groups[I.group];
        for (int k = G.volBegin; k < G.volEnd; ++k) {
          const int vi = S.groupVolumes[k];
          float3 lo, ld;
          localRay(I, ray.o, ray.d, lo, ld);
          BoxHit bh = intersectBox(lo, ld, S.volumes[vi].boundsLo, S.volumes[vi].boundsHi);
          const bool h = bh.hit && bh.tfar >= ray.tmin && bh.tnear <= ray.tmax;
          const float t = fmaxf(ray.tmin, bh.tnear);
          if (h && t < vT) { vT = t; vFar = bh.tfar; vIdx = vi; vlo = lo; vld = ld; }
        }
      }
      if (vIdx >= 0) {
        const DVolume &V = S.volumes[vIdx];
        const float3 lo = vlo, ld = vld;
        const float tmin = vT;
        const float tmax = fminf(ray.tmax, vFar);
        const float3 Sv = ld3(V.S);
        const float3 o = Sv * (lo + ld3(V.T));
        const float3 d = Sv * ld;
        it.o = make_float4(o.x, o.y, o.z, tmin);
        it.d = make_float4(d.x, d.y, d.z, tmax);
        it.info = make_int4(p, vIdx, 0, 0);
        march = tmin <= tmax;
        const float dt = V.cellSize * R.samplingRateInv;
        if (march && dt > 0.f) {
          // samples in [tmin, tmax] plus one for rounding; pass 3 marches on
          // where the segments end short of tmax
          const float ns = floorf((tmax - tmin) / dt) + 2.f;
          if (ns < (float)kMaxMarchSteps) nseg = ((int)ns + kSegSamples - 1) / kSegSamples;
        }
      }
      if (!march) writeSample(F, x, y, false, bg, 1e31f, f3(0.f), f3(0.f));
    }
    // the counters this block adds to were zeroed by kMarchReset
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    const unsigned mask = __ballot_sync(kFull, march);
    const int numRays = __popc(mask);
    const int rank = __popc(mask & ((1u << lane) - 1u));
    const int units = (int)__reduce_max_sync(kFull, (unsigned)nseg);
    // one set of atomics per block: warp totals are scanned in shared memory
    __shared__ unsigned sTot[3][8], sBase[3];
    const int warp = threadIdx.x >> 5;
    if (lane == 0) {
      sTot[0][warp] = (unsigned)numRays;
      sTot[1][warp] = mask ? 1u : 0u;
      sTot[2][warp] = (unsigned)units;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      unsigned sum = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        const unsigned v = sTot[threadIdx.x][w];
        sTot[threadIdx.x][w] = sum;
        sum += v;
      }
      const int which = threadIdx.x == 0 ? 0 : (threadIdx.x == 1 ? 3 : 2);
      sBase[threadIdx.x] = sum ? atomicAdd(&M.counters[which], sum) : 0u;
    }
    __syncthreads();
    const unsigned off = sBase[0] + sTot[0][warp];
    const unsigned gid = sBase[1] + sTot[1][warp];
    const unsigned ub = sBase[2] + sTot[2][warp];
    __syncthreads();  // sTot and sBase are reused by the next iteration
    if (!mask) continue;
    int numUnits = units;
    if (units && (ub > M.unitCap || (unsigned)units > M.unitCap - ub)) {
      // no room: these rays are marched whole; the part of the unit range
      // inside the list is marked unused
      const unsigned end = min(ub + (unsigned)units, M.unitCap);
      for (unsigned k = ub + lane; k < end; k += 32) M.unitGroup[k] = -1;
      numUnits = 0;
      nseg = 0;
    } else {
      for (int k = lane; k < units; k += 32) M.unitGroup[ub + k] = (int)gid;
    }
    if (march) {
      it.info.w = nseg;
      items[off + rank] = it;
    }
    if (lane == 0) {
      groups[gid] = MarchGroup{(int)off, numRays, (int)ub, numUnits};
      M.groupDone[gid] = 0u;
    }
  }
}

// t after n sequential additions t += dt, exactly as that loop computes it.
// Inside one binade [2^e, 2^(e+1)) t is a multiple of u = ulp(t), so an
// addition whose exact sum stays below 2^(e+1) adds round_u(dt), the same
// for every step, unless dt is an exact tie between multiples of u; k such
// additions are then the single exact fma t + k*round_u(dt). A step whose
// result is at most 2^(e+1) - u had its exact sum below 2^(e+1) - u/2, so
// it did not leave the binade. Steps that cross a binade, ties and t <= 0
// are made literally.
__device__ float advanceT(float t, float dt, int n) {
  for (int round = 0; n > 0 && round < 64; ++round) {
    const int bt = (__float_as_int(t) >> 23) & 0xff;  // biased exponent
    if (t > 0.f && bt >= 24 && bt <= 253) {
      const float u = __int_as_float((bt - 23) << 23);
      const float invU = __int_as_float((277 - bt) << 23);
      const float q = dt * invU;  // exact: power-of-two scaling
      const float r = rintf(q);
      if (q < 16777216.f && fabsf(q - r) != 0.5f) {
        const float dq = r * u;
        const float lim = __int_as_float((bt + 1) << 23) - u;  // last t a step may reach
        int k = n;
        if (dq > 0.f) {
          const float kf = floorf((lim - t) / dq);  // estimate, made exact below
          if (kf < (float)k) k = kf > 0.f ? (int)kf : 0;
          while (k > 0 && fmaf((float)k, dq, t) > lim) --k;
        }
        if (k > 0) {
          t = fmaf((float)k, dq, t);
          n -= k;
          if (n == 0) break;
        }
      }
    }
    t += dt;
    --n;
  }
  for (; n > 0; --n) t += dt;
  return t;
}

// Sample positions of one 64-sample chunk: lane `lane` takes the values
// after 2*lane and 2*lane+1 additions, by the closed form of advanceT when
// the whole chunk stays inside t0's binade, else literally.
__device__ __forceinline__ void chunkT(float t0, float dt, int lane, float &ta, float &tb) {
  const int bt = (__float_as_int(t0) >> 23) & 0xff;
  if (t0 > 0.f && bt >= 24 && bt <= 253) {
    const float u = __int_as_float((bt - 23) << 23);
    const float invU = __int_as_float((277 - bt) << 23);
    const float q = dt * invU;
    const float r = rintf(q);
    if (q < 16777216.f && fabsf(q - r) != 0.5f) {
      const float dq = r * u;
      // every step's result, up to t0 + 63 dq, at most 2^(e+1) - u
      if (fmaf(63.f, dq, t0) < __int_as_float((bt + 1) << 23)) {
        ta = fmaf((float)(2 * lane), dq, t0);
        tb = fmaf((float)(2 * lane + 1), dq, t0);
        return;
      }
    }
  }
  float t = t0;
  for (int k = 0; k < 2 * lane; ++k) t += dt;
  ta = t;
  tb = t + dt;
}

// one sample: classified colour premultiplied by the step opacity
__device__ __forceinline__ void marchSample(const DVolume &V, const float4 *tf, float3 o, float3 d,
                                            float t, float expo, bool hw, float &c0, float &c1,
                                            float &c2, float &a, float &tr) {
  const float4 sm = classify(V, tf, fieldAt(V, o + d * t, hw), hw);
  const float stepTr = hw ? __powf(1.f - sm.w, expo) : powf(1.f - sm.w, expo);
  a = 1.f - stepTr;
  tr = stepTr;
  c0 = a * sm.x; c1 = a * sm.y; c2 = a * sm.z;
}

// inclusive warp scan of the front-to-back operator
__device__ __forceinline__ void overScan(float &c0, float &c1, float &c2, float &a, float &tr) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const float pc0 = __shfl_up_sync(kFull, c0, off);
    const float pc1 = __shfl_up_sync(kFull, c1, off);
    const float pc2 = __shfl_up_sync(kFull, c2, off);
    const float pa = __shfl_up_sync(kFull, a, off);
    const float ptr = __shfl_up_sync(kFull, tr, off);
    if (lane >= off) {  // (prev) o (mine)
      c0 = pc0 + ptr * c0;
      c1 = pc1 + ptr * c1;
      c2 = pc2 + ptr * c2;
      a = pa + ptr * a;
      tr = ptr * tr;
    }
  }
}

// The whole warp marches one ray from tChunk on, 64 samples per chunk, two
// consecutive ones per lane: each lane composites its pair, the warp scans
// the pairs, and the accumulated alpha before every sample decides whether
// it is kept. Warp-uniform arguments and state.
__device__ void warpMarch(const DVolume &V, const float4 *tf, float3 o, float3 d, float t1,
                          float dt, float expo, bool hw, float tChunk, float &Cr, float &Cg,
                          float &Cb, float &A, float &T, uint32_t &err,
                          unsigned long long &samples) {
  const int lane = threadIdx.x & 31;
  int steps = 0;
  while (tChunk <= t1 && A < 0.99f) {
    if (!(dt > 0.f) || (steps += 64) > kMaxMarchSteps) {
      err |= ERR_MARCH_LIMIT;
      break;
    }
    float ta, tb;
    chunkT(tChunk, dt, lane, ta, tb);
    const float tLast = __shfl_sync(kFull, tb, 31);
    const bool inA = ta <= t1, inB = tb <= t1;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, aa = 0.f, atr = 1.f;  // first sample of the pair
    float b0 = 0.f, b1 = 0.f, b2 = 0.f, ba = 0.f, btr = 1.f;  // second
    if (inA) marchSample(V, tf, o, d, ta, expo, hw, a0, a1, a2, aa, atr);
    if (inB) marchSample(V, tf, o, d, tb, expo, hw, b0, b1, b2, ba, btr);
    float c0 = a0 + atr * b0, c1 = a1 + atr * b1, c2 = a2 + atr * b2;
    float al = aa + atr * ba, tr = atr * btr;
    overScan(c0, c1, c2, al, tr);
    // exclusive prefix (everything before this lane's pair)
    float p0 = __shfl_up_sync(kFull, c0, 1), p1 = __shfl_up_sync(kFull, c1, 1);
    float p2 = __shfl_up_sync(kFull, c2, 1), pa = __shfl_up_sync(kFull, al, 1);
    float pt = __shfl_up_sync(kFull, tr, 1);
    if (lane == 0) { p0 = 0.f; p1 = 0.f; p2 = 0.f; pa = 0.f; pt = 1.f; }
    // prefix through the first sample of the pair
    const float x0 = p0 + pt * a0, x1 = p1 + pt * a1, x2 = p2 + pt * a2;
    const float xa = pa + pt * aa, xt = pt * atr;
    const bool keepA = inA && (A + T * pa) < 0.99f;
    const bool keepB = inB && (A + T * xa) < 0.99f;
    const int cut = __popc(__ballot_sync(kFull, keepA)) + __popc(__ballot_sync(kFull, keepB));
    if (cut > 0) {
      // composite of the first `cut` samples: the prefix before pair cut/2,
      // plus its first sample when cut is odd; all 64 is lane 31's scan
      const int src = cut == 64 ? 31 : (cut >> 1);
      const bool odd = cut & 1;
      float s0 = cut == 64 ? c0 : (odd ? x0 : p0);
      float s1 = cut == 64 ? c1 : (odd ? x1 : p1);
      float s2 = cut == 64 ? c2 : (odd ? x2 : p2);
      float sa = cut == 64 ? al : (odd ? xa : pa);
      float st = cut == 64 ? tr : (odd ? xt : pt);
      s0 = __shfl_sync(kFull, s0, src);
      s1 = __shfl_sync(kFull, s1, src);
      s2 = __shfl_sync(kFull, s2, src);
      sa = __shfl_sync(kFull, sa, src);
      st = __shfl_sync(kFull, st, src);
      Cr += T * s0; Cg += T * s1; Cb += T * s2;
      A += T * sa;
      T *= st;
      samples += cut;
    }
    if (cut < 64) break;  // ran past tmax or reached alpha 0.99
    tChunk = tLast + dt;
  }
}

__device__ __forceinline__ void stageTable(const DScene &S, float4 *sTF, int stageTF) {
  if (stageTF) {
    const DVolume &V0 = S.volumes[0];
    for (int i = threadIdx.x; i < V0.tfSize; i += blockDim.x) sTF[i] = V0.tf[i];
    __syncthreads();
  }
}

// Pass 2: lane i of a warp marches segment j of work unit u's group's ray i.
__device__ __forceinline__ void marchUnit(const DScene &S, const DRenderer &R,
                                          const MarchScratch &M, const float4 *sTF, int stageTF,
                                          unsigned u, int lane) {
  const MarchItem *items = reinterpret_cast<const MarchItem *>(M.items);
  const MarchGroup *groups = reinterpret_cast<const MarchGroup *>(M.groups);
  SegOut *segOut = reinterpret_cast<SegOut *>(M.segOut);
  const int gid = M.unitGroup[u];
  if (gid < 0) return;
  const MarchGroup G = groups[gid];
  if (lane >= G.numRays) return;
  const MarchItem it = items[G.itemBase + lane];
  const int j = (int)u - G.unitBase;
  if (j >= it.info.w) return;
  const bool hw = R.hwFilter != 0;
  const DVolume &V = S.volumes[it.info.y];
  const float4 *tf = (stageTF && it.info.y == 0) ? sTF : V.tf;
  const float3 o = f3(it.o.x, it.o.y, it.o.z), d = f3(it.d.x, it.d.y, it.d.z);
  const float t1 = it.d.w;
  const float dt = V.cellSize * R.samplingRateInv;
  const float expo = dt / V.unitDistance;
  const float tStart = advanceT(it.o.w, dt, j * kSegSamples);
  // field values first, so that the segment's texture fetches overlap
  float val[kSegSamples];
  float t = tStart, tEnd = tStart;
  int n = 0;
#pragma unroll
  for (int i = 0; i < kSegSamples; ++i) {
    if (t <= t1) {
      val[i] = fieldAt(V, o + d * t, hw);
      n = i + 1;
      tEnd = t + dt;
    }
    t += dt;
  }
  float C0 = 0.f, C1 = 0.f, C2 = 0.f, A = 0.f, T = 1.f;
#pragma unroll
  for (int i = 0; i < kSegSamples; ++i) {
    if (i < n) {
      const float4 sm = classify(V, tf, val[i], hw);
      const float stepTr = hw ? __powf(1.f - sm.w, expo) : powf(1.f - sm.w, expo);
      const float w = T * (1.f - stepTr);
      C0 += w * sm.x; C1 += w * sm.y; C2 += w * sm.z;
      A += w;
      T *= stepTr;
    }
  }
  SegOut so;
  so.c = make_float4(C0, C1, C2, A);
  so.m = make_float4(T, tStart, tEnd, __int_as_float(n));
  segOut[(size_t)u * 32 + lane] = so;
}

// Combination of one group, one lane per ray: the ray's segment composites
// in order, until the one after which the accumulated alpha reaches 0.99;
// rays with samples left (that segment, segments ending short of tmax, rays
// without segments) are then marched by the whole warp, one at a time.
template <bool Count, int kPf = VSR_COMBINE_PREFETCH>
__device__ __forceinline__ void combineGroup(const DScene &S, const DRenderer &R, const DFrame &F,
                             const MarchScratch &M, const float4 *sTF, int stageTF, int gid,
                             int lane, uint32_t &err, unsigned long long &samples) {
  const MarchItem *items = reinterpret_cast<const MarchItem *>(M.items);
  const MarchGroup *groups = reinterpret_cast<const MarchGroup *>(M.groups);
  const SegOut *segOut = reinterpret_cast<const SegOut *>(M.segOut);
  const int4 G = *reinterpret_cast<const int4 *>(groups + gid);  // itemBase, rays, unitBase
  const bool active = lane < G.y;
  MarchItem it{};
  float Cr = 0.f, Cg = 0.f, Cb = 0.f, A = 0.f, T = 1.f, tNext = 0.f;
  unsigned long long own = 0;
  if (active) {
    it = items[G.x + lane];
    tNext = it.o.w;
    const int nseg = it.info.w;
    const float4 *mine = reinterpret_cast<const float4 *>(segOut + (size_t)G.z * 32 + lane);
    bool stop = false;
    for (int j0 = 0; j0 < nseg && !stop; j0 += kPf) {
      float4 sc[kPf], sm[kPf];  // loads in flight together
#pragma unroll
      for (int k = 0; k < kPf; ++k)
        if (j0 + k < nseg) {
          // L2 loads: in the fused pass other SMs wrote them in this grid
          sc[k] = __ldcg(mine + (size_t)(j0 + k) * 64);
          sm[k] = __ldcg(mine + (size_t)(j0 + k) * 64 + 1);
        }
#pragma unroll
      for (int k = 0; k < kPf; ++k) {
        if (stop || j0 + k >= nseg) break;
        if (A + T * sc[k].w >= 0.99f) {  // alpha reaches 0.99 inside: march it again
          tNext = sm[k].y;
          stop = true;
          break;
        }
        Cr += T * sc[k].x; Cg += T * sc[k].y; Cb += T * sc[k].z;
        A += T * sc[k].w;
        T *= sm[k].x;
        tNext = sm[k].z;
        own += (unsigned)__float_as_int(sm[k].w);
      }
    }
  }
  const bool hw = R.hwFilter != 0;
  unsigned rest = __ballot_sync(kFull, active && tNext <= it.d.w && A < 0.99f);
  while (rest) {
    const int src = __ffs(rest) - 1;
    rest &= rest - 1;
    const float ox = __shfl_sync(kFull, it.o.x, src), oy = __shfl_sync(kFull, it.o.y, src);
    const float oz = __shfl_sync(kFull, it.o.z, src), dx = __shfl_sync(kFull, it.d.x, src);
    const float dy = __shfl_sync(kFull, it.d.y, src), dz = __shfl_sync(kFull, it.d.z, src);
    const float t1 = __shfl_sync(kFull, it.d.w, src);
    const int vIdx = __shfl_sync(kFull, it.info.y, src);
    float wr = __shfl_sync(kFull, Cr, src), wg = __shfl_sync(kFull, Cg, src);
    float wb = __shfl_sync(kFull, Cb, src), wa = __shfl_sync(kFull, A, src);
    float wt = __shfl_sync(kFull, T, src);
    const float t0 = __shfl_sync(kFull, tNext, src);
    const DVolume &V = S.volumes[vIdx];
    const float4 *tf = (stageTF && vIdx == 0) ? sTF : V.tf;
    const float dt = V.cellSize * R.samplingRateInv;
    unsigned long long extra = 0;
    warpMarch(V, tf, f3(ox, oy, oz), f3(dx, dy, dz), t1, dt, dt / V.unitDistance, hw, t0, wr, wg,
              wb, wa, wt, err, extra);
    if (lane == src) {
      Cr = wr; Cg = wg; Cb = wb; A = wa; T = wt;
      own += extra;
    }
  }
  if (active) {
    const float4 bg = make_float4(R.bg[0], R.bg[1], R.bg[2], R.bg[3]);
    const int p = it.info.x;
    const int y = p / F.width;
    const float4 res = make_float4(A * Cr + (1.f - A) * bg.x, A * Cg + (1.f - A) * bg.y,
                                   A * Cb + (1.f - A) * bg.z, A + (1.f - A) * bg.w);
    writeSample(F, p - y * F.width, y, false, res, 1e31f, f3(0.f), f3(0.f));
  }
  if (Count) samples += own;
}

// Pass 2: warp w marches work units w, w + warps, ...; Fused: and combines
// each group whose last unit it finished, then the groups without units.
template <bool Fused>
__global__ void __launch_bounds__(256, Fused ? VSR_SEG_FUSED_MIN_BLOCKS : VSR_SEG_MIN_BLOCKS)
    kVolumeSegments(DScene S, DRenderer R, DFrame F, MarchScratch M, int stageTF) {
  extern __shared__ float4 sTF[];
  stageTable(S, sTF, stageTF);
  // the set-up pass's ray list and counters are complete and visible
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::);
  const int lane = threadIdx.x & 31;
  const unsigned numUnits = min(M.counters[2], M.unitCap);
  const unsigned warps = gridDim.x * (blockDim.x >> 5);
  const unsigned warpId = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  uint32_t err = 0;
  unsigned long long samples = 0;
  for (unsigned u = warpId; u < numUnits; u += warps) {
    marchUnit(S, R, M, sTF, stageTF, u, lane);
    if (Fused) {
      const int gid = M.unitGroup[u];
      if (gid < 0) continue;
      // this unit's composites are visible before the count says so
      __threadfence();
      __syncwarp();
      unsigned last = 0;
      if (lane == 0) {
        const int n = reinterpret_cast<const MarchGroup *>(M.groups)[gid].numUnits;
        last = atomicAdd(&M.groupDone[gid], 1u) == (unsigned)n - 1u ? 1u : 0u;
      }
      if (__shfl_sync(kFull, last, 0)) {
        __threadfence();
        combineGroup<false, VSR_SEG_FUSED_PREFETCH>(S, R, F, M, sTF, stageTF, gid, lane, err,
                                                    samples);
      }
    }
  }
  if (Fused) {
    const MarchGroup *groups = reinterpret_cast<const MarchGroup *>(M.groups);
    const unsigned numGroups = M.counters[3];
    for (unsigned g = warpId; g < numGroups; g += warps)
      if (groups[g].numUnits == 0)
        combineGroup<false, VSR_SEG_FUSED_PREFETCH>(S, R, F, M, sTF, stageTF, (int)g, lane, err,
                                                    samples);
    if (err) atomicOr(F.errorFlags, err);
  }
}

// One-pass alternative (VSR_VOLUME_REFILL): persistent warps, one ray per
// lane marched sample after sample in the reference's order (the
// compositing sums are the reference's, not re-associated); every
// VSR_REFILL_SAMPLES samples the lanes whose ray ended take the next pixels
// (one atomic per warp on the frame's pixel counter), set up their ray (camera,
// clip planes, closest volume box entry) and write the pixels that miss
// every volume at once.
template <bool Count>
__global__ void __launch_bounds__(256, VSR_REFILL_MIN_BLOCKS)
    kVolumeRefill(DScene S, DCamera C, DRenderer R, DFrame F, MarchScratch M, int stageTF) {
  extern __shared__ float4 sTF[];
  stageTable(S, sTF, stageTF);
  // the pixel counter was zeroed by kMarchReset
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  const int lane = threadIdx.x & 31;
  const int numPix = F.width * F.height;
  const bool hw = R.hwFilter != 0;
  const float4 bg = make_float4(R.bg[0], R.bg[1], R.bg[2], R.bg[3]);
  Rng none;
  none.state = 0;
  bool active = false, exhausted = false;
  int pix = 0, vIdx = 0, steps = 0;
  float3 o = f3(0.f), d = f3(0.f);
  float t = 0.f, t1 = 0.f, dt = 0.f, expo = 0.f;
  float Cr = 0.f, Cg = 0.f, Cb = 0.f, A = 0.f, T = 1.f;
  uint32_t err = 0;
  unsigned long long samples = 0;
  auto finish = [&]() {
    const float4 res = make_float4(A * Cr + (1.f - A) * bg.x, A * Cg + (1.f - A) * bg.y,
                                   A * Cb + (1.f - A) * bg.z, A + (1.f - A) * bg.w);
    const int y = pix / F.width;
    writeSample(F, pix - y * F.width, y, false, res, 1e31f, f3(0.f), f3(0.f));
    active = false;
  };
  for (int guard = 0; guard < (1 << 30); ++guard) {
    // refill the lanes without a ray
    while (!exhausted) {
      const unsigned need = __ballot_sync(kFull, !active);
      if (!need) break;
      unsigned base = 0;
      if (lane == 0) base = atomicAdd(&M.counters[0], (unsigned)__popc(need));
      base = __shfl_sync(kFull, base, 0);
      if (base >= (unsigned)numPix) {
        exhausted = true;
        break;
      }
      if (!active) {
        const unsigned p = base + (unsigned)__popc(need & ((1u << lane) - 1u));
        if (p < (unsigned)numPix) {
          pix = (int)p;
          const int x = pix % F.width, y = pix / F.width;
          Ray ray = primaryRay<false>(C, none, (float)x, (float)y, (float)F.width, (float)F.height);
          clipRay(ray, R);
          int vi = -1;
          float vT = FLT_MAX, vFar = 0.f;
          float3 vlo = f3(0.f), vld = f3(0.f);
          for (int i = 0; i < S.numInstances; ++i) {
            const DInstance &I = S.instances[i];
            const DGroup &G = S.groups[I.group];
            for (int k = G.volBegin; k < G.volEnd; ++k) {
              const int w = S.groupVolumes[k];
              float3 lo, ld;
              localRay(I, ray.o, ray.d, lo, ld);
              BoxHit bh = intersectBox(lo, ld, S.volumes[w].boundsLo, S.volumes[w].boundsHi);
              const bool h = bh.hit && bh.tfar >= ray.tmin && bh.tnear <= ray.tmax;
              const float tt = fmaxf(ray.tmin, bh.tnear);
              if (h && tt < vT) { vT = tt; vFar = bh.tfar; vi = w; vlo = lo; vld = ld; }
            }
          }
          bool march = false;
          if (vi >= 0) {
            const DVolume &V = S.volumes[vi];
            const float3 Sv = ld3(V.S);
            o = Sv * (vlo + ld3(V.T));
            d = Sv * vld;
            t = vT;
            t1 = fminf(ray.tmax, vFar);
            dt = V.cellSize * R.samplingRateInv;
            expo = dt / V.unitDistance;
            vIdx = vi;
            march = t <= t1;
          }
          Cr = Cg = Cb = A = 0.f;
          T = 1.f;
          steps = 0;
          if (march) active = true;
          else writeSample(F, x, y, false, bg, 1e31f, f3(0.f), f3(0.f));
        }
      }
    }
    if (!__any_sync(kFull, active)) break;
    // rayMarchVolume<0>'s loop (VolumeIntegration.h:410-466), a few samples:
    // the field values first (their fetches overlap), then the compositing
    // in order with the loop's test before every sample
    if (active) {
      const DVolume &V = S.volumes[vIdx];
      const float4 *tf = (stageTF && vIdx == 0) ? sTF : V.tf;
      if (!(dt > 0.f) || steps > kMaxMarchSteps) {
        err |= ERR_MARCH_LIMIT;
        finish();
      } else {
        float val[VSR_REFILL_SAMPLES];
        float tk = t;
        int n = 0;
#pragma unroll
        for (int k = 0; k < VSR_REFILL_SAMPLES; ++k) {
          if (tk <= t1) {
            val[k] = fieldAt(V, o + d * tk, hw);
            n = k + 1;
          }
          tk += dt;
        }
        bool done = n < VSR_REFILL_SAMPLES;
#pragma unroll
        for (int k = 0; k < VSR_REFILL_SAMPLES; ++k) {
          if (k >= n) break;
          if (!(A < 0.99f)) {
            done = true;
            break;
          }
          const float4 sm = classify(V, tf, val[k], hw);
          const float stepTr = hw ? __powf(1.f - sm.w, expo) : powf(1.f - sm.w, expo);
          const float w = T * (1.f - stepTr);
          Cr += w * sm.x; Cg += w * sm.y; Cb += w * sm.z;
          A += w;
          T *= stepTr;
          t += dt;
          ++steps;
          if (Count) ++samples;
        }
        if (done || !(t <= t1 && A < 0.99f)) finish();
      }
    }
  }
  if (Count) {
    for (int off = 16; off > 0; off >>= 1) samples += __shfl_xor_sync(kFull, samples, off);
    if (lane == 0 && samples) atomicAdd(&F.counters[3], samples);
  }
  if (err) atomicOr(F.errorFlags, err);
}

// Pass 3: one warp per group.
template <bool Count>
__global__ void __launch_bounds__(256) kVolumeCombine(DScene S, DRenderer R, DFrame F,
                                                      MarchScratch M, int stageTF) {
  extern __shared__ float4 sTF[];
  stageTable(S, sTF, stageTF);
  // the segment composites are complete and visible
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  const int lane = threadIdx.x & 31;
  const unsigned numGroups = M.counters[3];
  const unsigned warps = gridDim.x * (blockDim.x >> 5);
  uint32_t err = 0;
  unsigned long long samples = 0;
  for (unsigned g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g < numGroups;
       g += warps)
    combineGroup<Count>(S, R, F, M, sTF, stageTF, (int)g, lane, err, samples);
  if (Count) {
    for (int o = 16; o > 0; o >>= 1) samples += __shfl_xor_sync(kFull, samples, o);
    if (lane == 0 && samples) atomicAdd(&F.counters[3], samples);
  }
  if (err) atomicOr(F.errorFlags, err);
}

}  // namespace

namespace {

// resident blocks per SM of a persistent kernel at 256 threads, queried once
// per (kernel, dynamic shared memory) and kept, so that a frame's launches
// follow each other without host-side queries in between
int persistentBlocksPerSM(const void *fn, size_t smem) {
  struct Entry {
    const void *fn;
    size_t smem;
    int perSM;
  };
  static Entry cache[16];
  static int count = 0;
  static std::mutex mtx;
  std::lock_guard<std::mutex> lk(mtx);
  for (int i = 0; i < count; ++i)
    if (cache[i].fn == fn && cache[i].smem == smem) return cache[i].perSM;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int perSM = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fn, 256, smem);
  perSM = perSM > 0 ? perSM : 1;
  if (count < 16) cache[count++] = Entry{fn, smem, perSM};
  return perSM;
}

}  // namespace

cudaError_t launchVolumeMarch(const DScene &S, const DCamera &C, const DRenderer &R,
                              const DFrame &F, int stageTFSize, bool count,
                              const MarchScratch &M, cudaStream_t stream) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const size_t smem = stageTFSize > 0 ? sizeof(float4) * (size_t)stageTFSize : 0;
  const int stage = stageTFSize > 0;
  const int numPix = F.width * F.height;
  kMarchReset<<<1, 32, 0, stream>>>(M.counters);
  if (VSR_VOLUME_REFILL) {
    const void *fn = count ? (const void *)kVolumeRefill<true> : (const void *)kVolumeRefill<false>;
    const int perSM = persistentBlocksPerSM(fn, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sms * perSM);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (count) cudaLaunchKernelEx(&cfg, kVolumeRefill<true>, S, C, R, F, M, stage);
    else cudaLaunchKernelEx(&cfg, kVolumeRefill<false>, S, C, R, F, M, stage);
    return cudaGetLastError();
  }
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(min((numPix + 255) / 256, sms * 8));
    cfg.blockDim = dim3(256);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kVolumeSetup, S, C, R, F, M);
  }
  // programmatic dependent launch: a pass's blocks start (and stage the
  // transfer function) while the previous pass drains, and wait for its
  // results with griddepcontrol.wait
  auto persistent = [&](auto kernel, auto... args) {
    const int perSM = persistentBlocksPerSM((const void *)kernel, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sms * perSM);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
  };
  if (count) {
    // the counting frame: segments, then combination as its own pass
    persistent(kVolumeSegments<false>, S, R, F, M, stage);
    persistent(kVolumeCombine<true>, S, R, F, M, stage);
  } else if (VSR_SEG_FUSE) {
    persistent(kVolumeSegments<true>, S, R, F, M, stage);
  } else {
    persistent(kVolumeSegments<false>, S, R, F, M, stage);
    persistent(kVolumeCombine<false>, S, R, F, M, stage);
  }
  return cudaGetLastError();
}

}  // namespace vsr
