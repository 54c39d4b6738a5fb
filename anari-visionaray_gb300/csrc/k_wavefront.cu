// Wavefront path tracer: the per-pixel megakernel of the reference
// (renderer/Pathtrace_impl.cpp:498-640 with shade() :93-487) split into
//   kWaveInit  : per pixel, seed the LCG pair, start sample 0, enqueue;
//   kWaveTrace : BVH traversal of each queued pixel's current ray;
//   kWaveShade : stochastic opacity, delta tracking, the radiance / shadow /
//                AO state machine, Russian roulette, sample accumulation,
//                next-sample regeneration and the frame write; pixels that
//                still have work are appended to the next queue with one
//                atomic per warp (ballot + popc).
// Each pixel keeps the reference's single random stream across its samples,
// so the image is the same as the megakernel's sample for sample. The
// traversal kernel has no shading state and runs at high occupancy; the
// queue keeps every lane of a warp on a live ray.
#include "kernels.h"
#include "render_common.cuh"

namespace vsr {
namespace {

enum { RT_RADIANCE = 0, RT_SHADOW = 1, RT_AO = 2, RT_MISS = 3 };

// flags layout
__device__ __forceinline__ uint32_t fRayType(uint32_t f) { return f & 3u; }
__device__ __forceinline__ uint32_t fFirstHit(uint32_t f) { return (f >> 2) & 1u; }
__device__ __forceinline__ uint32_t fBounce(uint32_t f) { return (f >> 3) & 511u; }
__device__ __forceinline__ uint32_t fAO(uint32_t f) { return (f >> 12) & 511u; }
__device__ __forceinline__ uint32_t fSample(uint32_t f) { return (f >> 21) & 511u; }
__device__ __forceinline__ uint32_t fRetrace(uint32_t f) { return (f >> 30) & 1u; }
__device__ __forceinline__ uint32_t mkFlags(uint32_t rt, uint32_t first, uint32_t bounce, uint32_t ao,
                                            uint32_t sample, uint32_t retrace) {
  return rt | (first << 2) | (bounce << 3) | (ao << 12) | (sample << 21) | (retrace << 30);
}

struct Path {
  float3 o, d;
  float tmin, tmax;
  float3 thr, inten, base, shaded, hpo, sn, bdir, bf;
  float visLight, visAO, aoW, aoC, bpdf, bcos, tmin0, retraces;
  float4 acc;
  float3 pNg, pAlb, cNg, cAlb;
  float pDepth, cDepth;
  uint32_t rnd, rng, flags, pass;
};

__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 pack(float3 v, float w) { return make_float4(v.x, v.y, v.z, w); }

__device__ __forceinline__ void loadPath(const DWave &Wv, uint32_t p, Path &s) {
  float4 a = Wv.rayO[p], b = Wv.rayD[p];
  s.o = xyz(a); s.tmin = a.w; s.d = xyz(b); s.tmax = b.w;
  a = Wv.thr[p]; s.thr = xyz(a); s.visLight = a.w;
  a = Wv.inten[p]; s.inten = xyz(a); s.visAO = a.w;
  a = Wv.base[p]; s.base = xyz(a); s.aoW = a.w;
  a = Wv.shaded[p]; s.shaded = xyz(a); s.aoC = a.w;
  a = Wv.hpo[p]; s.hpo = xyz(a); s.bpdf = a.w;
  a = Wv.sn[p]; s.sn = xyz(a); s.bcos = a.w;
  a = Wv.bdir[p]; s.bdir = xyz(a); s.tmin0 = a.w;
  a = Wv.bf[p]; s.bf = xyz(a); s.retraces = a.w;
  s.acc = Wv.acc[p];
  a = Wv.pNg[p]; s.pNg = xyz(a); s.pDepth = a.w;
  a = Wv.pAlb[p]; s.pAlb = xyz(a); s.cDepth = a.w;
  s.cNg = xyz(Wv.cNg[p]);
  s.cAlb = xyz(Wv.cAlb[p]);
  uint4 m = Wv.meta[p];
  s.rnd = m.x; s.rng = m.y; s.flags = m.z; s.pass = m.w;
}

__device__ __forceinline__ void storePath(const DWave &Wv, uint32_t p, const Path &s) {
  Wv.rayO[p] = pack(s.o, s.tmin);
  Wv.rayD[p] = pack(s.d, s.tmax);
  Wv.thr[p] = pack(s.thr, s.visLight);
  Wv.inten[p] = pack(s.inten, s.visAO);
  Wv.base[p] = pack(s.base, s.aoW);
  Wv.shaded[p] = pack(s.shaded, s.aoC);
  Wv.hpo[p] = pack(s.hpo, s.bpdf);
  Wv.sn[p] = pack(s.sn, s.bcos);
  Wv.bdir[p] = pack(s.bdir, s.tmin0);
  Wv.bf[p] = pack(s.bf, s.retraces);
  Wv.acc[p] = s.acc;
  Wv.pNg[p] = pack(s.pNg, s.pDepth);
  Wv.pAlb[p] = pack(s.pAlb, s.cDepth);
  Wv.cNg[p] = pack(s.cNg, 0.f);
  Wv.cAlb[p] = pack(s.cAlb, 0.f);
  Wv.meta[p] = make_uint4(s.rnd, s.rng, s.flags, s.pass);
}

// Start sample `sample` of a pixel: jitter, primary ray (renderer/
// Pathtrace_impl.cpp:528-556) and a fresh ShadeState (:15-35).
__device__ __forceinline__ void startSample(const DCamera &C, const DRenderer &R, int x, int y,
                                            int W, int H, uint32_t sample, Path &s) {
  Rng rnd;
  rnd.state = s.rnd;
  float xf = (float)x, yf = (float)y;
  const float jx = rnd() - .5f;
  const float jy = rnd() - .5f;
  xf += jx;
  yf += jy;
  Ray r = primaryRay<true>(C, rnd, xf, yf, (float)W, (float)H);
  clipRay(r, R);
  s.rnd = rnd.state;
  s.o = r.o; s.d = r.d; s.tmin = r.tmin; s.tmax = r.tmax;
  s.thr = f3(1.f); s.inten = f3(0.f);
  s.base = f3(0.f); s.shaded = f3(0.f); s.hpo = f3(0.f); s.sn = f3(0.f);
  s.bdir = f3(0.f); s.bf = f3(0.f);
  s.visLight = 1.f; s.visAO = 1.f; s.aoW = 0.f; s.aoC = 0.f; s.bpdf = 0.f; s.bcos = 0.f;
  s.tmin0 = r.tmin; s.retraces = 0.f;
  s.pNg = f3(0.f); s.pAlb = f3(0.f); s.pDepth = 1e31f;
  s.flags = mkFlags(RT_RADIANCE, 0, 0, 0, sample, 0);
  s.pass = 0;
}

__device__ __forceinline__ void warpAppend(bool active, uint32_t p, uint32_t *queue,
                                           uint32_t *counter) {
  const int lane = threadIdx.x & 31;
  const unsigned mask = __ballot_sync(0xffffffffu, active);
  if (!mask) return;
  const int leader = __ffs(mask) - 1;
  uint32_t off = 0;
  if (lane == leader) off = atomicAdd(counter, (uint32_t)__popc(mask));
  off = __shfl_sync(0xffffffffu, off, leader);
  if (active) queue[off + __popc(mask & ((1u << lane) - 1u))] = p;
}

// A pixel that has finished all samples: dco::Frame::writeSample.
__device__ __forceinline__ void finishPixel(const DFrame &F, const DRenderer &R, int x, int y,
                                            const Path &s) {
  const float inv = 1.f / R.pixelSamples;
  writeSample(F, x, y, true,
              make_float4(s.acc.x * inv, s.acc.y * inv, s.acc.z * inv, s.acc.w * inv), s.cDepth,
              s.cNg, s.cAlb);
}

__global__ void __launch_bounds__(256) kWaveInit(DScene S, DCamera C, DRenderer R, DFrame F,
                                                 DWave Wv) {
  const uint32_t n = (uint32_t)F.width * F.height;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += stride) {
    const uint32_t p = base + (threadIdx.x & 31);
    bool active = false;
    if (p < n && (!F.sampleMask || F.sampleMask[p])) {
      const int x = (int)(p % F.width), y = (int)(p / F.width);
      Rng rng;
      rng.init(p, (uint32_t)F.accumID);
      Path s;
      s.rnd = rng.state;
      s.rng = rng.state;
      s.acc = make_float4(0.f, 0.f, 0.f, 0.f);
      s.cNg = f3(0.f); s.cAlb = f3(0.f); s.cDepth = 1e31f;
      if (S.numInstances == 0) {
        // empty world: every sample is the background (camera draws only)
        for (int k = 0; k < R.pixelSamples; ++k) {
          startSample(C, R, x, y, F.width, F.height, k, s);
          s.acc = make_float4(s.acc.x + R.bg[0], s.acc.y + R.bg[1], s.acc.z + R.bg[2],
                              s.acc.w + R.bg[3]);
        }
        finishPixel(F, R, x, y, s);
      } else {
        startSample(C, R, x, y, F.width, F.height, 0, s);
        storePath(Wv, p, s);
        active = true;
      }
    }
    warpAppend(active, p, Wv.queue[0], &Wv.count[0]);
  }
}

template <bool Count>
__global__ void __launch_bounds__(256, VSR_WAVE_TRACE_MIN_BLOCKS) kWaveTrace(
    DScene S, DWave Wv, int cur, uint32_t *errFlags, unsigned long long *cnt) {
  const uint32_t n = Wv.count[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) Wv.count[cur ^ 1] = 0;
  const uint32_t *q = Wv.queue[cur];
  uint32_t err = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t p = q[i];
    const float4 a = Wv.rayO[p], b = Wv.rayD[p];
    const uint32_t flags = Wv.meta[p].z;
    const uint32_t rt = fRayType(flags);
    Ray r;
    r.o = xyz(a); r.tmin = a.w; r.d = xyz(b); r.tmax = b.w;
    Hit h;
    bool hit = false;
    if (rt == RT_SHADOW && S.numLights == 0) {
      // the shadow ray of a light-less scene has no direction: a miss
      h.inst = -1;
    } else if (S.hasSurfaces) {
      const bool anyHit = (rt == RT_SHADOW || rt == RT_AO) && S.allOpaque && !fRetrace(flags);
      hit = traceSurfaces<Count>(S, r, anyHit, h, err, cnt);
    }
    Wv.hit[p] = hit ? make_int4(__float_as_int(h.t), h.inst, h.tri, h.leaf)
                    : make_int4(__float_as_int(FLT_MAX), -1, -1, -1);
  }
  if (err) atomicOr(errFlags, err);
}

// Persistent traversal with dynamic ray fetch (Aila and Laine's scheme):
// each lane traverses one queued ray over BVH2 groups, keeping its
// traversal state (node, stack, closest hit, instance) across iterations
// of the warp's loop; whenever kRefill or more lanes of the warp are idle,
// the warp takes that many new queue entries with one atomic, so lanes do
// not wait for the warp's longest ray. Hits follow the same closest-hit
// order (t, instance, triangle) and any-hit rule as traceSurfaces, so the
// hit records equal kWaveTrace's. Queue entries are handed out through a
// per-parity counter in Wv.count[2 + cur], zeroed by the previous trace
// launch (and by the frame's initial memset).
constexpr unsigned kFullMask = 0xffffffffu;
#ifndef VSR_WAVE_REFILL
#define VSR_WAVE_REFILL 8  // idle lanes of a warp that trigger a fetch of new rays
#endif
constexpr int kRefill = VSR_WAVE_REFILL;

template <bool Count>
__global__ void __launch_bounds__(128, VSR_WAVE_DYN_MIN_BLOCKS) kWaveTraceDyn(
    DScene S, DWave Wv, int cur, uint32_t *errFlags, unsigned long long *cnt) {
  const uint32_t n = Wv.count[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Wv.count[cur ^ 1] = 0;
    Wv.count[2 + (cur ^ 1)] = 0;
  }
  const uint32_t *q = Wv.queue[cur];
  uint32_t *fetch = &Wv.count[2 + cur];
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  uint32_t err = 0;
  bool active = false, exhausted = false;
  uint32_t p = 0;
  // the lane's ray in its current instance's object space
  float3 o = f3(0.f), d = f3(0.f), inv = f3(0.f), oi = f3(0.f);
  float tmin = 0.f;
  const float4 *nodes = nullptr, *tris = nullptr;
  Hit best;
  best.t = 0.f; best.u = best.v = 0.f; best.inst = best.tri = best.leaf = -1;
  int node = 0, sp = 0, inst = 0;
  bool anyHit = false, found = false, done = true;
  int stack[kTraversalStack];
  unsigned nodeVisits = 0, triTests = 0;

  // first instance at or after `inst` with triangles: transform the ray
  auto enterInstance = [&]() -> bool {
    while (inst < S.numInstances && S.groups[S.instances[inst].group].numNodes == 0) ++inst;
    if (inst >= S.numInstances) return false;
    const DInstance &I = S.instances[inst];
    const DGroup &G = S.groups[I.group];
    const float4 a = Wv.rayO[p], b = Wv.rayD[p];
    localRay(I, xyz(a), xyz(b), o, d);
    inv = f3(slabInv(d.x), slabInv(d.y), slabInv(d.z));
    oi = f3(-o.x * inv.x, -o.y * inv.y, -o.z * inv.z);
    nodes = G.nodes;
    tris = G.tris;
    node = 0;
    sp = 0;
    done = false;
    return true;
  };
  auto finish = [&]() {
    Wv.hit[p] = found ? make_int4(__float_as_int(best.t), best.inst, best.tri, best.leaf)
                      : make_int4(__float_as_int(FLT_MAX), -1, -1, -1);
    if (Count) {
      atomicAdd(&cnt[0], 1ull);
      atomicAdd(&cnt[1], (unsigned long long)nodeVisits);
      atomicAdd(&cnt[2], (unsigned long long)triTests);
      const int bin = nodeVisits ? min(31 - __clz(nodeVisits), 15) : 0;
      atomicAdd(&cnt[8 + bin], 1ull);
    }
    active = false;
  };

  while (true) {
    // ---- dynamic fetch
    const unsigned idle = __ballot_sync(kFullMask, !active);
    if (!exhausted && idle && (__popc(idle) >= kRefill || idle == kFullMask)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(idle));
      base = __shfl_sync(kFullMask, base, leader);
      if (base + (uint32_t)__popc(idle) >= n) exhausted = true;
      if (!active) {
        const uint32_t i = base + (uint32_t)__popc(idle & below);
        if (i < n) {
          p = q[i];
          const uint32_t flags = Wv.meta[p].z;
          const uint32_t rt = fRayType(flags);
          tmin = Wv.rayO[p].w;
          best.t = Wv.rayD[p].w;
          best.u = best.v = 0.f;
          best.inst = best.tri = best.leaf = -1;
          found = false;
          nodeVisits = triTests = 0;
          inst = 0;
          anyHit = (rt == RT_SHADOW || rt == RT_AO) && S.allOpaque && !fRetrace(flags);
          const bool skip = (rt == RT_SHADOW && S.numLights == 0) || !S.hasSurfaces;
          active = true;
          if (skip || !enterInstance()) finish();
        }
      }
    }
    if (!__any_sync(kFullMask, active)) {
      if (exhausted) break;
      continue;
    }
    if (!active) continue;
    // ---- one while-while step of the lane's traversal
    while (!done && node >= 0) {
      const float4 *N = nodes + 4 * (size_t)node;
      const float4 n0 = __ldg(N), n1 = __ldg(N + 1), n2 = __ldg(N + 2);
      const int4 n3 = __ldg(reinterpret_cast<const int4 *>(N + 3));
      if (Count) ++nodeVisits;
      const float tb = best.t;
      float a0 = fmaf(n0.x, inv.x, oi.x), b0 = fmaf(n0.y, inv.x, oi.x);
      float a1 = fmaf(n0.z, inv.y, oi.y), b1 = fmaf(n0.w, inv.y, oi.y);
      float a2 = fmaf(n2.x, inv.z, oi.z), b2 = fmaf(n2.y, inv.z, oi.z);
      const float c0min = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fmaxf(fminf(a2, b2), tmin));
      const float c0max = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fminf(fmaxf(a2, b2), tb));
      a0 = fmaf(n1.x, inv.x, oi.x); b0 = fmaf(n1.y, inv.x, oi.x);
      a1 = fmaf(n1.z, inv.y, oi.y); b1 = fmaf(n1.w, inv.y, oi.y);
      a2 = fmaf(n2.z, inv.z, oi.z); b2 = fmaf(n2.w, inv.z, oi.z);
      const float c1min = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fmaxf(fminf(a2, b2), tmin));
      const float c1max = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fminf(fmaxf(a2, b2), tb));
      const bool h0 = c0min <= c0max, h1 = c1min <= c1max;
      if (!h0 && !h1) {
        if (sp == 0) done = true;
        else node = stack[--sp];
      } else {
        int near = h0 ? n3.x : n3.y;
        if (h0 && h1) {
          int far = n3.y;
          if (c1min < c0min) { near = n3.y; far = n3.x; }
          if (sp < kTraversalStack) stack[sp++] = far;
          else err |= ERR_STACK_OVERFLOW;
        }
        node = near;
      }
    }
    while (!done && node < 0) {
      const uint32_t code = ~(uint32_t)node;
      const int first = (int)(code & kLeafFirstMask);
      const int count = (int)(code >> kLeafCountShift) + 1;
      for (int k = 0; k < count; ++k) {
        const float4 *T = tris + 3 * (size_t)(first + k);
        const float4 ta = __ldg(T), tbv = __ldg(T + 1), tc = __ldg(T + 2);
        if (Count) ++triTests;
        const float3 v1 = f3(ta.x, ta.y, ta.z), e1 = f3(tbv.x, tbv.y, tbv.z),
                     e2 = f3(tc.x, tc.y, tc.z);
        const float3 s1 = cross(d, e2);
        const float div = dot(s1, e1);
        if (div == 0.f) continue;
        const float idiv = 1.f / div;
        const float3 dd = o - v1;
        const float bb1 = dot(dd, s1) * idiv;
        if (bb1 < 0.f || bb1 > 1.f) continue;
        const float3 s2 = cross(dd, e1);
        const float bb2 = dot(d, s2) * idiv;
        if (bb2 < 0.f || bb1 + bb2 > 1.f) continue;
        const float t = dot(e2, s2) * idiv;
        if (!(t >= tmin)) continue;
        const int local = __float_as_int(ta.w);
        const bool closer =
            t < best.t || (t == best.t && best.inst >= 0 &&
                           (inst < best.inst || (inst == best.inst && local < best.tri)));
        if (!closer) continue;
        best.t = t; best.u = bb1; best.v = bb2; best.inst = inst; best.tri = local;
        best.leaf = first + k;
        found = true;
      }
      if ((anyHit && found) || sp == 0) done = true;
      else node = stack[--sp];
    }
    if (done) {
      // this instance is through: the next one, or the ray is finished
      ++inst;
      if ((anyHit && found) || !enterInstance()) finish();
    }
  }
  if (err) atomicOr(errFlags, err);
}

template <bool Count>
__global__ void __launch_bounds__(256, VSR_WAVE_SHADE_MIN_BLOCKS) kWaveShade(
    DScene S, DCamera C, DRenderer R, DFrame F, DWave Wv, int cur) {
  const uint32_t n = Wv.count[cur];
  const uint32_t *qin = Wv.queue[cur];
  uint32_t *qout = Wv.queue[cur ^ 1];
  uint32_t *cout = &Wv.count[cur ^ 1];
  unsigned long long *cnt = F.counters;
  const float3 ambient = ld3(R.ambient);
  const int maxPasses = (R.maxBounce + 2) * (2 + R.ambientSamples) + 8;
  uint32_t err = 0;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += stride) {
    const uint32_t i = base + (threadIdx.x & 31);
    bool active = false;
    uint32_t p = 0;
    if (i < n) {
      p = qin[i];
      active = true;
      Path s;
      loadPath(Wv, p, s);
      const int4 hv = Wv.hit[p];
      Rng rnd, rng;
      rnd.state = s.rnd;
      rng.state = s.rng;
      const int x = (int)(p % F.width), y = (int)(p / F.width);
      int rayType = (int)fRayType(s.flags);
      uint32_t firstHitF = fFirstHit(s.flags);
      uint32_t bounceID = fBounce(s.flags);
      uint32_t aoSamples = fAO(s.flags);
      uint32_t sampleID = fSample(s.flags);
      bool sampleDone = false;
      bool retraceNow = false;

      // ---- intersectAll: surfaces (with stochastic opacity), then volumes
      bool surfHit = hv.y >= 0;
      Hit hs;
      hs.t = __int_as_float(hv.x);
      hs.inst = hv.y;
      hs.tri = hv.z;
      hs.leaf = hv.w;
      if (surfHit) {
        const DGroup &G = S.groups[S.instances[hs.inst].group];
        const float opacity = materialOpacity(S.materials[__ldg(G.triSurface + hs.tri)]);
        const float u = rnd();
        if (u > opacity && s.retraces < 65535.f) {
          const float3 hp = s.o + hs.t * s.d;
          if (!fRetrace(s.flags)) s.tmin0 = s.tmin;
          s.tmin = hs.t + epsilonFrom(hp, s.d, hs.t);
          s.retraces += 1.f;
          retraceNow = true;
        }
      }
      if (retraceNow) {
        s.flags = mkFlags(rayType, firstHitF, bounceID, aoSamples, sampleID, 1);
      } else {
        if (fRetrace(s.flags)) s.tmin = s.tmin0;  // the pass's own ray for volumes/shading
        s.retraces = 0.f;
        Ray ray;
        ray.o = s.o; ray.d = s.d; ray.tmin = s.tmin; ray.tmax = s.tmax;
        bool volHit = false, hitAny, volumeHit;
        float volT = FLT_MAX;
        float3 volAlbedo = f3(0.f);
        int volInst = -1;
        const bool skip = rayType == RT_SHADOW && S.numLights == 0;
        if (skip) surfHit = false;
        if (S.numVolumes > 0 && !skip) {
          for (int ii = 0; ii < S.numInstances; ++ii) {
            const DInstance &I = S.instances[ii];
            const DGroup &G = S.groups[I.group];
            for (int k = G.volBegin; k < G.volEnd; ++k) {
              float3 lo, ld;
              localRay(I, ray.o, ray.d, lo, ld);
              float t;
              float3 alb;
              if (deltaTrack<Count>(S.volumes[S.groupVolumes[k]], lo, ld, ray.tmin, ray.tmax, rnd,
                                    t, alb, err, cnt, R.hwFilter != 0) &&
                  t < volT) {
                volHit = true;
                volT = t;
                volAlbedo = alb;
                volInst = ii;
              }
            }
          }
        }
        hitAny = surfHit || volHit;
        volumeHit = volHit && (!surfHit || volT < hs.t);

        // ---- shade(), renderer/Pathtrace_impl.cpp:93-487
        float3 lsDir = f3(0.f);
        float lsPdf = 0.f, lsDist = 0.f;
        if (rayType == RT_RADIANCE) {
          s.base = f3(0.f);
          s.visLight = 1.f;
          s.visAO = 1.f;
          aoSamples = 0;
          s.aoW = 0.f;
          s.aoC = 0.f;
          if (!hitAny) {
            s.shaded = f3(0.f);
          } else {
            const float3 viewDir = -normalize(ray.d);
            float3 hitPos, gn, color;
            float eps;
            const DMaterial *mat = nullptr;
            if (volumeHit) {
              const DInstance &I = S.instances[volInst];
              hitPos = ray.o + volT * ray.d;
              eps = epsilonFrom(hitPos, ray.d, volT);
              gn = f3(0.f);
              if (R.ambientSamples > 0) {
                const float u1 = rnd(), u2 = rnd();
                gn = uniformSampleSphere(u1, u2);
              }
              s.sn = mat3mul(I.normalXfm, gn);
              gn = mat3mul(I.normalXfm, gn);
              s.sn = faceforward(s.sn, viewDir, gn);
              gn = faceforward(gn, viewDir, gn);
              color = volAlbedo;
              if (bounceID == 0) s.pDepth = volT;
            } else {
              const DInstance &I = S.instances[hs.inst];
              const DGroup &G = S.groups[I.group];
              hitPos = ray.o + hs.t * ray.d;
              eps = epsilonFrom(hitPos, ray.d, hs.t);
              mat = &S.materials[__ldg(G.triSurface + hs.tri)];
              const float4 *E = G.tris + 3 * (size_t)hs.leaf;
              const float4 e1 = __ldg(E + 1), e2 = __ldg(E + 2);
              gn = normalize(cross(f3(e1.x, e1.y, e1.z), f3(e2.x, e2.y, e2.z)));
              s.sn = normalize(mat3mul(I.normalXfm, gn));
              gn = s.sn;
              s.sn = faceforward(s.sn, viewDir, gn);
              gn = faceforward(gn, viewDir, gn);
              color = materialColor(*mat);
              if (bounceID == 0) s.pDepth = hs.t;
            }
            if (bounceID == 0) {
              s.pNg = gn;
              s.pAlb = color;
            }
            s.hpo = hitPos + s.sn * eps;
            LightSample ls;
            ls.intensity = f3(0.f); ls.dir = f3(0.f); ls.pdf = 0.f; ls.dist = 0.f; ls.dist2 = 0.f;
            if (S.numLights > 0) {
              int lightID = int(rnd() * S.numLights);
              if (lightID == S.numLights) lightID = 0;
              ls = sampleLight<true>(S.lights[lightID], hitPos, rnd);
            }
            lsDir = ls.dir;
            lsPdf = ls.pdf;
            lsDist = ls.dist;
            const float3 lightDir = normalize(ls.dir);
            const float3 lightIntensity = ls.intensity * safeRcp(ls.dist2);
            const float NdotL = fmaxf(0.f, dot(s.sn, lightDir));
            if (volumeHit) {
              s.shaded = volAlbedo * lightIntensity * safeRcp(ls.pdf) * safeRcp(ls.dist2);
              const float u1 = rnd(), u2 = rnd();
              s.bdir = uniformSampleSphere(u1, u2);
              s.bf = volAlbedo;
              s.bpdf = 1.f;
              s.bcos = 1.f;
            } else {
              const float3 f = evalMaterial(*mat, s.sn, viewDir, lightDir);
              s.shaded = f * lightIntensity * NdotL * safeRcp(ls.pdf) * float(S.numLights);
              BSDFSample b = sampleMaterial(*mat, gn, s.sn, viewDir, rnd);
              s.bdir = b.dir;
              s.bf = b.f;
              s.bpdf = b.pdf;
              s.bcos = b.cosT;
            }
            s.base = color;
          }
        } else if (rayType == RT_SHADOW) {
          s.visLight = float((surfHit ? 0 : 1) * (volumeHit ? 0 : 1)) * (volHit ? 0.f : 1.f);
        } else {  // AO
          aoSamples++;
          const float weight = fmaxf(0.f, dot(ray.d, s.sn));
          s.aoW += weight;
          if (weight > 0.f && hitAny) s.aoC += weight;
        }
        // ---- advance the state machine (prepareNextRay, :37-90)
        const bool radianceHit = rayType == RT_RADIANCE && hitAny;
        const bool wantShadow = radianceHit && lsPdf >= 0.f;
        bool wantAO = false, wantBounce = false;
        if (radianceHit && !wantShadow) {
          wantAO = aoSamples < (uint32_t)R.ambientSamples;
          wantBounce = !wantAO && s.bpdf >= 0.f;
        } else if (rayType == RT_SHADOW) {
          wantAO = aoSamples < (uint32_t)R.ambientSamples;
          wantBounce = !wantAO && s.bpdf >= 0.f;
        } else if (rayType == RT_AO) {
          wantAO = aoSamples < (uint32_t)R.ambientSamples;
          if (!wantAO) {
            float aoV = 0.f;
            if (s.aoW > 0.f) aoV = 1.f - (s.aoC / s.aoW);
            s.visAO *= aoV;
            wantBounce = s.bpdf >= 0.f;
          }
        }
        int nextType = RT_MISS;
        if (wantShadow) {
          nextType = RT_SHADOW;
          s.o = s.hpo;
          s.d = normalize(lsDir);
          s.tmin = 0.f;
          s.tmax = lsDist;
        } else if (wantAO) {
          float3 u, v, w = s.sn;
          orthonormalBasis(u, v, w);
          const float u1 = rnd(), u2 = rnd();
          const float3 sp = cosineSampleHemisphere(u1, u2);
          nextType = RT_AO;
          s.o = s.hpo;
          s.d = normalize(sp.x * u + sp.y * v + sp.z * w);
          s.tmin = 0.f;
          s.tmax = R.occlusionDistance;
        } else if (wantBounce) {
          nextType = RT_RADIANCE;
          s.o = s.hpo;
          s.d = normalize(s.bdir);
          s.tmin = 0.f;
          s.tmax = 1e31f;
        }
        if (s.pass == 0 && bounceID == 0) firstHitF = hitAny ? 1u : 0u;
        rayType = nextType;
        if (rayType == RT_MISS || rayType == RT_RADIANCE) {
          const float3 direct = s.shaded * s.visLight;
          const float3 amb = s.base * ambient * s.visAO;
          const float mis = S.numLights > 0 ? 1.f : 0.f;
          s.inten += s.thr * mis * direct;
          s.inten += s.thr * amb;
          s.thr *= s.bf * s.bcos * safeRcp(s.bpdf);
          bounceID++;
        }
        s.pass++;
        if (rayType == RT_MISS || bounceID > (unsigned)R.maxBounce) {
          sampleDone = true;
        } else if (bounceID > 1) {
          const float prob = maxe(s.thr);
          if (rng() > prob) sampleDone = true;
          else s.thr /= prob;
        }
        if (!sampleDone && (int)s.pass >= maxPasses) {
          err |= ERR_PATH_LIMIT;
          sampleDone = true;
        }
        if (!sampleDone) {
          Ray nr;
          nr.o = s.o; nr.d = s.d; nr.tmin = s.tmin; nr.tmax = s.tmax;
          clipRay(nr, R);
          s.tmin = nr.tmin;
          s.tmax = nr.tmax;
          s.flags = mkFlags(rayType, firstHitF, bounceID, aoSamples, sampleID, 0);
        }
      }
      if (sampleDone) {
        // end of sample: accumulate, keep the closest G-buffer sample
        float4 pc = firstHitF ? make_float4(s.inten.x, s.inten.y, s.inten.z, 1.f)
                              : make_float4(R.bg[0], R.bg[1], R.bg[2], R.bg[3]);
        if (!finiteSample(pc)) {
          pc = make_float4(0.f, 0.f, 0.f, 0.f);
          err |= ERR_NONFINITE;
        }
        s.acc = make_float4(s.acc.x + pc.x, s.acc.y + pc.y, s.acc.z + pc.z, s.acc.w + pc.w);
        if (s.pDepth < s.cDepth) {
          s.cDepth = s.pDepth;
          s.cNg = s.pNg;
          s.cAlb = s.pAlb;
        }
        sampleID++;
        s.rnd = rnd.state;
        s.rng = rng.state;
        if ((int)sampleID < R.pixelSamples) {
          startSample(C, R, x, y, F.width, F.height, sampleID, s);
          rnd.state = s.rnd;
        } else {
          finishPixel(F, R, x, y, s);
          active = false;
        }
      }
      if (active) {
        s.rnd = rnd.state;
        s.rng = rng.state;
        storePath(Wv, p, s);
      }
    }
    warpAppend(active, p, qout, cout);
  }
  if (err) atomicOr(F.errorFlags, err);
}

int gridFor(const void *kernel, int block) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
  return sms * (per > 0 ? per : 1);
}

} // namespace

cudaError_t launchPathtraceWavefront(const DScene &S, const DCamera &C, const DRenderer &R,
                                     const DFrame &F, const DWave &Wv, uint32_t *pinnedCount,
                                     bool count, cudaStream_t stream, int *iterations) {
  const int B = 256;
  cudaError_t e = cudaMemsetAsync(Wv.count, 0, 4 * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  const int gInit = gridFor((const void *)kWaveInit, B);
  kWaveInit<<<gInit, B, 0, stream>>>(S, C, R, F, Wv);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const void *tk = count ? (const void *)kWaveTrace<true> : (const void *)kWaveTrace<false>;
  const void *sk = count ? (const void *)kWaveShade<true> : (const void *)kWaveShade<false>;
  const void *dk = count ? (const void *)kWaveTraceDyn<true> : (const void *)kWaveTraceDyn<false>;
  const int gTrace = gridFor(tk, B), gShade = gridFor(sk, B), gDyn = gridFor(dk, 128);
  // persistent dynamic-fetch traversal for worlds of 2-wide BVHs
  const bool dyn = S.maxGroupWidth == 2;
  int cur = 0, iters = 0;
  const int batch = 16;
  // every pixel finishes after at most spp * maxPasses iterations (plus
  // opacity retraces); the poll below ends the loop as soon as the queue
  // is empty
  const long long maxIters =
      (long long)R.pixelSamples * ((R.maxBounce + 2) * (2 + R.ambientSamples) + 8) * 4 + 64;
  while (iters < maxIters) {
    for (int b = 0; b < batch; ++b) {
      if (count) {
        if (dyn) kWaveTraceDyn<true><<<gDyn, 128, 0, stream>>>(S, Wv, cur, F.errorFlags, F.counters);
        else kWaveTrace<true><<<gTrace, B, 0, stream>>>(S, Wv, cur, F.errorFlags, F.counters);
        kWaveShade<true><<<gShade, B, 0, stream>>>(S, C, R, F, Wv, cur);
      } else {
        if (dyn) kWaveTraceDyn<false><<<gDyn, 128, 0, stream>>>(S, Wv, cur, F.errorFlags, F.counters);
        else kWaveTrace<false><<<gTrace, B, 0, stream>>>(S, Wv, cur, F.errorFlags, F.counters);
        kWaveShade<false><<<gShade, B, 0, stream>>>(S, C, R, F, Wv, cur);
      }
      cur ^= 1;
      ++iters;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(pinnedCount, &Wv.count[cur], sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             stream)) != cudaSuccess)
      return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    if (*pinnedCount == 0) break;
  }
  if (iterations) *iterations = iters;
  return cudaGetLastError();
}

} // namespace vsr
