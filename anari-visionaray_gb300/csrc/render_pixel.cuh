// Per-pixel bodies of the raycast and pathtrace renderers, shared by the
// per-frame kernels (k_render.cu) and the batched kernel (k_batch.cu).
//
// Both keep one thread per pixel and the reference's per-pixel random
// stream (renderer/Pathtrace_impl.cpp:512-513), so the GPU image tracks the
// CPU restatement sample for sample; the frame write (G-buffer,
// accumulation, colour conversion) is fused into the end of each body.
#pragma once

#include "render_common.cuh"

namespace vsr {

// ------------------------------------------------------------------ raycast
// renderSample, renderer/Raycast_impl.cpp:10-243 (default render mode).
// Full = true is the variant with the optional features (gradient shading,
// with its six extra field samples per step; point and spot lights), kept
// out of the plain kernels' register allocation.
template <bool Count, bool Surfaces, bool Full>
__device__ void raycastSample(const DScene &S, const DRenderer &R, Ray ray, const float4 *sTF,
                              float4 &outColor, float &outDepth, float3 &outNg, float3 &outAlbedo,
                              uint32_t &err, unsigned long long *cnt) {
  const float4 bg = make_float4(R.bg[0], R.bg[1], R.bg[2], R.bg[3]);
  outColor = bg;
  outDepth = 1e31f;
  outNg = f3(0.f);
  outAlbedo = f3(0.f);
  if (S.numInstances == 0) return;
  float3 surfaceColor = f3(0.f);
  float surfaceAlpha = 0.f;
  if (Surfaces && S.hasSurfaces) {
    Hit hr;
    bool hit = traceSurfaces<Count, Full>(S, ray, false, hr, err, cnt);
    bool first = true;
    int layers = 0;
    while (hit) {
      if (++layers > kMaxSurfaceLayers) {
        err |= ERR_LAYER_LIMIT;
        break;
      }
      const DInstance &I = S.instances[hr.inst];
      const DGroup &G = S.groups[I.group];
      const uint32_t sid = hitSurface<Full>(G, hr);
      const DMaterial *matP = &S.materials[sid];
      const float3 hitPos = ray.o + hr.t * ray.d;
      // getNormals (renderer/common.h:241-275)
      float3 gn = hitNormal<Full>(G, I, hr, ray.o, ray.d);
      float3 sn = gn;
      DMaterial matR;
      if (Full && S.attributes) {
        // shading normal and attributes (Raycast_impl.cpp:45-60): the
        // "worldNormal" attribute is the object-space normal and the
        // "objectNormal" one the transformed normal, as the reference
        // passes them
        AttrCtx ac = hitAttrCtx(S, G, hr, sid);
        if (ac.sa) sn = shadingNormal(*ac.sa, ac.primID, hr.u, hr.v, gn);
        float3 lo, ld;
        localRay(I, ray.o, ray.d, lo, ld);
        ac.worldPos = hitPos;
        ac.worldNormal = gn;
        ac.objectPos = lo + hr.t * ld;
        gn = normalize(mat3mul(I.normalXfm, gn));
        sn = normalize(mat3mul(I.normalXfm, sn));
        ac.objectNormal = gn;
        matR = resolveMaterial(S, *matP, ac);
        matP = &matR;
      } else {
        gn = normalize(mat3mul(I.normalXfm, gn));
        sn = normalize(mat3mul(I.normalXfm, sn));
      }
      const DMaterial &mat = *matP;
      const float3 color = materialColor(mat);
      float3 shaded = f3(0.f);
      const float3 viewDir = -ray.d;
      for (int li = 0; li < S.numLights; ++li) {
        Rng dummy;
        dummy.state = 0;
        LightSample ls = sampleLight<Full>(S.lights[li], hitPos, dummy);
        const float3 lightDir = normalize(ls.dir);
        const float3 li3 = ls.intensity * safeRcp(ls.dist2);
        const float NdotL = fmaxf(0.f, dot(sn, lightDir));
        const float3 bsdf = evalMaterial(mat, sn, normalize(viewDir), lightDir);
        shaded += bsdf * li3 * NdotL * safeRcp(ls.pdf);
      }
      shaded += color * ld3(R.ambient);
      const float a = materialOpacity(mat);
      surfaceColor += (1.f - surfaceAlpha) * a * shaded;
      surfaceAlpha += (1.f - surfaceAlpha) * a;
      if (first) {
        outDepth = hr.t;
        outNg = gn;
        outAlbedo = color;
        first = false;
      }
      if (surfaceAlpha < 0.999f) {
        const float eps = epsilonFrom(hitPos, ray.d, hr.t);
        ray.tmin = hr.t + eps;
        hit = traceSurfaces<Count, Full>(S, ray, false, hr, err, cnt);
      } else {
        ray.tmax = hr.t;
        break;
      }
    }
  }
  // behind the surfaces: a quad or HDRI light the ray meets (its intensity
  // along the ray, alpha 1), else the background (Raycast_impl.cpp:158-172)
  float4 back = bg;
  if (Full && S.areaLights) {
    float tl;
    const int li = intersectLights(S, ray.o, ray.d, ray.tmin, ray.tmax, 0, tl);
    if (li >= 0) {
      const DLight &L = S.lights[li];
      const float3 I = L.type == LIGHT_HDRI ? hdriIntensity(L, ray.d) : ld3(L.intensity);
      back = make_float4(I.x, I.y, I.z, 1.f);
    }
  }
  float4 result = make_float4(surfaceColor.x + (1.f - surfaceAlpha) * back.x,
                              surfaceColor.y + (1.f - surfaceAlpha) * back.y,
                              surfaceColor.z + (1.f - surfaceAlpha) * back.z,
                              surfaceAlpha + (1.f - surfaceAlpha) * back.w);
  // intersectVolumeBounds: closest volume box entry.
  int vInst = -1, vIdx = -1;
  float vT = FLT_MAX;
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
      if (h && t < vT) { vT = t; vInst = i; vIdx = vi; }
    }
  }
  if (vIdx >= 0) {
    const DVolume &V = S.volumes[vIdx];
    float3 lo, ld;
    localRay(S.instances[vInst], ray.o, ray.d, lo, ld);
    // rayMarchVolume<0>, renderer/VolumeIntegration.h:374-468
    BoxHit bh = intersectBox(lo, ld, V.boundsLo, V.boundsHi);
    const float tmin = fmaxf(ray.tmin, bh.tnear);
    const float tmax = fminf(ray.tmax, bh.tfar);
    const float3 Sv = ld3(V.S);
    const float3 o = Sv * (lo + ld3(V.T));
    const float3 d = Sv * ld;
    const float dt = V.cellSize * R.samplingRateInv;
    const float expo = dt / V.unitDistance;
    const float4 *tf = (sTF && vIdx == 0) ? sTF : V.tf;
    float3 color = f3(0.f);
    float alpha = 0.f, transmittance = 1.f;
    unsigned samples = 0;
    const bool hw = R.hwFilter != 0;
    // for (t = tmin; t <= tmax && alpha < 0.99; t += dt) { composite sample(t) },
    // with the field fetches of four consecutive steps issued before they are
    // composited: the positions do not depend on the values, so four
    // fetches are in flight per thread. Same t sequence, same early exit.
    float t = tmin;
    constexpr int kBatch = VSR_MARCH_BATCH;
    int steps = 0;
    while (t <= tmax && alpha < 0.99f) {
      // dt <= 0, or dt below the float spacing of t, would never end
      if (!(dt > 0.f) || (steps += kBatch) > kMaxMarchSteps) {
        err |= ERR_MARCH_LIMIT;
        break;
      }
      float tk[kBatch], vk[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; ++k) {
        tk[k] = t;
        vk[k] = t <= tmax ? fieldAt(V, o + d * t, hw) : 0.f;
        t += dt;
      }
#pragma unroll
      for (int k = 0; k < kBatch; ++k) {
        if (tk[k] <= tmax && alpha < 0.99f) {
          const float4 s = classify(V, tf, vk[k], hw);
          // the texture path is already approximate (fixed-point filter
          // weights): use the fast pow there, the exact one otherwise
          const float stepTr = hw ? __powf(1.f - s.w, expo) : powf(1.f - s.w, expo);
          const float w = transmittance * (1.f - stepTr);
          float3 rgb = f3(s.x, s.y, s.z);
          if (Full && R.gradientShading)
            rgb = gradientShade(S, R, V, o + d * tk[k], Sv * V.cellSize, -d, rgb, hw);
          color += w * rgb;
          alpha += w;
          transmittance *= stepTr;
          if (Count) ++samples;
        }
      }
    }
    if (Count) atomicAdd(&cnt[3], (unsigned long long)samples);
    result = make_float4(alpha * color.x + (1.f - alpha) * result.x,
                         alpha * color.y + (1.f - alpha) * result.y,
                         alpha * color.z + (1.f - alpha) * result.z,
                         alpha + (1.f - alpha) * result.w);
    outNg = f3(0.f);
    outAlbedo = f3(0.f);
  }
  outColor = result;
}

// One pixel of the raycast renderer: pixelSamples camera rays through the
// pixel centre, averaged (renderer/Raycast_impl.cpp:282-322). sTF is the
// first volume's TF staged in shared memory, or null.
template <bool Count, bool Surfaces, bool Full = false>
__device__ __forceinline__ void raycastPixel(const DScene &S, const DCamera &C, const DRenderer &R,
                                             const DFrame &F, int x, int y, const float4 *sTF) {
  uint32_t err = 0;
  unsigned long long *cnt = F.counters;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 c0;
  float d0 = 1e31f;
  float3 n0 = f3(0.f), a0 = f3(0.f);
  Rng none;
  none.state = 0;
  for (int s = 0; s < R.pixelSamples; ++s) {
    Ray ray = primaryRay<false>(C, none, (float)x, (float)y, (float)F.width, (float)F.height);
    clipRay(ray, R);
    float4 c;
    float dd;
    float3 nn, aa;
    raycastSample<Count, Surfaces, Full>(S, R, ray, sTF, c, dd, nn, aa, err, cnt);
    acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
    if (s == 0) { c0 = c; d0 = dd; n0 = nn; a0 = aa; }
  }
  (void)c0;
  const float inv = 1.f / R.pixelSamples;
  writeSample(F, x, y, false, make_float4(acc.x * inv, acc.y * inv, acc.z * inv, acc.w * inv), d0,
              n0, a0);
  if (err) atomicOr(F.errorFlags, err);
}

// --------------------------------------------------------------- pathtrace
enum RayType { RT_RADIANCE = 0, RT_SHADOW = 1, RT_AO = 2, RT_MISS = 3 };

struct HitRec {
  bool surfHit, volHit, hit, volumeHit;
  bool lightHit;  // a quad light is the nearest hit (Full variants)
  Hit surf;
  float volT;
  float3 volAlbedo;
  int volInst;
  int volIdx;  // the volume hit
  int lightID;
  float lightT;
};

// intersectAll, renderer/common.h:1605-1620, with intersectSurfaces<1>
// (:1502-1543: one draw per surface hit) and the volume free-flight
// sampling of every volume in the world.
template <bool Count, bool Full>
__device__ __forceinline__ void intersectAll(const DScene &S, const Ray &ray, bool shadow, Rng &rnd,
                                             HitRec &h, uint32_t &err, unsigned long long *cnt,
                                             bool hwFilter, unsigned bounceID = 0) {
  h.surfHit = false;
  h.lightHit = false;
  h.lightID = -1;
  h.lightT = FLT_MAX;
  long long tc0 = 0;
  if (Count) tc0 = clock64();
  if (S.hasSurfaces) {
    Ray r = ray;
    const bool anyHit = shadow && S.allOpaque;
    bool hit = traceSurfaces<Count, Full>(S, r, anyHit, h.surf, err, cnt);
    int guard = 1 << 16;
    while (hit) {
      const DGroup &G = S.groups[S.instances[h.surf.inst].group];
      const uint32_t sid = hitSurface<Full>(G, h.surf);
      // intersectSurfaces<EvalOpacity> (renderer/common.h:1502-1543): the
      // attributes at the hit, hit attributes zero
      const float opacity =
          Full && S.attributes
              ? materialOpacity(resolveMaterial(S, S.materials[sid], hitAttrCtx(S, G, h.surf, sid)))
              : materialOpacity(S.materials[sid]);
      const float u = rnd();
      if (u > opacity && --guard > 0) {
        const float3 hp = r.o + h.surf.t * r.d;
        r.tmin = h.surf.t + epsilonFrom(hp, r.d, h.surf.t);
        hit = traceSurfaces<Count, Full>(S, r, false, h.surf, err, cnt);
      } else {
        break;
      }
    }
    h.surfHit = hit;
  } else {
    h.surf.t = FLT_MAX;
  }
  if (Count) {
    const long long tc1 = clock64();
    atomicAdd(&cnt[25], (unsigned long long)(tc1 - tc0));
    tc0 = tc1;
  }
  h.volHit = false;
  h.volT = FLT_MAX;
  if (S.numVolumes > 0) {
    for (int i = 0; i < S.numInstances; ++i) {
      const DInstance &I = S.instances[i];
      const DGroup &G = S.groups[I.group];
      for (int k = G.volBegin; k < G.volEnd; ++k) {
        float3 lo, ld;
        localRay(I, ray.o, ray.d, lo, ld);
        float t;
        float3 alb;
        if (deltaTrack<Count>(S.volumes[S.groupVolumes[k]], lo, ld, ray.tmin, ray.tmax, rnd, t, alb,
                              err, cnt, hwFilter) &&
            t < h.volT) {
          h.volHit = true;
          h.volT = t;
          h.volAlbedo = alb;
          h.volInst = i;
          h.volIdx = S.groupVolumes[k];
        }
      }
    }
  }
  if (Count && S.numVolumes > 0) atomicAdd(&cnt[26], (unsigned long long)(clock64() - tc0));
  bool lh = false;
  if (Full && S.areaLights) {
    h.lightID = intersectLights(S, ray.o, ray.d, ray.tmin, ray.tmax, bounceID, h.lightT);
    lh = h.lightID >= 0;
  }
  // renderer/common.h:1605-1620: a light hit takes precedence over surface
  // and volume hits at equal distance (<=), a volume over a surface only
  // when nearer
  h.hit = h.surfHit || h.volHit || lh;
  h.lightHit = lh && (!h.surfHit || h.lightT <= h.surf.t) && (!h.volHit || h.lightT <= h.volT);
  h.volumeHit = h.volHit && (!h.surfHit || h.volT < h.surf.t) && (!lh || h.volT < h.lightT);
}

// Per-pixel body of VisionarayRendererPathtrace::renderFrame
// (renderer/Pathtrace_impl.cpp:498-640) with shade() (:93-487) inlined.
// Full = true is the variant with gradient shading of volume hits and point
// and spot lights (kept out of the plain kernels' register allocation).
// chunk >= 0: sample chunk `chunk` of R.sampleChunks: R.pixelSamples /
// R.sampleChunks samples seeded as accumulation ID sampleChunks * accumID +
// chunk, written to F.chunkOut for kCombineChunks instead of the frame.
template <bool Count, bool Full>
__device__ __forceinline__ void pathtracePixel(const DScene &S, const DCamera &C,
                                               const DRenderer &R, const DFrame &F, int x, int y,
                                               int chunk = -1) {
  uint32_t err = 0;
  unsigned long long *cnt = F.counters;
  long long tStart = 0;
  if (Count) tStart = clock64();
  const int W = F.width, H = F.height;
  const int spp = chunk >= 0 ? R.pixelSamples / R.sampleChunks : R.pixelSamples;
  const uint32_t seedFrame =
      chunk >= 0 ? (uint32_t)F.accumID * (uint32_t)R.sampleChunks + (uint32_t)chunk
                 : (uint32_t)F.accumID;
  Rng rng;
  rng.init((uint32_t)(x + W * y), seedFrame);
  Rng rnd = rng;
  const float3 ambient = ld3(R.ambient);
  float4 accum = make_float4(0.f, 0.f, 0.f, 0.f);
  float lumSq = 0.f;  // sum of squared sample luminances (variance channel)
  float cDepth = 1e31f;
  float3 cNg = f3(0.f), cAlb = f3(0.f);
  // TAA (Full variant): the motion vector of the closest sample; a sample's
  // is that of its path's last radiance hit, as the reference overwrites it
  // at every radiance hit (Pathtrace_impl.cpp:290-297)
  float2 cMV = make_float2(0.f, 0.f);
  const bool taa = Full && R.taa && chunk < 0;
  const int maxPasses = (R.maxBounce + 2) * (2 + R.ambientSamples) + 8;
  for (int sampleID = 0; sampleID < spp; ++sampleID) {
    float2 pMV = make_float2(0.f, 0.f);
    bool closestNow = false;
    float xf = (float)x, yf = (float)y;
    const float jx = rnd() - .5f;
    const float jy = rnd() - .5f;
    xf += jx;
    yf += jy;
    Ray ray = primaryRay<true>(C, rnd, xf, yf, (float)W, (float)H);
    float4 pc = make_float4(R.bg[0], R.bg[1], R.bg[2], R.bg[3]);
    if (S.numInstances > 0) {
      bool firstHit = false;
      int rayType = RT_RADIANCE;
      float3 throughput = f3(1.f), intensity = f3(0.f);
      // ShadeState
      float3 baseColor = f3(0.f), shadedColor = f3(0.f), hitPosOff = f3(0.f), sn = f3(0.f);
      int aoSamples = 0;
      float aoWeights = 0.f, aoCount = 0.f;
      BSDFSample bsdf;
      bsdf.dir = f3(0.f); bsdf.f = f3(0.f); bsdf.pdf = 0.f; bsdf.cosT = 0.f;
      float misWeightNEE = 0.f, visLight = 1.f, visAO = 1.f;
      unsigned bounceID = 0;
      for (int passID = 0; true; ++passID) {
        if (passID >= maxPasses) { err |= ERR_PATH_LIMIT; break; }
        clipRay(ray, R);
        // the pass's light sample (zero when the scene has no light): it is
        // used by this pass only, so it is not carried across the traversal
        LightSample ls;
        ls.intensity = f3(0.f); ls.dir = f3(0.f); ls.pdf = 0.f; ls.dist = 0.f; ls.dist2 = 0.f;
        HitRec hr;
        if (rayType == RT_SHADOW && S.numLights == 0) {
          // the shadow ray of a light-less scene has a NaN direction and
          // cannot hit anything: skip the traversal
          hr.surfHit = hr.volHit = hr.hit = hr.volumeHit = hr.lightHit = false;
        } else {
          // every ray type tests the quad lights (a radiance ray's emission,
          // an AO ray's occluder; a shadow ray's volume hit beyond the light
          // does not count)
          intersectAll<Count, Full>(S, ray, rayType == RT_SHADOW || rayType == RT_AO, rnd, hr, err,
                                    cnt, R.hwFilter != 0, bounceID);
        }
        int nextType = RT_MISS;
        bool lightHitNow = false;
        if (rayType == RT_RADIANCE) {
          baseColor = f3(0.f);
          visLight = 1.f;
          visAO = 1.f;
          aoSamples = 0;
          aoWeights = 0.f;
          aoCount = 0.f;
          if (!hr.hit) {
            shadedColor = f3(0.f);
          } else if (Full && hr.lightHit) {
            // a quad or HDRI light seen by the ray: its intensity, weighted
            // after a bounce by the BSDF sample's MIS weight against the
            // light's density for that direction, ends the path
            // (Pathtrace_impl.cpp:139-182)
            const DLight &L = S.lights[hr.lightID];
            const bool hdri = L.type == LIGHT_HDRI;
            shadedColor = hdri ? hdriIntensity(L, ray.d) : ld3(L.intensity);
            misWeightNEE = 1.f;
            if (bounceID > 0) {
              float lightPDF;
              if (hdri) {
                lightPDF = hdriHitPdf(L, ray.d);
              } else {
                const float3 hp = ray.o + hr.lightT * ray.d;
                const float ld = length(hp - ray.o);
                const float3 Ld = normalize(hp - ray.o);
                const float LdotNl = fabsf(dot(-Ld, ld3(L.normal)));
                const float solidAngle = (LdotNl * (L.area1 + L.area2)) / (ld * ld);
                lightPDF = 1.f / solidAngle;
              }
              shadedColor = shadedColor * powerHeuristic(bsdf.pdf, lightPDF / float(S.numLights));
            }
            lightHitNow = true;
          } else {
            const float3 viewDir = -normalize(ray.d);
            float3 hitPos, gn, color;
            float eps;
            const DMaterial *mat = nullptr;
            DMaterial matR;
            if (hr.volumeHit) {
              const DInstance &I = S.instances[hr.volInst];
              hitPos = ray.o + hr.volT * ray.d;
              eps = epsilonFrom(hitPos, ray.d, hr.volT);
              gn = f3(0.f);
              if (Full && R.gradientShading) {
                // the field gradient at the instance-local hit position in
                // voxel space (renderer/Pathtrace_impl.cpp:204-212)
                const DVolume &V = S.volumes[hr.volIdx];
                float3 lo, ld;
                localRay(I, ray.o, ray.d, lo, ld);
                const float3 Sv = ld3(V.S);
                gn = fieldGradient(V, Sv * (lo + hr.volT * ld + ld3(V.T)), Sv * V.cellSize,
                                   R.hwFilter != 0);
              }
              if (R.ambientSamples > 0 && length(gn) < 1e-3f) {
                const float u1 = rnd(), u2 = rnd();
                gn = uniformSampleSphere(u1, u2);
              }
              sn = mat3mul(I.normalXfm, gn);
              gn = mat3mul(I.normalXfm, gn);
              sn = faceforward(sn, viewDir, gn);
              gn = faceforward(gn, viewDir, gn);
              color = hr.volAlbedo;
            } else {
              const DInstance &I = S.instances[hr.surf.inst];
              const DGroup &G = S.groups[I.group];
              hitPos = ray.o + hr.surf.t * ray.d;
              eps = epsilonFrom(hitPos, ray.d, hr.surf.t);
              const uint32_t sid = hitSurface<Full>(G, hr.surf);
              mat = &S.materials[sid];
              gn = hitNormal<Full>(G, I, hr.surf, ray.o, ray.d);
              if (Full && S.attributes) {
                // shading normal, attributes and the material's looked-up
                // parameters (Pathtrace_impl.cpp:240-270)
                AttrCtx ac = hitAttrCtx(S, G, hr.surf, sid);
                sn = ac.sa ? shadingNormal(*ac.sa, ac.primID, hr.surf.u, hr.surf.v, gn) : gn;
                float3 lo, ld;
                localRay(I, ray.o, ray.d, lo, ld);
                ac.worldPos = hitPos;
                ac.worldNormal = gn;
                ac.objectPos = lo + hr.surf.t * ld;
                gn = normalize(mat3mul(I.normalXfm, gn));
                sn = normalize(mat3mul(I.normalXfm, sn));
                sn = faceforward(sn, viewDir, gn);
                gn = faceforward(gn, viewDir, gn);
                ac.objectNormal = gn;
                matR = resolveMaterial(S, *mat, ac);
                mat = &matR;
              } else {
                sn = normalize(mat3mul(I.normalXfm, gn));
                gn = sn;
                sn = faceforward(sn, viewDir, gn);
                gn = faceforward(gn, viewDir, gn);
              }
              color = materialColor(*mat);
            }
            if (bounceID == 0) {
              // the closest first hit over the pixel's samples feeds the
              // G-buffer (Pathtrace_impl.cpp:616-618), merged right here
              const float d0 = hr.volumeHit ? hr.volT : hr.surf.t;
              if (d0 < cDepth) {
                cDepth = d0;
                cNg = gn;
                cAlb = color;
                closestNow = true;
              }
            }
            hitPosOff = hitPos + sn * eps;
            if (taa) {
              const float2 a = projectWin(F.prevMVP, hitPos, (float)W, (float)H);
              const float2 b = projectWin(F.currMVP, hitPos, (float)W, (float)H);
              pMV = make_float2(a.x - b.x, a.y - b.y);
            }
            bool areaSample = false;
            if (S.numLights > 0) {
              int lightID = int(rnd() * S.numLights);
              if (lightID == S.numLights) lightID = 0;
              ls = sampleLight<Full>(S.lights[lightID], hitPos, rnd);
              areaSample = Full && (S.lights[lightID].type == LIGHT_QUAD ||
                                    S.lights[lightID].type == LIGHT_HDRI);
            }
            const float3 lightDir = normalize(ls.dir);
            const float3 lightIntensity = ls.intensity * safeRcp(ls.dist2);
            const float NdotL = fmaxf(0.f, dot(sn, lightDir));
            if (hr.volumeHit) {
              if (Full && R.gradientShading && length(gn) > 1e-10f)  // matte along the gradient
                shadedColor = hr.volAlbedo * kInvPi * lightIntensity * NdotL * safeRcp(ls.pdf) *
                              float(S.numLights);
              else
                shadedColor = hr.volAlbedo * lightIntensity * safeRcp(ls.pdf) * safeRcp(ls.dist2);
              const float u1 = rnd(), u2 = rnd();
              bsdf.dir = uniformSampleSphere(u1, u2);
              bsdf.f = hr.volAlbedo;
              bsdf.pdf = 1.f;
              bsdf.cosT = 1.f;
            } else {
              const float3 f = evalMaterial(*mat, sn, viewDir, lightDir);
              shadedColor = f * lightIntensity * NdotL * safeRcp(ls.pdf) * float(S.numLights);
              bsdf = sampleMaterial(*mat, gn, sn, viewDir, rnd);
            }
            // Pathtrace_impl.cpp:365-375: MIS weight of the light sample
            // against the BSDF sample for area lights, 1 for delta lights
            misWeightNEE = S.numLights > 0 ? 1.f : 0.f;
            if (areaSample) misWeightNEE = powerHeuristic(ls.pdf / float(S.numLights), bsdf.pdf);
            baseColor = color;
          }
        } else if (rayType == RT_SHADOW) {
          const int surfV = hr.surfHit ? 0 : 1;
          const int volV = hr.volumeHit ? 0 : 1;
          visLight = float(surfV * volV) * (hr.volHit ? 0.f : 1.f);
        } else {  // AO
          aoSamples++;
          const float weight = fmaxf(0.f, dot(ray.d, sn));
          aoWeights += weight;
          if (weight > 0.f && hr.hit) aoCount += weight;
        }
        // advance the state machine (prepareNextRay, :37-90)
        const bool radianceHit = rayType == RT_RADIANCE && hr.hit && !lightHitNow;
        bool wantShadow = radianceHit && ls.pdf >= 0.f;
        bool wantAO = false, wantBounce = false;
        if (radianceHit && !wantShadow) {
          wantAO = aoSamples < R.ambientSamples;
          wantBounce = !wantAO && bsdf.pdf >= 0.f;
        } else if (rayType == RT_SHADOW) {
          wantAO = aoSamples < R.ambientSamples;
          wantBounce = !wantAO && bsdf.pdf >= 0.f;
        } else if (rayType == RT_AO) {
          wantAO = aoSamples < R.ambientSamples;
          if (!wantAO) {
            float aoV = 0.f;
            if (aoWeights > 0.f) aoV = 1.f - (aoCount / aoWeights);
            visAO *= aoV;
            wantBounce = bsdf.pdf >= 0.f;
          }
        }
        if (wantShadow) {
          nextType = RT_SHADOW;
          ray.o = hitPosOff;
          ray.d = normalize(ls.dir);
          ray.tmin = 0.f;
          ray.tmax = ls.dist;
        } else if (wantAO) {
          float3 u, v, w = sn;
          orthonormalBasis(u, v, w);
          const float u1 = rnd(), u2 = rnd();
          const float3 sp = cosineSampleHemisphere(u1, u2);
          nextType = RT_AO;
          ray.o = hitPosOff;
          ray.d = normalize(sp.x * u + sp.y * v + sp.z * w);
          ray.tmin = 0.f;
          ray.tmax = R.occlusionDistance;
        } else if (wantBounce) {
          nextType = RT_RADIANCE;
          ray.o = hitPosOff;
          ray.d = normalize(bsdf.dir);
          ray.tmin = 0.f;
          ray.tmax = 1e31f;
        }
        if (passID == 0 && bounceID == 0) firstHit = hr.hit;
        rayType = nextType;
        if (rayType == RT_MISS || rayType == RT_RADIANCE) {
          const float3 direct = shadedColor * visLight;
          const float3 amb = baseColor * ambient * visAO;
          intensity += throughput * misWeightNEE * direct;
          intensity += throughput * amb;
          throughput *= bsdf.f * bsdf.cosT * safeRcp(bsdf.pdf);
          bounceID++;
        }
        if (rayType == RT_MISS || bounceID > (unsigned)R.maxBounce) break;
        if (bounceID > 1) {
          const float prob = maxe(throughput);
          if (rng() > prob) break;
          throughput /= prob;
        }
      }
      if (firstHit) pc = make_float4(intensity.x, intensity.y, intensity.z, 1.f);
    }
    if (!finiteSample(pc)) {
      pc = make_float4(0.f, 0.f, 0.f, 0.f);
      err |= ERR_NONFINITE;
    }
    accum.x += pc.x; accum.y += pc.y; accum.z += pc.z; accum.w += pc.w;
    const float lum = 0.3f * pc.x + 0.59f * pc.y + 0.11f * pc.z;
    lumSq += lum * lum;
    if (closestNow) cMV = pMV;
  }
  const float inv = 1.f / spp;
  if (Count) atomicAdd(&cnt[24], (unsigned long long)(clock64() - tStart));
  const float4 mean = make_float4(accum.x * inv, accum.y * inv, accum.z * inv, accum.w * inv);
  if (chunk >= 0) {
    const size_t np = (size_t)W * H, i = (size_t)chunk * np + (size_t)y * W + x;
    const size_t plane = (size_t)R.sampleChunks * np;
    F.chunkOut[i] = mean;
    F.chunkOut[plane + i] = make_float4(lumSq * inv, cDepth, cNg.x, cNg.y);
    F.chunkOut[2 * plane + i] = make_float4(cNg.z, cAlb.x, cAlb.y, cAlb.z);
  } else if (taa) {
    fillGBufferTaa(F, x, y, mean, cDepth, cNg, cAlb, cMV);
  } else {
    writeSample(F, x, y, true, mean, cDepth, cNg, cAlb, lumSq * inv);
  }
  if (err) atomicOr(F.errorFlags, err);
}

// The frame write of a chunked path-traced frame: per pixel, the chunks'
// results accumulated in chunk order as consecutive sub-frames
// (dco::Frame::writeSample for each, accumulation ID sampleChunks *
// accumID + c, pixelSamples / sampleChunks samples each), as the reference
// accumulates that many frames.
__device__ __forceinline__ void combineChunks(const DRenderer &R, const DFrame &F, int x, int y) {
  const int K = R.sampleChunks;
  const size_t np = (size_t)F.width * F.height, p = (size_t)y * F.width + x;
  const size_t plane = (size_t)K * np;
  DFrame Fc = F;
  Fc.pixelSamples = R.pixelSamples / K;
  for (int c = 0; c < K; ++c) {
    const float4 col = F.chunkOut[(size_t)c * np + p];
    const float4 a = F.chunkOut[plane + (size_t)c * np + p];
    const float4 b = F.chunkOut[2 * plane + (size_t)c * np + p];
    Fc.accumID = F.accumID * K + c;
    writeSample(Fc, x, y, true, col, a.y, f3(a.z, a.w, b.x), f3(b.y, b.z, b.w), a.x);
  }
}

// The TAA resolve pass of one pixel (frame/Frame.cpp:339-381 with
// dco::Frame::accumSample, DeviceCopyableObjects.h:2692-2720): the previous
// resolved image is read at the pixel moved by its motion vector with the
// history filter; the blend weight is taaAlpha, or 1 where the albedo at
// the reprojected pixel differs from this pixel's (by 1e-2 or more in a
// channel); the result replaces this frame's colour and is converted into
// the frame's colour channel.
__device__ __forceinline__ void taaResolvePixel(const DRenderer &R, const DFrame &F, int x, int y) {
  const int W = F.width, H = F.height;
  const size_t idx = (size_t)y * W + x;
  const float2 mv = F.motionVec[idx];
  int px = (int)((float)x + mv.x), py = (int)((float)y + mv.y);
  px = min(max(px, 0), W - 1);
  py = min(max(py, 0), H - 1);
  const size_t pidx = (size_t)py * W + px;
  float alpha = R.taaAlpha;
  const float *pa = F.taaPrevAlbedo + 3 * pidx, *ca = F.taaCurrAlbedo + 3 * idx;
  if (!(fabsf(pa[0] - ca[0]) < 1e-2f && fabsf(pa[1] - ca[1]) < 1e-2f &&
        fabsf(pa[2] - ca[2]) < 1e-2f))
    alpha = 1.f;
  const float u = ((float)x + mv.x + 0.5f) / (float)W, v = ((float)y + mv.y + 0.5f) / (float)H;
  const float4 h = historyAt(F.taaPrev, W, H, u, v);
  const float4 c = F.taaCurr[idx];
  const float4 o = make_float4((1.f - alpha) * h.x + alpha * c.x, (1.f - alpha) * h.y + alpha * c.y,
                               (1.f - alpha) * h.z + alpha * c.z, (1.f - alpha) * h.w + alpha * c.w);
  F.taaCurr[idx] = o;
  if (F.colorType == COLOR_FLOAT4)
    reinterpret_cast<float4 *>(F.color)[idx] = o;
  else if (F.colorType == COLOR_UFIXED8 || F.colorType == COLOR_SRGB8)
    reinterpret_cast<uint32_t *>(F.color)[idx] = packRGBA8(o, F.colorType == COLOR_SRGB8);
}

} // namespace vsr
