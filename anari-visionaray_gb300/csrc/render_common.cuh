// Device functions of the per-pixel hot path: RNG, cameras, clip planes,
// BVH2 traversal, triangle test, materials, directional light, structured
// field sampling, transfer-function lookup, DDA, delta tracking and frame
// writes. Each function names the reference code whose behaviour it
// reproduces (file:line in anari-visionaray).
#pragma once

#include "vsr_device.h"
#include <float.h>
#include <stdint.h>

namespace vsr {

// ----------------------------------------------------------------- float3 ops
__device__ __forceinline__ float3 f3(float a) { return make_float3(a, a, a); }
__device__ __forceinline__ float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
__device__ __forceinline__ float3 ld3(const float *p) { return make_float3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ void operator+=(float3 &a, float3 b) { a = a + b; }
__device__ __forceinline__ void operator*=(float3 &a, float3 b) { a = a * b; }
__device__ __forceinline__ void operator/=(float3 &a, float s) { a = a / s; }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) { return a / length(a); }
__device__ __forceinline__ float3 fabs3(float3 a) { return f3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__device__ __forceinline__ float3 min3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ float3 max3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ float maxe(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ float mine(float3 a) { return fminf(a.x, fminf(a.y, a.z)); }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }
__device__ __forceinline__ float3 lerpR(float3 a, float3 b, float t) { return a * (1.f - t) + b * t; }
__device__ __forceinline__ float3 mat3mul(const float *m, float3 v) {
  return f3(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
            m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 6.28318530717958647692f;
constexpr float kInvPi = 0.31830988618379067154f;

// faceforward: n flipped into the hemisphere (around nref) that i lies in.
__device__ __forceinline__ float3 faceforward(float3 n, float3 i, float3 nref) {
  return dot(i, nref) < 0.f ? -n : n;
}
// reflect: mirror of i (pointing away from the surface) about n.
__device__ __forceinline__ float3 reflect(float3 i, float3 n) { return 2.f * dot(n, i) * n - i; }
// refract: i points away from the surface, eta = eta_t/eta_i; 0 on TIR.
__device__ __forceinline__ float3 refract(float3 i, float3 n, float eta) {
  float r = 1.f / eta;
  float cosi = dot(i, n);
  float k = 1.f - r * r * (1.f - cosi * cosi);
  if (k < 0.f) return f3(0.f);
  return -r * i + (r * cosi - sqrtf(k)) * n;
}
__device__ __forceinline__ float3 cosineSampleHemisphere(float u1, float u2) {
  float r = sqrtf(u1);
  float phi = kTwoPi * u2;
  float s, c;
  sincosf(phi, &s, &c);
  return f3(r * c, r * s, sqrtf(fmaxf(0.f, 1.f - u1)));
}
__device__ __forceinline__ float3 uniformSampleSphere(float u1, float u2) {
  float z = 1.f - 2.f * u1;
  float r = sqrtf(fmaxf(0.f, 1.f - z * z));
  float phi = kTwoPi * u2;
  float s, c;
  sincosf(phi, &s, &c);
  return f3(r * c, r * s, z);
}
__device__ __forceinline__ void orthonormalBasis(float3 &u, float3 &v, float3 w) {
  v = fabsf(w.x) > fabsf(w.y) ? normalize(f3(-w.z, 0.f, w.x)) : normalize(f3(0.f, w.z, -w.y));
  u = cross(v, w);
}
__device__ __forceinline__ float luminance(float3 c) { return 0.3f * c.x + 0.59f * c.y + 0.11f * c.z; }
__device__ __forceinline__ float safeRcp(float f) { return f > 0.f ? 1.f / f : 0.f; }

// epsilonFrom, renderer/common.h:14-18.
__device__ __forceinline__ float epsilonFrom(float3 P, float3 dir, float t) {
  float3 aP = fabs3(P);
  float m = fmaxf(fmaxf(aP.x, aP.y), fmaxf(aP.z, maxe(fabs3(dir)) * t));
  return m * 0x1.fp-18f;
}

// LCG<4>, common.h:55-102.
struct Rng {
  uint32_t state;
  __device__ __forceinline__ void init(uint32_t v0, uint32_t v1) {
    uint32_t s0 = 0;
#pragma unroll
    for (int n = 0; n < 4; n++) {
      s0 += 0x9e3779b9u;
      v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
      v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    state = v0;
  }
  __device__ __forceinline__ float operator()() {
    state = 1664525u * state + 1013904223u;
    return (state & 0x00FFFFFFu) / (float)0x01000000;
  }
};

struct Ray {
  float3 o, d;
  float tmin, tmax;
};

// ------------------------------------------------------------------ camera
// dco::Camera::primary_ray (DeviceCopyableObjects.h:2583-2600) for the
// thin-lens, matrix, orthographic and omnidirectional cameras. The thin
// lens draws two numbers (used only with a positive aperture) and every
// stochastic primary ray draws one more for ray.time.
template <bool Stochastic>
__device__ __forceinline__ Ray primaryRay(const DCamera &c, Rng &rng, float x, float y, float w,
                                          float h) {
  Ray r;
  r.tmin = 0.f;
  r.tmax = FLT_MAX;
  if (c.type == CAM_PERSPECTIVE) {
    float sx = (x + 0.5f) / w, sy = (y + 0.5f) / h;
    sx = (1.f - sx) * c.region[0] + sx * c.region[2];
    sy = (1.f - sy) * c.region[1] + sy * c.region[3];
    float u = 2.f * sx - 1.f, v = 2.f * sy - 1.f;
    float3 U = ld3(c.U), V = ld3(c.V), W = ld3(c.W);
    r.o = ld3(c.eye);
    r.d = normalize(U * u + V * v + W);
    if (Stochastic) {
      float l1 = rng(), l2 = rng();
      if (c.lensRadius > 0.f) {
        float3 focal = r.o + r.d * (c.focusDistance / dot(r.d, W));
        float a = 2.f * l1 - 1.f, b = 2.f * l2 - 1.f, rr, phi;
        if (a == 0.f && b == 0.f) { rr = 0.f; phi = 0.f; }
        else if (fabsf(a) > fabsf(b)) { rr = a; phi = (kPi / 4.f) * (b / a); }
        else { rr = b; phi = (kPi / 2.f) - (kPi / 4.f) * (a / b); }
        float dx = rr * cosf(phi) * c.lensRadius, dy = rr * sinf(phi) * c.lensRadius;
        r.o = ld3(c.eye) + normalize(U) * dx + normalize(V) * dy;
        r.d = normalize(focal - r.o);
      }
    }
  } else if (c.type == CAM_MATRIX) {
    float u = 2.f * (x + 0.5f) / w - 1.f, v = 2.f * (y + 0.5f) / h - 1.f;
    const float *m = c.inv;
    float4 p0, p1;
    p0.x = m[0] * u + m[4] * v + m[8] * -1.f + m[12];
    p0.y = m[1] * u + m[5] * v + m[9] * -1.f + m[13];
    p0.z = m[2] * u + m[6] * v + m[10] * -1.f + m[14];
    p0.w = m[3] * u + m[7] * v + m[11] * -1.f + m[15];
    p1.x = m[0] * u + m[4] * v + m[8] + m[12];
    p1.y = m[1] * u + m[5] * v + m[9] + m[13];
    p1.z = m[2] * u + m[6] * v + m[10] + m[14];
    p1.w = m[3] * u + m[7] * v + m[11] + m[15];
    float3 a = f3(p0.x / p0.w, p0.y / p0.w, p0.z / p0.w);
    float3 b = f3(p1.x / p1.w, p1.y / p1.w, p1.z / p1.w);
    r.o = a;
    r.d = normalize(b - a);
  } else if (c.type == CAM_ORTHO) {
    float sx = (x + 0.5f) / w, sy = (y + 0.5f) / h;
    sx = (1.f - sx) * c.region[0] + sx * c.region[2];
    sy = (1.f - sy) * c.region[1] + sy * c.region[3];
    r.o = ld3(c.U) * sx + ld3(c.V) * sy + ld3(c.W);
    r.d = normalize(ld3(c.dir));
  } else {  // omnidirectional
    float sx = (x + 0.5f) / w, sy = (y + 0.5f) / h;
    float theta = kPi * sy, phi = kTwoPi * sx;
    float3 ld = f3(sinf(theta) * cosf(phi), cosf(theta), sinf(theta) * sinf(phi));
    r.o = ld3(c.U) * sx + ld3(c.V) * sy + ld3(c.W);
    r.d = ld * f3(1.f, -1.f, 1.f);
  }
  if (Stochastic) (void)rng();  // ray.time = lerp(shutter, rng())
  return r;
}

// clipRay, renderer/common.h:1469-1482.
__device__ __forceinline__ void clipRay(Ray &r, const DRenderer &R) {
  for (int i = 0; i < R.numClipPlanes; ++i) {
    float3 N = f3(R.clip[i][0], R.clip[i][1], R.clip[i][2]);
    float D = R.clip[i][3];
    float s = dot(N, r.d);
    if (s != 0.f) {
      float t = (D - dot(N, r.o)) / s;
      if (s < 0.f) r.tmin = fmaxf(r.tmin, t);
      else r.tmax = fminf(r.tmax, t);
    }
  }
}

// ------------------------------------------------------------ traversal
struct Hit {
  float t, u, v;
  int inst;   // instance index, -1 = none
  int tri;    // local triangle id within the instance's group
  int leaf;   // position of the triangle in the group's leaf-ordered array
};

__device__ __forceinline__ void localRay(const DInstance &I, float3 o, float3 d, float3 &lo,
                                         float3 &ld) {
  lo = mat3mul(I.affineInv, o + ld3(I.transInv));
  ld = mat3mul(I.affineInv, d);
}

// Ray/sphere test in the form of Visionaray's basic_sphere intersection
// (used by the reference through intersect(ray, bls.asSphere),
// DeviceCopyableObjects.h:1486-1507): the two roots of
// |o + t d - c|^2 = r^2 from the cancellation-free quadratic formula, the
// smaller one returned (a ray starting inside the sphere reports the
// negative root and so misses it). Misses return -FLT_MAX.
__device__ __forceinline__ float sphereHitT(float3 o, float3 d, float4 sph) {
  const float3 oc = o - f3(sph.x, sph.y, sph.z);
  const float A = dot(d, d);
  const float B = 2.f * dot(d, oc);
  const float C = dot(oc, oc) - sph.w * sph.w;
  const float disc = B * B - 4.f * A * C;
  if (!(disc >= 0.f)) return -FLT_MAX;
  const float rd = sqrtf(disc);
  const float q = B < 0.f ? -0.5f * (B - rd) : -0.5f * (B + rd);
  const float t1 = q / A, t2 = C / q;
  return t1 > t2 ? t2 : t1;
}

// Capped cone from (v1, r1) to (v2, r2), intersect(Ray, Cone),
// DeviceCopyableObjects.h:933-1007 (after Quilez's cone intersector): the
// cap discs first (the one the origin lies behind), then the body as the
// smaller root of the quadratic; u = 0 / 1 on the caps and y / |v2-v1|^2 on
// the body, v = y (the unnormalised axis parameter the normal needs).
__device__ __forceinline__ float coneHitT(float3 ro, float3 rd, float4 A, float4 B, float &u,
                                          float &v) {
  const float3 pa = f3(A.x, A.y, A.z), pb = f3(B.x, B.y, B.z);
  const float ra = A.w, rb = B.w;
  const float3 ba = pb - pa, oa = ro - pa, ob = ro - pb;
  const float m0 = dot(ba, ba), m1 = dot(oa, ba), m2 = dot(rd, ba);
  const float m3 = dot(rd, oa), m5 = dot(oa, oa), m9 = dot(ob, ba);
  if (m1 < 0.f) {
    const float3 w = oa * m2 - rd * m1;
    if (dot(w, w) < ra * ra * m2 * m2) {
      u = 0.f;
      v = 0.f;
      return -m1 / m2;
    }
  } else if (m9 > 0.f) {
    const float t = -m9 / m2;
    const float3 w = ob + rd * t;
    if (dot(w, w) < rb * rb) {
      u = 1.f;
      v = 0.f;
      return t;
    }
  }
  const float rr = ra - rb;
  const float hy = m0 + rr * rr;
  const float k2 = m0 * m0 - m2 * m2 * hy;
  const float k1 = m0 * m0 * m3 - m1 * m2 * hy + m0 * ra * (rr * m2 * 1.f);
  const float k0 = m0 * m0 * m5 - m1 * m1 * hy + m0 * ra * (rr * m1 * 2.f - m0 * ra);
  const float h = k1 * k1 - k2 * k0;
  if (h < 0.f) return -FLT_MAX;
  const float t = (-k1 - sqrtf(h)) / k2;
  const float y = m1 + t * m2;
  if (y > 0.f && y < m0) {
    u = y / m0;
    v = y;
    return t;
  }
  return -FLT_MAX;
}

// Capped cylinder from v1 to v2 of radius r (Visionaray's basic_cylinder
// test is not part of the reference; this is Quilez's published capped-
// cylinder intersector): the body as the smaller root of the quadratic in
// the plane normal to the axis, else the cap plane the body root falls
// beyond, accepted inside the radius.
__device__ __forceinline__ float cylinderHitT(float3 ro, float3 rd, float4 A, float4 B) {
  const float3 pa = f3(A.x, A.y, A.z), pb = f3(B.x, B.y, B.z);
  const float ra = A.w;
  const float3 ba = pb - pa, oc = ro - pa;
  const float baba = dot(ba, ba), bard = dot(ba, rd), baoc = dot(ba, oc);
  const float k2 = baba - bard * bard;
  const float k1 = baba * dot(oc, rd) - baoc * bard;
  const float k0 = baba * dot(oc, oc) - baoc * baoc - ra * ra * baba;
  float h = k1 * k1 - k2 * k0;
  if (h < 0.f) return -FLT_MAX;
  h = sqrtf(h);
  float t = (-k1 - h) / k2;
  const float y = baoc + t * bard;
  if (y > 0.f && y < baba) return t;
  t = ((y < 0.f ? 0.f : baba) - baoc) / bard;
  if (fabsf(k1 + k2 * t) < h) return t;
  return -FLT_MAX;
}

// One analytic-primitive leaf: its hit parameter (-FLT_MAX on a miss) and
// the (u, v) the normal needs. For cones and cylinders the origin is first
// moved along the ray to twice the bounding-sphere radius before the point
// nearest the sphere's centre (never backwards): the roots are the same,
// but the quadratics' terms, which grow with the squared distance of the
// origin, no longer cancel (in float the unshifted forms move about 0.5 %
// of hits by more than 1e-4 relative for a one-ulp change of the ray, and
// the shifted forms none). An origin outside the bounding sphere keeps the
// cone's cap selection exact.
// ---------------------------------------------------------- Bezier curves
// The cubic's point and derivative at t, as BezierCurve::f / dfdt write
// them (DeviceCopyableObjects.h:1034-1057).
struct Curve {
  float3 w0, w1, w2, w3;
  float r;
  __device__ __forceinline__ float3 f(float t) const {
    const float ti = 1.0f - t;
    return ti * ti * ti * w0 + 3.0f * ti * ti * t * w1 + 3.0f * ti * t * t * w2 + t * t * t * w3;
  }
  __device__ __forceinline__ float3 dfdt(float t) const {
    const float ti = 1.0f - t;
    return -3.0f * ti * ti * w0 + 3.0f * (3.0f * t * t - 4.0f * t + 1.0f) * w1 +
           3.0f * (2.0f - 3.0f * t) * t * w2 + 3.0f * t * t * w3;
  }
};

__device__ __forceinline__ Curve loadCurve(const DGroup &G, int leaf) {
  const float4 *P = G.apPrims + kApStride * (size_t)leaf;
  const float4 a = __ldg(P), b = __ldg(P + 1), c = __ldg(P + 2), e = __ldg(P + 3);
  Curve cv;
  cv.w0 = f3(a.x, a.y, a.z);
  cv.w1 = f3(b.x, b.y, b.z);
  cv.w2 = f3(c.x, c.y, c.z);
  cv.w3 = f3(e.x, e.y, e.z);
  cv.r = a.w;
  return cv;
}

// The Phantom ray-hair intersector (Reshetov and Luebke 2018) as
// intersect(Ray, BezierCurve) writes it (DeviceCopyableObjects.h:1072-1289):
// an early-out against a cylinder around the end points (radius: the
// farther of the curve points at t = 1/3 and 2/3 from the axis, plus r),
// the curve moved into the ray-centric frame (e3 = the normalised ray
// direction, e1, e2 make_orthonormal_basis, origin at the ray's), then up
// to 40 Newton steps on the ray / cone (here cylinder) test from one end
// (the end the ray direction points away from), regula falsi when the step
// changes sign (bisection every 4th step), the other end if that fails;
// converged at |dt| < 5e-5. t is the distance along the normalised
// direction; u the curve parameter. The RCC transform is applied as the
// frame's transpose (its inverse).
static __device__ __noinline__ float curveHitT(float3 o, float3 d, const Curve &c, float &uOut) {
  auto distToAxis = [&](float3 pt) {
    return length(cross(pt - c.w0, pt - c.w3)) / length(c.w3 - c.w0);
  };
  float rmax = fmaxf(distToAxis(c.f(0.33333f)), distToAxis(c.f(0.66667f))) + c.r;
  const float3 axis = normalize(c.w3 - c.w0);
  const float3 p0 = c.w0 - axis * c.r, p1 = c.w3 + axis * c.r;
  {
    const float3 ba = p1 - p0, oc = o - p0;
    const float baba = dot(ba, ba), bard = dot(ba, d), baoc = dot(ba, oc);
    const float k2 = baba - bard * bard;
    const float k1 = baba * dot(oc, d) - baoc * bard;
    const float k0 = baba * dot(oc, oc) - baoc * baoc - rmax * rmax * baba;
    float h = k1 * k1 - k2 * k0;
    if (h < 0.0f) return -FLT_MAX;
    h = sqrtf(h);
    float t = (-k1 - h) / k2;
    const float y = baoc + t * bard;
    bool hitCyl = y > 0.0f && y < baba;
    if (!hitCyl) {
      t = ((y < 0.0f ? 0.0f : baba) - baoc) / bard;
      hitCyl = fabsf(k1 + k2 * t) < h;
    }
    if (!hitCyl) return -FLT_MAX;
  }
  float3 e1, e2;
  const float3 e3 = normalize(d);
  orthonormalBasis(e1, e2, e3);
  auto rcc = [&](float3 p) {
    const float3 q = p - o;
    return f3(dot(e1, q), dot(e2, q), dot(e3, q));
  };
  Curve x;
  x.w0 = rcc(c.w0);
  x.w1 = rcc(c.w1);
  x.w2 = rcc(c.w2);
  x.w3 = rcc(c.w3);
  x.r = c.r;
  float tstart = dot(x.w3 - x.w0, d) > 0.0f ? 0.0f : 1.0f;
  for (int ep = 0; ep < 2; ++ep) {
    float t = tstart, told = 0.f, dt1 = 0.f, dt2 = 0.f;
    for (int i = 0; i < 40; ++i) {
      const float3 c0 = x.f(t), cd = x.dfdt(t);
      // RayConeIntersection::intersect(r, 0) (appendix A)
      const float r2 = c.r * c.r;
      float ddd = cd.x * cd.x + cd.y * cd.y;
      const float dp = c0.x * c0.x + c0.y * c0.y;
      const float cdd = c0.x * cd.x + c0.y * cd.y;
      const float cxd = c0.x * cd.y - c0.y * cd.x;
      const float cc = ddd;
      const float b = cd.z * (0.0f - cdd);
      const float cdz2 = cd.z * cd.z;
      ddd += cdz2;
      const float a = 2.0f * 0.0f * cdd + cxd * cxd - ddd * r2 + dp * cdz2;
      const float discr = b * b - a * cc;
      const float sRoot = (b - (discr > 0.0f ? sqrtf(discr) : 0.0f)) / cc;
      float dt = (sRoot * cd.z - cdd) / ddd;
      if (discr > 0.0f && fabsf(dt) < 5e-5f) {
        uOut = t;
        return sRoot + c0.z;
      }
      dt = fminf(dt, 0.5f);
      dt = fmaxf(dt, -0.5f);
      dt1 = dt2;
      dt2 = dt;
      if (dt1 * dt2 < 0.0f) {
        const float tnext = (i & 3) == 0 ? 0.5f * (told + t) : (dt2 * told - dt1 * t) / (dt2 - dt1);
        told = t;
        t = tnext;
      } else {
        told = t;
        t += dt;
      }
      if (t < 0.0f || t > 1.0f) break;
    }
    tstart = 1.0f - tstart;
  }
  return -FLT_MAX;
}

__device__ __forceinline__ float analyticHitT(const DGroup &G, int leaf, uint32_t kind, float3 o,
                                              float3 d, float &u, float &v) {
  const float4 A = __ldg(G.apPrims + kApStride * (size_t)leaf);
  u = 0.f;
  v = 0.f;
  if (kind == AP_SPHERE) return sphereHitT(o, d, A);
  if (kind == AP_CURVE) return curveHitT(o, d, loadCurve(G, leaf), u);
  const float4 B = __ldg(G.apPrims + kApStride * (size_t)leaf + 1);
  const float3 pa = f3(A.x, A.y, A.z), pb = f3(B.x, B.y, B.z);
  const float R = 0.5f * length(pb - pa) + fmaxf(A.w, B.w);
  const float L2 = dot(d, d);
  const float tc = dot(0.5f * (pa + pb) - o, d) / L2;
  const float t0 = fmaxf(0.f, tc - 2.f * R / sqrtf(L2));
  const float3 o2 = o + t0 * d;
  const float t = kind == AP_CONE ? coneHitT(o2, d, A, B, u, v) : cylinderHitT(o2, d, A, B);
  return t == -FLT_MAX ? t : t0 + t;
}

// The slab tests below evaluate (plane - o) / d as fma(plane, 1/d, -o/d).
// A zero direction component would make 1/d infinite and the fma
// inf - inf = NaN, so every box would be missed by axis-parallel rays
// (orthographic cameras looking down an axis, say); such a component is
// replaced by +-1e-30, which keeps the interval's signs and stays finite
// for coordinates up to 1e8.
__device__ __forceinline__ float slabInv(float d) {
  return 1.f / (fabsf(d) < 1e-30f ? copysignf(1e-30f, d) : d);
}

// Stack-based BVH2 traversal, near child first, in the while-while form
// (an inner-node loop, then a leaf loop) so the lanes of a warp stay in
// step. One loop serves closest-hit and any-hit rays (anyHit stops at the
// first accepted hit), so shadow/AO rays and radiance rays in one warp share
// the same instructions. Closest hits are ordered by (t, instance, triangle),
// the order the CPU restatement uses, so any valid BVH gives the same hit.
// Analytic = true walks the group's BVH of spheres, cones and cylinders.
template <bool Count, bool Analytic = false>
__device__ __forceinline__ bool traverseGroup(const DGroup &G, float3 o, float3 d, float tmin,
                                              int inst, bool anyHit, Hit &best, uint32_t &err,
                                              unsigned long long *cnt) {
  const float3 inv = f3(slabInv(d.x), slabInv(d.y), slabInv(d.z));
  const float3 oi = f3(-o.x * inv.x, -o.y * inv.y, -o.z * inv.z);
  int stack[kTraversalStack];
  int sp = 0;
#if VSR_SMEM_STACK > 0
  // the stack's first VSR_SMEM_STACK entries in shared memory (one column
  // per thread: conflict-free), deeper ones in the local array
  __shared__ int sstack[VSR_SMEM_STACK][256];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const bool useS = tid < 256;
#define VSR_PUSH(v)                                                             \
  do {                                                                          \
    if (useS && sp < VSR_SMEM_STACK) sstack[sp][tid] = (v);                     \
    else stack[useS ? sp - VSR_SMEM_STACK : sp] = (v);                          \
    ++sp;                                                                       \
  } while (0)
#define VSR_POP() (--sp, (useS && sp < VSR_SMEM_STACK) ? sstack[sp][tid] : stack[useS ? sp - VSR_SMEM_STACK : sp])
#else
#define VSR_PUSH(v) (stack[sp++] = (v))
#define VSR_POP() stack[--sp]
#endif
  int node = 0;
  bool found = false, done = false;
  unsigned nodeVisits = 0, triTests = 0;
  unsigned long long innerW = 0, leafW = 0;
  unsigned leafL = 0;
  while (!done) {
    // inner nodes until a leaf comes up or nothing is left
    while (node >= 0) {
      const float4 *N = (Analytic ? G.apNodes : G.nodes) + 4 * (size_t)node;
      const float4 n0 = __ldg(N), n1 = __ldg(N + 1), n2 = __ldg(N + 2);
      const int4 n3 = __ldg(reinterpret_cast<const int4 *>(N + 3));
      if (Count) {
        ++nodeVisits;
        innerW += 65536u / (unsigned)__popc(__activemask());
      }
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
        if (sp == 0) {
          done = true;
          break;
        }
        node = VSR_POP();
      } else {
        int near = h0 ? n3.x : n3.y;
        if (h0 && h1) {
          int far = n3.y;
          if (c1min < c0min) { near = n3.y; far = n3.x; }
          if (sp < kTraversalStack) VSR_PUSH(far);
          else err |= ERR_STACK_OVERFLOW;
        }
        node = near;
      }
    }
    // leaves until an inner node comes up or nothing is left
    while (!done && node < 0) {
      if (Count) {
        ++leafL;
        leafW += 65536u / (unsigned)__popc(__activemask());
      }
      const uint32_t code = ~(uint32_t)node;
      const int first = (int)(code & kLeafFirstMask);
      const int count = (int)(code >> kLeafCountShift) + 1;
      for (int k = 0; k < count; ++k) {
        if constexpr (Analytic) {
          if (Count) ++triTests;
          const uint32_t lk = __ldg(G.apLocal + first + k);
          float u, v;
          const float t = analyticHitT(G, first + k, lk >> kApKindShift, o, d, u, v);
          if (!(t >= tmin)) continue;
          const int local = G.numTris + (int)(lk & kApLocalMask);
          const bool closer =
              t < best.t || (t == best.t && best.inst >= 0 &&
                             (inst < best.inst || (inst == best.inst && local < best.tri)));
          if (!closer) continue;
          best.t = t; best.u = u; best.v = v; best.inst = inst; best.tri = local;
          best.leaf = first + k;
          found = true;
          continue;
        }
        const float4 *T = G.tris + 3 * (size_t)(first + k);
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
      if ((anyHit && found) || sp == 0) {
        done = true;
        break;
      }
      node = VSR_POP();
    }
  }
  if (Count) {
    atomicAdd(&cnt[1], (unsigned long long)nodeVisits);
    atomicAdd(&cnt[2], (unsigned long long)triTests);
    // histogram of inner-node visits per traversal, bins [2^k, 2^(k+1))
    const int bin = nodeVisits ? min(31 - __clz(nodeVisits), 15) : 0;
    atomicAdd(&cnt[8 + bin], 1ull);
    atomicAdd(&cnt[27], innerW);
    atomicAdd(&cnt[28], (unsigned long long)leafL);
    atomicAdd(&cnt[29], leafW);
  }
  return found;
}

__device__ __forceinline__ void cswap(float &ka, int &ca, float &kb, int &cb) {
  if (kb < ka) {
    const float tk = ka; ka = kb; kb = tk;
    const int tc = ca; ca = cb; cb = tc;
  }
}

// Same contract as traverseGroup, over 4-wide nodes (vsr_device.h): one
// 128-byte fetch tests four child boxes; hit children are ordered by entry
#undef VSR_PUSH
#undef VSR_POP

// distance (a five-exchange sorting network), the nearest is visited next
// and the others are pushed farthest first.
template <bool Count>
__device__ __forceinline__ bool traverseGroup4(const DGroup &G, float3 o, float3 d, float tmin,
                                               int inst, bool anyHit, Hit &best, uint32_t &err,
                                               unsigned long long *cnt) {
  const float3 inv = f3(slabInv(d.x), slabInv(d.y), slabInv(d.z));
  const float3 oi = f3(-o.x * inv.x, -o.y * inv.y, -o.z * inv.z);
  int stack[kTraversalStack];
  int sp = 0;
  int node = 0;
  bool found = false, done = false;
  unsigned nodeVisits = 0, triTests = 0;
  while (!done) {
    while (node >= 0) {
      const float4 *N = G.nodes + 8 * (size_t)node;
      const float4 lx = __ldg(N), hx = __ldg(N + 1), ly = __ldg(N + 2), hy = __ldg(N + 3),
                   lz = __ldg(N + 4), hz = __ldg(N + 5);
      const int4 cc = __ldg(reinterpret_cast<const int4 *>(N + 6));
      if (Count) ++nodeVisits;
      const float tb = best.t;
      float k[4];
      int c[4] = {cc.x, cc.y, cc.z, cc.w};
      const float lxs[4] = {lx.x, lx.y, lx.z, lx.w}, hxs[4] = {hx.x, hx.y, hx.z, hx.w};
      const float lys[4] = {ly.x, ly.y, ly.z, ly.w}, hys[4] = {hy.x, hy.y, hy.z, hy.w};
      const float lzs[4] = {lz.x, lz.y, lz.z, lz.w}, hzs[4] = {hz.x, hz.y, hz.z, hz.w};
      int hits = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float a0 = fmaf(lxs[j], inv.x, oi.x), b0 = fmaf(hxs[j], inv.x, oi.x);
        const float a1 = fmaf(lys[j], inv.y, oi.y), b1 = fmaf(hys[j], inv.y, oi.y);
        const float a2 = fmaf(lzs[j], inv.z, oi.z), b2 = fmaf(hzs[j], inv.z, oi.z);
        const float cmin = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fmaxf(fminf(a2, b2), tmin));
        const float cmax = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fminf(fmaxf(a2, b2), tb));
        // empty slots are excluded by their code: no box encoding is safe
        // against a slab test that orders the two planes itself
        const bool h = cmin <= cmax && c[j] != kEmptyChild;
        k[j] = h ? cmin : FLT_MAX;
        hits += h;
      }
      if (hits == 0) {
        if (sp == 0) {
          done = true;
          break;
        }
        node = stack[--sp];
        continue;
      }
      cswap(k[0], c[0], k[1], c[1]);
      cswap(k[2], c[2], k[3], c[3]);
      cswap(k[0], c[0], k[2], c[2]);
      cswap(k[1], c[1], k[3], c[3]);
      cswap(k[1], c[1], k[2], c[2]);
      if (sp + hits - 1 > kTraversalStack) {
        err |= ERR_STACK_OVERFLOW;
        hits = 1 + (kTraversalStack - sp);
      }
      if (hits > 3) stack[sp++] = c[3];
      if (hits > 2) stack[sp++] = c[2];
      if (hits > 1) stack[sp++] = c[1];
      node = c[0];
    }
    while (!done && node < 0) {
      const uint32_t code = ~(uint32_t)node;
      const int first = (int)(code & kLeafFirstMask);
      const int count = (int)(code >> kLeafCountShift) + 1;
      for (int kk = 0; kk < count; ++kk) {
        const float4 *T = G.tris + 3 * (size_t)(first + kk);
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
        best.leaf = first + kk;
        found = true;
      }
      if ((anyHit && found) || sp == 0) {
        done = true;
        break;
      }
      node = stack[--sp];
    }
  }
  if (Count) {
    atomicAdd(&cnt[1], (unsigned long long)nodeVisits);
    atomicAdd(&cnt[2], (unsigned long long)triTests);
    const int bin = nodeVisits ? min(31 - __clz(nodeVisits), 15) : 0;
    atomicAdd(&cnt[8 + bin], 1ull);
  }
  return found;
}

// Iso-surface test, intersect(Ray, ISOSurface), DeviceCopyableObjects.h:
// 825-911, as the reference's CPU device runs it but without its 16^3
// empty-space grid. That is a known divergence, not an equivalence: the
// reference walks the grid's cells by DDA and restarts the march in each
// cell whose value range holds an iso value, so a lattice interval that
// straddles the boundary between such a cell and an empty one is not
// sampled there, while this march samples it; a crossing right next to an
// empty macro-cell can therefore come out at a slightly different t (the
// reference CUDA device builds no grid at all and marches 1 world unit per
// step). Here: in voxel space with the direction normalised, samples on
// the lattice anchored at
// tmin - dt/2 (by repeated addition, dt = step * |S d|) over [tmin, tmax]
// clipped to the field box; the first lattice interval whose two values
// bracket an iso value (inclusive) gives the hit by linear interpolation
// (the smallest over the iso values bracketed there; an interval bracketing
// one with equal ends stops the march without a hit, as there). Samples use
// the exact fp32 filter. Returns the object-space t, or -FLT_MAX. Kept out
// of line: inlined at every surface-trace site it would take the
// full-feature kernels from about 150 to 254 registers.
__device__ __forceinline__ float fieldAt(const DVolume &V, float3 P, bool hw);
static __device__ __noinline__ float isoHitT(const DIso &I, float3 o, float3 d, float tmin, float tmax,
                                      uint32_t &err) {
  const DVolume &V = I.field;
  const float3 inv = f3(1.f / d.x, 1.f / d.y, 1.f / d.z);
  const float3 t1b = (ld3(V.boundsLo) - o) * inv, t2b = (ld3(V.boundsHi) - o) * inv;
  const float tnear = maxe(min3(t1b, t2b)), tfar = mine(max3(t1b, t2b));
  if (!(tnear <= tfar)) return -FLT_MAX;
  tmin = fmaxf(tmin, tnear);
  tmax = fminf(tmax, tfar);
  const float3 Sv = ld3(V.S);
  const float3 ov = Sv * (o + ld3(V.T));
  float3 dv = Sv * d;
  const float scale = length(dv);
  dv = normalize(dv);
  const float t0v = tmin * scale, t1v = tmax * scale;
  const float dt = scale * I.step;
  if (!(dt > 0.f)) return -FLT_MAX;
  int budget = 1 << 22;
  float t0 = t0v - dt / 2.f, t1 = t0v - dt / 2.f;
  while (t0 < t0v) {
    t0 += dt;
    if (--budget <= 0) { err |= ERR_MARCH_LIMIT; return -FLT_MAX; }
  }
  while (t1 < t1v) {
    t1 += dt;
    if (--budget <= 0) { err |= ERR_MARCH_LIMIT; return -FLT_MAX; }
  }
  float v1 = fieldAt(V, ov + dv * t0, false);
  for (float t = t0; t < t1; t += dt) {
    if (--budget <= 0) { err |= ERR_MARCH_LIMIT; return -FLT_MAX; }
    const float v2 = fieldAt(V, ov + dv * (t + dt), false);
    const float lo = fminf(v1, v2), hi = fmaxf(v1, v2);
    bool hit = false;
    float best = FLT_MAX;
    for (int i = 0; i < I.numValues; ++i) {
      const float iso = __ldg(I.values + i);
      if (iso >= lo && iso <= hi) {
        const float f = (iso - v1) / (v2 - v1);
        const float tHit = t + dt * f;
        if (tHit < best) best = tHit;
        hit = true;
      }
    }
    if (hit) return best < FLT_MAX ? best / scale : -FLT_MAX;
    v1 = v2;
  }
  return -FLT_MAX;
}

// intersectSurfaces(Ray, TLS, shadow), DeviceCopyableObjects.h:1826-1839,
// with intersect(Ray, Instance) :1772-1814 for the instance transform.
template <bool Count, bool Full = false>
__device__ __forceinline__ bool traceSurfaces(const DScene &S, const Ray &r, bool anyHit, Hit &h,
                                              uint32_t &err, unsigned long long *cnt) {
  h.t = r.tmax;
  h.inst = -1;
  h.tri = -1;
  h.leaf = -1;
  h.u = h.v = 0.f;
  if (Count) atomicAdd(&cnt[0], 1ull);
  bool any = false;
  for (int i = 0; i < S.numInstances; ++i) {
    const DInstance &I = S.instances[i];
    const DGroup &G = S.groups[I.group];
    if (!Full && G.numNodes == 0) continue;
    float3 lo, ld;
    localRay(I, r.o, r.d, lo, ld);
    bool f = false;
    if (!Full || G.numNodes > 0)
      f = G.width == 4 ? traverseGroup4<Count>(G, lo, ld, r.tmin, i, anyHit, h, err, cnt)
                       : traverseGroup<Count>(G, lo, ld, r.tmin, i, anyHit, h, err, cnt);
    if (Full && G.apNumNodes > 0 && !(anyHit && f))
      f = traverseGroup<Count, true>(G, lo, ld, r.tmin, i, anyHit, h, err, cnt) || f;
    if (Full && G.numIso > 0) {
      for (int k = 0; k < G.numIso && !(anyHit && f); ++k) {
        const float t = isoHitT(G.isos[k], lo, ld, r.tmin, h.t, err);
        if (!(t >= r.tmin)) continue;
        const int local = G.numTris + G.numAP + k;
        const bool closer = t < h.t || (t == h.t && h.inst >= 0 &&
                                        (i < h.inst || (i == h.inst && local < h.tri)));
        if (!closer) continue;
        h.t = t; h.u = 0.f; h.v = 0.f; h.inst = i; h.tri = local; h.leaf = k;
        f = true;
      }
    }
    if (f) {
      any = true;
      if (anyHit) break;
    }
  }
  if (!any) h.t = FLT_MAX;
  return any;
}

// Surface index of a hit (a triangle's, or with Full an analytic
// primitive's).
template <bool Full>
__device__ __forceinline__ uint32_t hitSurface(const DGroup &G, const Hit &h) {
  if (Full && h.tri >= G.numTris + G.numAP) return G.isos[h.leaf].surface;
  if (Full && h.tri >= G.numTris) return __ldg(G.apSurface + (h.tri - G.numTris));
  return __ldg(G.triSurface + h.tri);
}

// Object-space geometric normal of a hit at the instance-local hit position
// P, getNormals (renderer/common.h:241-303): normalize(e1 x e2) for a
// triangle (for a quad's triangles the stored normal of the quad); normalize((P - c) / r) for a sphere; for a cone the cap axis
// (u <= 0, u >= 1) or the body normal from the axis parameter v; for a
// cylinder the cap axis within the radius of an end point, else P minus
// its projection on the axis; for an iso-surface the normalised central-
// difference field gradient (renderer/common.h:304-314; NaN where the
// difference is zero, as there).
__device__ __forceinline__ float3 fieldGradient(const DVolume &V, float3 P, float3 delta, bool hw);
// (out of line for the same reason as isoHitT)
static __device__ __noinline__ float3 isoNormal(const DIso &I, float3 P) {
  const DVolume &V = I.field;
  const float3 Sv = ld3(V.S);
  return fieldGradient(V, Sv * (P + ld3(V.T)), Sv * V.cellSize, false);
}
template <bool Full>
__device__ __forceinline__ float3 hitNormal(const DGroup &G, const DInstance &I, const Hit &h,
                                            float3 o, float3 d) {
  if (Full && h.tri >= G.numTris + G.numAP) {  // iso-surface: the field gradient
    float3 lo, ld;
    localRay(I, o, d, lo, ld);
    return isoNormal(G.isos[h.leaf], lo + h.t * ld);
  }
  if (Full && h.tri >= G.numTris) {
    float3 lo, ld;
    localRay(I, o, d, lo, ld);
    const float3 P = lo + h.t * ld;
    const uint32_t kind = __ldg(G.apLocal + h.leaf) >> kApKindShift;
    const float4 A = __ldg(G.apPrims + kApStride * (size_t)h.leaf);
    const float3 v1 = f3(A.x, A.y, A.z);
    if (kind == AP_SPHERE) return normalize((P - v1) / A.w);
    if (kind == AP_CURVE) {  // getNormals: P minus the curve point at u (renderer/common.h:304-308)
      return normalize(P - loadCurve(G, h.leaf).f(h.u));
    }
    const float4 B = __ldg(G.apPrims + kApStride * (size_t)h.leaf + 1);
    const float3 v2 = f3(B.x, B.y, B.z);
    if (kind == AP_CONE) {
      const float3 ba = v2 - v1;
      const float m0 = dot(ba, ba);
      if (h.u <= 0.f) return -ba * (1.f / sqrtf(m0));
      if (h.u >= 1.f) return ba * (1.f / sqrtf(m0));
      const float ra = A.w, rr = A.w - B.w;
      const float hy = m0 + rr * rr;
      return normalize(m0 * (m0 * (P - v1) + rr * ba * ra) - ba * hy * h.v);
    }
    const float3 axis = normalize(v2 - v1);
    if (length(P - v1) < A.w) return -axis;
    if (length(P - v2) < A.w) return axis;
    const float s = dot(P - v1, axis);
    return normalize(P - (v1 + s * axis));
  }
  if (Full && G.triNormal) {  // quads: the normal getNormals picks for the quad
    const float4 n = __ldg(G.triNormal + h.tri);
    if (n.w != 0.f) return f3(n.x, n.y, n.z);
  }
  const float4 *E = G.tris + 3 * (size_t)h.leaf;
  const float4 e1 = __ldg(E + 1), e2 = __ldg(E + 2);
  return normalize(cross(f3(e1.x, e1.y, e1.z), f3(e2.x, e2.y, e2.z)));
}

// -------------------------------------------------- attributes, samplers
// toRGBA (common.h:265-360): the components an element has, the rest of
// (0, 0, 0, 1); unorm components as value / (2^bits - 1). An index past
// the array reads the default.
__device__ __forceinline__ float4 attrFetch(const DAttr &a, uint32_t i) {
  float c[4] = {0.f, 0.f, 0.f, 1.f};
  if (i < a.len) {
    const int n = a.comps;
    if (a.fixedBits == 8) {
      const uint8_t *p = (const uint8_t *)a.data + (size_t)i * n;
      for (int k = 0; k < n; ++k) c[k] = p[k] / 255.f;
    } else if (a.fixedBits == 16) {
      const uint16_t *p = (const uint16_t *)a.data + (size_t)i * n;
      for (int k = 0; k < n; ++k) c[k] = p[k] / 65535.f;
    } else {
      const float *p = (const float *)a.data + (size_t)i * n;
      for (int k = 0; k < n; ++k) c[k] = p[k];
    }
  }
  return make_float4(c[0], c[1], c[2], c[3]);
}

// lerp_r(a, b, c, u, v) over a triangle's corners: (1 - u - v) a + u b + v c
__device__ __forceinline__ float4 baryLerp(float4 a, float4 b, float4 c, float u, float v) {
  const float w = 1.f - u - v;
  return make_float4(w * a.x + u * b.x + v * c.x, w * a.y + u * b.y + v * c.y,
                     w * a.z + u * b.z + v * c.z, w * a.w + u * b.w + v * c.w);
}

// What getAttributes (renderer/common.h:523-543) sees of a surface hit.
struct AttrCtx {
  const DSurfAttr *sa;
  const DInstAttr *ia;
  uint32_t primID;
  float u, v;
  float3 worldPos, worldNormal, objectPos, objectNormal;
};

// getAttribute (renderer/common.h:365-521) for triangles: face-varying
// values, else per-vertex values, else the primitive's, interpolated with
// the hit's barycentrics; then the geometry's uniform value, then the
// instance's; else (0, 0, 0, 1). Hit attributes are (value, 1).
static __device__ __noinline__ float4 getAttr(const AttrCtx &c, int id) {
  if (id >= ATTR_WORLD_POS && id <= ATTR_OBJECT_NORMAL) {
    const float3 h = id == ATTR_WORLD_POS      ? c.worldPos
                     : id == ATTR_WORLD_NORMAL ? c.worldNormal
                     : id == ATTR_OBJECT_POS   ? c.objectPos
                                               : c.objectNormal;
    return make_float4(h.x, h.y, h.z, 1.f);
  }
  if (id < 0 || id > ATTR_COLOR || !c.sa) return make_float4(0.f, 0.f, 0.f, 1.f);
  const DSurfAttr &s = *c.sa;
  if (s.isTriangle) {
    const uint32_t p = c.primID;
    if (s.faceVarying[id].comps) {
      return baryLerp(attrFetch(s.faceVarying[id], 3 * p), attrFetch(s.faceVarying[id], 3 * p + 1),
                      attrFetch(s.faceVarying[id], 3 * p + 2), c.u, c.v);
    }
    if (s.vertex[id].comps) {
      uint32_t i0 = 3 * p, i1 = 3 * p + 1, i2 = 3 * p + 2;
      if (s.index) { i0 = s.index[i0]; i1 = s.index[i1]; i2 = s.index[i2]; }
      return baryLerp(attrFetch(s.vertex[id], i0), attrFetch(s.vertex[id], i1),
                      attrFetch(s.vertex[id], i2), c.u, c.v);
    }
    if (s.primitive[id].comps) return attrFetch(s.primitive[id], p);
  }
  if (s.uniformMask & (1u << id))
    return make_float4(s.uniform[id][0], s.uniform[id][1], s.uniform[id][2], s.uniform[id][3]);
  if (c.ia && (c.ia->mask & (1u << id)))
    return make_float4(c.ia->v[id][0], c.ia->v[id][1], c.ia->v[id][2], c.ia->v[id][3]);
  return make_float4(0.f, 0.f, 0.f, 1.f);
}

// Shading normal of a triangle hit in object space (getNormals, renderer/
// common.h:241-264): the vertex normals interpolated and normalised (with
// face-varying normals set, the reference reads the vertex normals at the
// face-varying positions 3 primID + k), else the geometric normal.
__device__ __forceinline__ float3 shadingNormal(const DSurfAttr &s, uint32_t p, float u, float v,
                                                float3 Ng) {
  if (!s.isTriangle || !s.vertexNormal) return Ng;
  uint32_t i0 = 3 * p, i1 = 3 * p + 1, i2 = 3 * p + 2;
  if (!s.fvNormal && s.index) { i0 = s.index[i0]; i1 = s.index[i1]; i2 = s.index[i2]; }
  if (i0 >= s.numVertexNormals || i1 >= s.numVertexNormals || i2 >= s.numVertexNormals) return Ng;
  const float *N = s.vertexNormal;
  const float4 a = make_float4(N[3 * i0], N[3 * i0 + 1], N[3 * i0 + 2], 0.f);
  const float4 b = make_float4(N[3 * i1], N[3 * i1 + 1], N[3 * i1 + 2], 0.f);
  const float4 c = make_float4(N[3 * i2], N[3 * i2 + 1], N[3 * i2 + 2], 0.f);
  const float4 n = baryLerp(a, b, c, u, v);
  return normalize(f3(n.x, n.y, n.z));
}

// mat4 (column-major) times a vector, columns summed in order.
__device__ __forceinline__ float4 mat4mul(const float *m, float4 v) {
  return make_float4(((m[0] * v.x + m[4] * v.y) + m[8] * v.z) + m[12] * v.w,
                     ((m[1] * v.x + m[5] * v.y) + m[9] * v.z) + m[13] * v.w,
                     ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w,
                     ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w);
}

// A texel index under the sampler's address mode: clampToEdge, repeat or
// mirrorRepeat (toAddressMode, sampler/Sampler.cpp).
__device__ __forceinline__ int wrapIndex(float fi, int n, int mode) {
  const int i = !(fi > -1e9f && fi < 1e9f) ? 0 : (int)fi;
  if (mode == WRAP_REPEAT) return ((i % n) + n) % n;
  if (mode == WRAP_MIRROR) {
    const int m = ((i % (2 * n)) + 2 * n) % (2 * n);
    return m < n ? m : 2 * n - 1 - m;
  }
  return i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
}

__device__ __forceinline__ float4 texel(const DSampler &s, int i, int j, int k) {
  const uchar4 t = s.texels[((size_t)k * s.dims[1] + j) * s.dims[0] + i];
  return make_float4(t.x / 255.f, t.y / 255.f, t.z / 255.f, t.w / 255.f);
}

// tex1D / tex2D / tex3D over the RGBA8 image: normalized coordinates,
// texel centres at (i + 0.5) / n; linear: the lattice neighbours weighted
// along x, then y, then z; nearest: the texel containing the point.
static __device__ __noinline__ float4 imageSample(const DSampler &s, float4 tc) {
  const int axes = s.type == SAMP_IMAGE1D ? 1 : (s.type == SAMP_IMAGE2D ? 2 : 3);
  const float c[3] = {tc.x, tc.y, tc.z};
  int i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0};
  float f[3] = {0.f, 0.f, 0.f};
  for (int a = 0; a < axes; ++a) {
    const int n = s.dims[a];
    if (s.linear) {
      const float x = c[a] * n - 0.5f;
      const float fl = floorf(x);
      f[a] = x - fl;
      i0[a] = wrapIndex(fl, n, s.wrap[a]);
      i1[a] = wrapIndex(fl + 1.f, n, s.wrap[a]);
    } else {
      i0[a] = i1[a] = wrapIndex(floorf(c[a] * n), n, s.wrap[a]);
    }
  }
  auto lerp4 = [](float4 p, float4 q, float t) {
    return make_float4(p.x + t * (q.x - p.x), p.y + t * (q.y - p.y), p.z + t * (q.z - p.z),
                       p.w + t * (q.w - p.w));
  };
  const float4 c00 = lerp4(texel(s, i0[0], i0[1], i0[2]), texel(s, i1[0], i0[1], i0[2]), f[0]);
  if (axes == 1) return c00;
  const float4 c10 = lerp4(texel(s, i0[0], i1[1], i0[2]), texel(s, i1[0], i1[1], i0[2]), f[0]);
  const float4 c0 = lerp4(c00, c10, f[1]);
  if (axes == 2) return c0;
  const float4 c01 = lerp4(texel(s, i0[0], i0[1], i1[2]), texel(s, i1[0], i0[1], i1[2]), f[0]);
  const float4 c11 = lerp4(texel(s, i0[0], i1[1], i1[2]), texel(s, i1[0], i1[1], i1[2]), f[0]);
  return lerp4(c0, lerp4(c01, c11, f[1]), f[2]);
}

// getSample (renderer/common.h:546-590): primitive samplers read element
// primID + offset; transform samplers map the input attribute; image
// samplers transform the input attribute (inTransform, inOffset), look the
// image up and transform the texel (outTransform, outOffset).
__device__ __forceinline__ float4 getSample(const DSampler &s, const AttrCtx &c) {
  if (s.type == SAMP_PRIMITIVE) return attrFetch(s.prim, c.primID + s.primOffset);
  float4 a = getAttr(c, s.inAttribute);
  if (s.type == SAMP_TRANSFORM) {
    const float4 r = mat4mul(s.outXfm, a);
    return make_float4(r.x + s.outOffset[0], r.y + s.outOffset[1], r.z + s.outOffset[2],
                       r.w + s.outOffset[3]);
  }
  a = mat4mul(s.inXfm, a);
  a = make_float4(a.x + s.inOffset[0], a.y + s.inOffset[1], a.z + s.inOffset[2], a.w + s.inOffset[3]);
  const float4 r = mat4mul(s.outXfm, imageSample(s, a));
  return make_float4(r.x + s.outOffset[0], r.y + s.outOffset[1], r.z + s.outOffset[2],
                     r.w + s.outOffset[3]);
}

__device__ __forceinline__ float4 materialParam(const DScene &S, int src, float4 value,
                                                const AttrCtx &c) {
  if (src == SRC_VALUE) return value;
  if (src >= SRC_SAMPLER) return getSample(S.samplers[src - SRC_SAMPLER], c);
  return getAttr(c, src);
}

// The material at a hit with its parameters looked up (getColor, getF,
// getOpacity; renderer/common.h:642-710): base colour from the colour
// parameter, opacity = colour.w x the opacity parameter, metallic and
// roughness from theirs (the .x of a sample or attribute).
static __device__ __noinline__ DMaterial resolveMaterial(const DScene &S, const DMaterial &m,
                                                  const AttrCtx &c) {
  DMaterial r = m;
  const float4 col = materialParam(S, m.src[MSRC_COLOR],
                                   make_float4(m.baseColor[0], m.baseColor[1], m.baseColor[2], 1.f), c);
  r.baseColor[0] = col.x;
  r.baseColor[1] = col.y;
  r.baseColor[2] = col.z;
  r.opacity = col.w * materialParam(S, m.src[MSRC_OPACITY], make_float4(m.opacity, 0.f, 0.f, 1.f), c).x;
  if (m.type == MAT_PBR) {
    r.metallic = materialParam(S, m.src[MSRC_METALLIC], make_float4(m.metallic, 0.f, 0.f, 1.f), c).x;
    r.roughness =
        materialParam(S, m.src[MSRC_ROUGHNESS], make_float4(m.roughness, 0.f, 0.f, 1.f), c).x;
  }
  return r;
}

// The attribute context of a surface hit: the surface's attribute record,
// the instance's, the primitive (triangles: its index in the geometry) and
// barycentrics; hit attributes as the caller fills them.
__device__ __forceinline__ AttrCtx hitAttrCtx(const DScene &S, const DGroup &G, const Hit &h,
                                              uint32_t surf) {
  AttrCtx c;
  c.sa = S.surfAttr ? S.surfAttr + surf : nullptr;
  c.ia = S.instAttr ? S.instAttr + h.inst : nullptr;
  c.primID = h.tri < G.numTris ? __ldg(G.triPrim + h.tri) : 0u;
  c.u = h.u;
  c.v = h.v;
  c.worldPos = c.worldNormal = c.objectPos = c.objectNormal = f3(0.f);
  return c;
}

// --------------------------------------------------------------- materials
// renderer/common.h:793-1415 with constant parameters and no tangent frame.
__device__ __forceinline__ float pow5(float f) { return f * f * f * f * f; }
__device__ __forceinline__ float mapRoughness(float r) { return fmaxf(0.045f, r); }
__device__ __forceinline__ float D_GGX(float NdotH, float alpha, float EPS) {
  float alpha2 = alpha * alpha;
  float d = (NdotH * alpha2 - NdotH) * NdotH + 1.f;
  float denom = kPi * d * d;
  return alpha2 / fmaxf(EPS, denom);
}

__device__ __forceinline__ float3 materialColor(const DMaterial &m) {
  float3 base = ld3(m.baseColor);
  return m.type == MAT_PBR ? lerpR(base, f3(0.f), m.metallic) : base;
}

__device__ __forceinline__ float materialOpacity(const DMaterial &m) {
  if (m.alphaMode == ALPHA_OPAQUE) return 1.f;
  if (m.alphaMode == ALPHA_BLEND) return m.opacity;
  return m.opacity >= m.alphaCutoff ? 1.f : 0.f;
}

__device__ inline float3 evalPBR(const DMaterial &m, float3 Ns, float3 viewDir, float3 lightDir) {
  const float metallic = m.metallic;
  const float pr = mapRoughness(m.roughness);
  const float pcr = mapRoughness(m.clearcoatRoughness);
  const float psr = mapRoughness(m.sheenRoughness);
  const float alpha = pr * pr;
  const float clearcoatAlpha = pcr * pcr;
  const float EPS = 1e-14f;
  const float3 H = normalize(lightDir + viewDir);
  const float NdotV = fabsf(dot(Ns, viewDir)) + EPS;
  const float NdotH = fmaxf(EPS, dot(Ns, H));
  const float NdotL = fmaxf(EPS, dot(Ns, lightDir));
  const float LdotH = fmaxf(EPS, dot(lightDir, H));
  const float VdotH = fmaxf(EPS, dot(viewDir, H));
  const float3 baseColor = ld3(m.baseColor);
  const float3 diffuseColor = lerpR(baseColor, f3(0.f), metallic);
  float f0s = (1.f - m.ior) / (1.f + m.ior);
  f0s = f0s * f0s;
  const float3 f0 = lerpR(f3(f0s), baseColor, metallic);
  const float3 F = f0 + (f3(1.f) - f0) * pow5(1.f - VdotH);
  const float f90 = 0.5f + 2.f * alpha * LdotH * LdotH;
  const float lightScatter = 1.f + (f90 - 1.f) * pow5(1.f - NdotL);
  const float viewScatter = 1.f + (f90 - 1.f) * pow5(1.f - NdotV);
  const float3 diffuseBRDF = diffuseColor * (lightScatter * viewScatter * kInvPi);
  const float D = D_GGX(NdotH, alpha, EPS);
  const float a2 = alpha * alpha;
  const float GGXV = NdotL / (NdotV + sqrtf(a2 + (1.f - a2) * NdotV * NdotV));
  const float GGXL = NdotV / (NdotL + sqrtf(a2 + (1.f - a2) * NdotL * NdotL));
  const float V = 0.5f / (GGXV + GGXL);
  const float3 specularBRDF = F * (D * V);
  const float Dc = D_GGX(NdotH, clearcoatAlpha, EPS);
  const float Vc = 0.25f / fmaxf(EPS, LdotH * LdotH);
  const float Fc = (0.04f + (1.f - 0.04f) * pow5(1.f - LdotH)) * m.clearcoat;
  const float Frc = (Dc * Vc) * Fc;
  const float sheenAlphaInv = 1.f / psr;
  const float cos2h = NdotH * NdotH;
  const float sin2h = fmaxf(1.f - cos2h, 0.0078125f);
  const float3 Ds =
      ld3(m.sheenColor) * ((2.f + sheenAlphaInv) * powf(sin2h, sheenAlphaInv * 0.5f) / kTwoPi);
  return ((diffuseBRDF + specularBRDF) * (1.f - Fc) + f3(Frc)) + Ds;
}

__device__ __forceinline__ float3 evalMaterial(const DMaterial &m, float3 Ns, float3 viewDir,
                                               float3 lightDir) {
  if (m.type == MAT_MATTE) return ld3(m.baseColor) * kInvPi;
  return evalPBR(m, Ns, viewDir, lightDir);
}

struct BSDFSample {
  float3 dir, f;
  float pdf, cosT;
};

__device__ __forceinline__ float3 sampleGGXVNDF(float3 V, float ax, float ay, float U1, float U2) {
  float3 Vh = normalize(V * f3(ax, ay, 1.f));
  float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  float3 T1 = lensq > 0.f ? f3(-Vh.y, Vh.x, 0.f) / sqrtf(lensq) : f3(1.f, 0.f, 0.f);
  float3 T2 = cross(Vh, T1);
  float r = sqrtf(U1);
  float phi = kTwoPi * U2;
  float sp, cp;
  sincosf(phi, &sp, &cp);
  float t1 = r * cp;
  float t2 = r * sp;
  float s = 0.5f * (1.f + Vh.z);
  t2 = (1.f - s) * sqrtf(fmaxf(0.f, 1.f - t1 * t1)) + s * t2;
  float3 Nh = t1 * T1 + t2 * T2 + sqrtf(1.f - t1 * t1 - t2 * t2) * Vh;
  return normalize(f3(Nh.x * ax, Nh.y * ay, fmaxf(0.f, Nh.z)));
}

__device__ __forceinline__ void pdfGGXVNDF(float3 L, float3 V, float ax, float eta_i, float eta_t,
                                           float3 Ns, float &pdfSpec, float &pdfTrans) {
  const float EPS = 1e-14f;
  pdfSpec = 0.f;
  pdfTrans = 0.f;
  const float NdotL = dot(Ns, L);
  const float NdotV = fmaxf(EPS, dot(Ns, V));
  const float ax2 = ax * ax;
  if (NdotL > 0.f) {
    float3 H = V + L;
    float lenH = length(H);
    if (lenH > 1e-4f) {
      H /= lenH;
      float NdotH = fmaxf(EPS, dot(Ns, H));
      float D = D_GGX(NdotH, ax, EPS);
      float G1 = 2.f * NdotV / (NdotV + sqrtf(ax2 + (1.f - ax2) * NdotV * NdotV));
      pdfSpec = (D * G1) / (4.f * NdotV);
    }
  } else if (NdotL < 0.f) {
    float3 H = -(V * eta_i + L * eta_t);
    float lenH = length(H);
    if (lenH > 1e-4f) {
      H /= lenH;
      if (dot(Ns, H) < 0.f) H = -H;
      float NdotH = fmaxf(EPS, dot(Ns, H));
      float LdotH = fabsf(dot(L, H));
      float VdotH = fabsf(dot(V, H));
      if (VdotH > 0.f && LdotH > 0.f) {
        float D = D_GGX(NdotH, ax, EPS);
        float G1 = 2.f * NdotV / (NdotV + sqrtf(ax2 + (1.f - ax2) * NdotV * NdotV));
        float pdfNe = (D * G1 * VdotH) / NdotV;
        float denom = (eta_i * VdotH + eta_t * LdotH);
        float jacobian = (eta_t * eta_t * LdotH) / (denom * denom);
        pdfTrans = pdfNe * jacobian;
      }
    }
  }
}

// sampleMaterial, renderer/common.h:1371-1415 and :1209-1368.
__device__ inline BSDFSample sampleMaterial(const DMaterial &m, float3 Ng, float3 Ns, float3 viewDir,
                                     Rng &rnd) {
  BSDFSample res;
  float3 w = faceforward(Ns, viewDir, Ng);
  float3 v = fabsf(w.x) > fabsf(w.y) ? normalize(f3(-w.z, 0.f, w.x)) : normalize(f3(0.f, w.z, -w.y));
  float3 u = cross(v, w);
  if (m.type == MAT_MATTE) {
    float u1 = rnd(), u2 = rnd();
    float3 sp = cosineSampleHemisphere(u1, u2);
    res.dir = normalize(sp.x * u + sp.y * v + sp.z * w);
    res.pdf = fmaxf(0.f, dot(Ns, res.dir)) * kInvPi;
  } else {
    const float EPS = 1e-14f;
    const float metallic = m.metallic;
    const float pr = mapRoughness(m.roughness);
    const float alpha = pr * pr;
    const float pcr = mapRoughness(m.clearcoatRoughness);
    const float clearcoatAlpha = pcr * pcr;
    const float NdotV = fmaxf(EPS, dot(Ns, viewDir));
    const float3 baseColor = ld3(m.baseColor);
    const float3 diffuseColor = lerpR(baseColor, f3(0.f), metallic);
    float f0s = (1.f - m.ior) / (1.f + m.ior);
    f0s = f0s * f0s;
    const float3 f0 = lerpR(f3(f0s), baseColor, metallic);
    const float3 F = f0 + (f3(1.f) - f0) * pow5(1.f - NdotV);
    const float fClear = m.clearcoat * 0.04f;
    const float baseEnergy = 1.f - fClear;
    const float fSpec = luminance(F);
    const float remainingEnergy = baseEnergy * (1.f - fSpec);
    const float wDiff = luminance(diffuseColor) * remainingEnergy * (1.f - m.transmission);
    const float wSpec = baseEnergy * fSpec;
    const float wTrans = remainingEnergy * m.transmission;
    const float wSum = wDiff + wSpec + wTrans + fClear;
    const float pDiff = wSum > 0.f ? wDiff / wSum : 0.0f;
    const float pSpec = wSum > 0.f ? wSpec / wSum : 0.333f;
    const float pTrans = wSum > 0.f ? wTrans / wSum : 0.667f;
    const float pClear = 1.f - pDiff - pSpec - pTrans;
    const float lobe = rnd();
    const float3 V = f3(dot(u, viewDir), dot(v, viewDir), dot(w, viewDir));
    const bool entering = dot(Ns, viewDir) > 0.f;
    const float eta_i = entering ? 1.0f : m.ior;
    const float eta_t = entering ? m.ior : 1.0f;
    const float u1 = rnd(), u2 = rnd();
    if (lobe < pDiff) {
      float3 sp = cosineSampleHemisphere(u1, u2);
      res.dir = normalize(sp.x * u + sp.y * v + sp.z * w);
    } else if (lobe < pDiff + pSpec) {
      float3 Ne = sampleGGXVNDF(V, alpha, alpha, u1, u2);
      res.dir = reflect(viewDir, u * Ne.x + v * Ne.y + w * Ne.z);
    } else if (lobe < pDiff + pSpec + pTrans) {
      float3 Ne = sampleGGXVNDF(V, alpha, alpha, u1, u2);
      if (dot(V, Ne) < 0.f) Ne = -Ne;
      float3 Nw = u * Ne.x + v * Ne.y + w * Ne.z;
      res.dir = refract(viewDir, Nw, eta_t / eta_i);
      if (length(res.dir) < 1e-4f) res.dir = reflect(viewDir, Nw);
    } else {
      float3 Ne = sampleGGXVNDF(V, clearcoatAlpha, clearcoatAlpha, u1, u2);
      res.dir = reflect(viewDir, u * Ne.x + v * Ne.y + w * Ne.z);
    }
    const float pdfDiff = fmaxf(0.f, dot(Ns, res.dir)) * kInvPi;
    float pdfSpec = 0.f, pdfTrans = 0.f;
    pdfGGXVNDF(res.dir, viewDir, alpha, eta_i, eta_t, Ns, pdfSpec, pdfTrans);
    float pdfClear = 0.f, dummy = 0.f;
    pdfGGXVNDF(res.dir, viewDir, clearcoatAlpha, entering ? 1.0f : 1.5f, entering ? 1.5f : 1.0f, Ns,
               pdfClear, dummy);
    res.pdf = pDiff * pdfDiff + pSpec * pdfSpec + pTrans * pdfTrans + pClear * pdfClear;
  }
  res.cosT = fmaxf(0.f, dot(Ns, res.dir));
  res.f = evalMaterial(m, Ns, viewDir, res.dir);
  return res;
}

// ------------------------------------------------------------------ light
// sampleLight, renderer/common.h:1432-1466, towards reference point P.
// Directional (scene/light/Directional.cpp:30-40): dist2 = 1, pdf = 1,
// dist = FLT_MAX; a positive angular diameter samples a uniform cone (two
// draws). Point (scene/light/Point.cpp:28-37: constant attenuation 1) and
// spot (DeviceCopyableObjects.h:2286-2321): direction P -> position, dist
// its length, dist2 = dist^2, pdf 1, three draws for a random light normal
// that delta lights do not use; the spot's intensity falls off with a
// smoothstep between the outer and inner cone cosines.
struct LightSample {
  float3 intensity, dir;
  float pdf, dist, dist2;
};

// ------------------------------------------------------------ HDRI light
// pi in double: the reference writes M_PI in these formulas
constexpr double kPiD = 3.14159265358979323846;

// upper_bound and sample_cdf of sampleCDF.h:16-55: the first bin whose CDF
// value exceeds x and that bin's probability. Past the table's end the
// reference reads an unset value; here the probability is 0 there.
__device__ __forceinline__ unsigned cdfBin(const float *d, unsigned n, float x, float &pdf) {
  unsigned first = 0;
  int count = (int)n;
  while (count > 0) {
    const int step = count / 2;
    const unsigned it = first + step;
    if (!(x < d[it])) {
      first = it + 1;
      count -= step + 1;
    } else {
      count = step;
    }
  }
  if (first == 0) pdf = d[0];
  else if (first < n) pdf = d[first] - d[first - 1];
  else pdf = 0.f;
  return first;
}

// sampleCDF (sampleCDF.h:84-94): the row from the CDF of row sums, then the
// column from that row's CDF. The light record's table named `rows` holds
// the row sums and `lastCol` the per-row tables (scene/light/HDRI.cpp:
// 156-157 assigns them crosswise, and sampleCDF takes them in that order),
// so the lookup is the usual marginal-then-conditional one.
__device__ __forceinline__ void hdriSampleCdf(const DLight &L, float rx, float ry, unsigned &x,
                                              unsigned &y, float &pdfx, float &pdfy) {
  const unsigned W = (unsigned)L.hdriW, H = (unsigned)L.hdriH;
  y = cdfBin(L.hdriLastCol, H, ry, pdfy);
  y = min(y, H - 1);
  x = cdfBin(L.hdriRows + (size_t)y * W, W, rx, pdfx);
}

// toPolar / toUV (sampleCDF.h:57-82); the angle arithmetic runs in double
// as the reference's M_PI constants make it, rounded to float where the
// reference stores a float.
__device__ __forceinline__ float3 hdriToPolar(float u, float v) {
  const float theta = (float)(2.0f * kPiD * (double)u + -kPiD / 2.0f);
  const float phi = (float)(kPiD * (double)v);
  float3 n;
  n.x = cosf(theta) * sinf(phi);
  n.z = sinf(theta) * sinf(phi);
  n.y = cosf(phi);
  n.x = -n.x;
  return n;
}
__device__ __forceinline__ float2 hdriToUV(float3 n) {
  float2 uv;
  uv.x = atan2f(n.x, n.z);
  uv.x = (float)(((double)uv.x + kPiD / 2.0f) / (kPiD * 2.0f) + kPiD * (double)(28.670f / 360.0f));
  uv.y = fminf(fmaxf((float)((double)acosf(n.y) / kPiD), .001f), .999f);
  return uv;
}

__device__ __forceinline__ float3 mat3mulCM(const float *m, float3 v) {
  return make_float3((m[0] * v.x + m[3] * v.y) + m[6] * v.z, (m[1] * v.x + m[4] * v.y) + m[7] * v.z,
                     (m[2] * v.x + m[5] * v.y) + m[8] * v.z);
}

// tex2D over the radiance image: normalized coordinates, texel centres at
// (i + 0.5) / n, bilinear, clamp (HDRI.cpp:129-131), filtered in software
// as the reference's CPU device does.
__device__ __forceinline__ float3 hdriTex(const DLight &L, float2 uv) {
  const int W = L.hdriW, H = L.hdriH;
  const float x = uv.x * W - 0.5f, y = uv.y * H - 0.5f;
  const float fx0 = floorf(x), fy0 = floorf(y);
  const float fx = x - fx0, fy = y - fy0;
  auto cl = [](float f, int n) { return !(f >= 0.f) ? 0 : (f > (float)(n - 1) ? n - 1 : (int)f); };
  const int x0 = cl(fx0, W), x1 = cl(fx0 + 1.f, W), y0 = cl(fy0, H), y1 = cl(fy0 + 1.f, H);
  const float4 a = L.hdriTex[(size_t)y0 * W + x0], b = L.hdriTex[(size_t)y0 * W + x1];
  const float4 c = L.hdriTex[(size_t)y1 * W + x0], d = L.hdriTex[(size_t)y1 * W + x1];
  auto lerp3 = [](float4 p, float4 q, float t) {
    return make_float3(p.x + t * (q.x - p.x), p.y + t * (q.y - p.y), p.z + t * (q.z - p.z));
  };
  const float3 r0 = lerp3(a, b, fx), r1 = lerp3(c, d, fx);
  return r0 + fy * (r1 - r0);
}

// intensity(dir) = tex2D(radiance, toUV(toLocal dir)).xyz * scale
// (DeviceCopyableObjects.h:2384-2388).
__device__ __forceinline__ float3 hdriIntensity(const DLight &L, float3 dir) {
  return hdriTex(L, hdriToUV(mat3mulCM(L.toLocal, dir))) * L.scale;
}

// The density the reference gives a direction that hits the HDRI light, for
// the MIS weight of a BSDF sample (Pathtrace_impl.cpp:160-172): the CDF is
// looked up with the direction's (u, v) as if they were random numbers,
// and the bin probabilities are divided by 2 pi^2 sin(theta) / (W H).
__device__ __forceinline__ float hdriHitPdf(const DLight &L, float3 rayDir) {
  const float3 dir = mat3mulCM(L.toLocal, rayDir);
  const float2 uv = hdriToUV(dir);
  unsigned x, y;
  float pdfx, pdfy;
  hdriSampleCdf(L, uv.x, uv.y, x, y, pdfx, pdfy);
  const float theta = acosf(fminf(fmaxf(dir.y, -1.f), 1.f));
  const float sinTheta = sinf(theta);
  if (sinTheta == 0.f) return 0.f;
  return (pdfx * pdfy) * (float)((unsigned)L.hdriW * (unsigned)L.hdriH) /
         (2.0f * kPi * kPi * sinTheta);
}

// Positional = false compiles the directional light only (the kernels
// that run near their register budget, for worlds without point or spot
// lights).
template <bool Positional>
__device__ __forceinline__ LightSample sampleLight(const DLight &L, float3 P, Rng &rnd) {
  LightSample s;
  if (Positional && L.type == LIGHT_QUAD) {
    // Quad light (the reference's area_light<float, dco::Quad>; Visionaray's
    // sampling is not in the reference, so its conventions are restated):
    // sample_surface(Quad) picks the first triangle when A1 / (A1 + A2) < r
    // (DeviceCopyableObjects.h:2258-2271), then a uniform point of the
    // triangle from two draws (v1 + sqrt(u1) (1 - u2) a + sqrt(u1) u2 b);
    // intensity = color * intensity; the pdf is the area density over the
    // light-side cosine, 1 / (A |cos|), so that intensity / dist^2 / pdf
    // is the light's contribution per unit solid angle as renderer/
    // common.h:1441-1464 and Pathtrace_impl.cpp:343-354 use it.
    const float r = rnd();
    const float3 e1 = ld3(L.e1), e2 = ld3(L.e2), d = e1 + e2;
    float3 a = d, b = e2;
    if (L.area1 / (L.area1 + L.area2) < r) { a = e1; b = d; }
    const float u1 = rnd(), u2 = rnd();
    const float su = sqrtf(u1);
    const float3 pos = ld3(L.pos) + a * (su * (1.f - u2)) + b * (su * u2);
    s.dir = pos - P;
    s.dist = length(s.dir);
    s.dist2 = s.dist * s.dist;
    const float cosL = fabsf(dot(s.dir, ld3(L.normal))) / s.dist;
    s.pdf = 1.f / ((L.area1 + L.area2) * cosL);
    s.intensity = ld3(L.intensity);
    return s;
  }
  if (Positional && L.type == LIGHT_HDRI) {
    // HDRI light (DeviceCopyableObjects.h:2371-2382): a texel from the
    // CDFs, its corner's direction through toPolar into world space,
    // pdf = pdfx pdfy W H / (4 pi), dist = FLT_MAX, dist2 = 1
    // (renderer/common.h:1459-1461), intensity looked up along that
    // direction. The two draws are arguments of one call, which C++ leaves
    // unordered; GCC, which builds the reference's CPU device, evaluates
    // them right to left, so the row's draw comes first.
    const float ry = rnd();
    const float rx = rnd();
    unsigned x, y;
    float pdfx, pdfy;
    hdriSampleCdf(L, rx, ry, x, y, pdfx, pdfy);
    const float invJacobian = (float)((unsigned)L.hdriW * (unsigned)L.hdriH) / (float)(4 * kPiD);
    const float3 Lp = hdriToPolar(x / (float)L.hdriW, y / (float)L.hdriH);
    s.dir = mat3mulCM(L.toWorld, Lp);
    s.dist = FLT_MAX;
    s.dist2 = 1.f;
    s.pdf = pdfx * pdfy * invJacobian;
    s.intensity = hdriIntensity(L, s.dir);
    return s;
  }
  if (Positional && L.type != LIGHT_DIRECTIONAL) {
    s.intensity = ld3(L.intensity);
    s.pdf = 1.f;
    s.dir = ld3(L.pos) - P;
    s.dist = length(s.dir);
    s.dist2 = s.dist * s.dist;
    (void)rnd(); (void)rnd(); (void)rnd();
    if (L.type == LIGHT_SPOT) {
      float spot = dot(normalize(ld3(L.dir)), normalize(-s.dir));
      if (spot < L.cosOuter) {
        s.intensity = f3(0.f);
      } else if (!(spot > L.cosInner)) {
        spot = (spot - L.cosOuter) / (L.cosInner - L.cosOuter);
        s.intensity = s.intensity * (spot * spot * (3.f - 2.f * spot));
      }
    }
    return s;
  }
  float3 d = ld3(L.dir);
  if (L.cosHalfAngle < 1.f) {
    float u1 = rnd(), u2 = rnd();
    float cz = 1.f - u1 * (1.f - L.cosHalfAngle);
    float sz = sqrtf(fmaxf(0.f, 1.f - cz * cz));
    float phi = kTwoPi * u2;
    float3 a, b;
    orthonormalBasis(a, b, d);
    d = normalize(a * (sz * cosf(phi)) + b * (sz * sinf(phi)) + d * cz);
  }
  s.dir = d;
  s.dist = FLT_MAX;
  s.pdf = 1.f;
  s.dist2 = 1.f;
  s.intensity = ld3(L.intensity);
  return s;
}

// power_heuristic(a, b) = a^2 / (a^2 + b^2) (the MIS weight of
// renderer/Pathtrace_impl.cpp:175, :367-369).
__device__ __forceinline__ float powerHeuristic(float a, float b) {
  const float a2 = a * a;
  return a2 / (a2 + b * b);
}

// The light the ray meets (intersectLights, renderer/common.h:1566-1603):
// a quad light by intersect(Ray, Quad), which tests the two tessellated
// triangles and keeps the nearer hit (DeviceCopyableObjects.h:2211-2237;
// both sides lit), taken when nearer than the hit so far; an HDRI light
// always, at distance FLT_MAX, taken when nothing was hit yet or, against
// another light at FLT_MAX, when it is visible and that one is not. At
// bounce 0 invisible lights are skipped. Returns the light's index or -1,
// and its distance.
__device__ __forceinline__ bool quadLightTriT(float3 o, float3 d, float3 v1, float3 e1, float3 e2,
                                              float tmin, float tmax, float &t) {
  const float3 s1 = cross(d, e2);
  const float div = dot(s1, e1);
  if (div == 0.f) return false;
  const float idiv = 1.f / div;
  const float3 dd = o - v1;
  const float bb1 = dot(dd, s1) * idiv;
  if (bb1 < 0.f || bb1 > 1.f) return false;
  const float3 s2 = cross(dd, e1);
  const float bb2 = dot(d, s2) * idiv;
  if (bb2 < 0.f || bb1 + bb2 > 1.f) return false;
  t = dot(e2, s2) * idiv;
  return t >= tmin && t <= tmax;
}
__device__ __forceinline__ int intersectLights(const DScene &S, float3 o, float3 d, float tmin,
                                               float tmax, unsigned bounceID, float &tl) {
  int id = -1;
  bool vis = false;
  tl = FLT_MAX;
  for (int i = 0; i < S.numLights; ++i) {
    const DLight &L = S.lights[i];
    if ((L.type != LIGHT_QUAD && L.type != LIGHT_HDRI) || (bounceID == 0 && !L.visible)) continue;
    if (L.type == LIGHT_HDRI) {
      if (id < 0 || (tl == FLT_MAX && L.visible && !vis)) {
        tl = FLT_MAX;
        vis = L.visible != 0;
        id = i;
      }
      continue;
    }
    const float3 v1 = ld3(L.pos), e1 = ld3(L.e1), e2 = ld3(L.e2), dd = e1 + e2;
    float t1 = FLT_MAX, t2 = FLT_MAX;
    const bool h1 = quadLightTriT(o, d, v1, e1, dd, tmin, tmax, t1);
    const bool h2 = quadLightTriT(o, d, v1, dd, e2, tmin, tmax, t2);
    float t = FLT_MAX;
    if (h1) t = t1;
    if (h2 && t2 < t) t = t2;
    if ((h1 || h2) && t < tl) {
      tl = t;
      vis = L.visible != 0;
      id = i;
    }
  }
  return id;
}

// Normalised central-difference gradient of the field at voxel-space point
// P, one offset of `delta` per axis (sampleGradient,
// DeviceCopyableObjects.h:582-597; a structured field is sampled
// everywhere, so the difference is always taken). A zero difference
// normalises to NaN components, as in the reference, and fails the length
// tests that follow.
__device__ __forceinline__ float fieldAt(const DVolume &V, float3 P, bool hw);
__device__ __forceinline__ float3 fieldGradient(const DVolume &V, float3 P, float3 delta, bool hw) {
  const float x1 = fieldAt(V, P + f3(delta.x, 0.f, 0.f), hw);
  const float x0 = fieldAt(V, P - f3(delta.x, 0.f, 0.f), hw);
  const float y1 = fieldAt(V, P + f3(0.f, delta.y, 0.f), hw);
  const float y0 = fieldAt(V, P - f3(0.f, delta.y, 0.f), hw);
  const float z1 = fieldAt(V, P + f3(0.f, 0.f, delta.z), hw);
  const float z0 = fieldAt(V, P - f3(0.f, 0.f, delta.z), hw);
  const float3 g = f3(x1, y1, z1) - f3(x0, y0, z0);
  return g / sqrtf(dot(g, g));
}

// Gradient shading of one classified sample (rayMarchVolume<1>,
// renderer/VolumeIntegration.h:420-460): a matte surface of the sample's
// colour along the gradient, lit by every light, plus the ambient term.
// Like the reference, the gradient and P are in voxel space and the light
// directions in world space (a point or spot light is sampled towards the
// voxel-space P, VolumeIntegration.h:435). viewDir need not be normalised.
// The raycast renderer has no random stream (renderer/Raycast_impl.cpp:267):
// each light is sampled with a zero-state generator, as for surfaces.
__device__ __forceinline__ float3 gradientShade(const DScene &S, const DRenderer &R,
                                                const DVolume &V, float3 P, float3 delta,
                                                float3 viewDir, float3 rgb, bool hw) {
  float3 gn = fieldGradient(V, P, delta, hw);
  gn = faceforward(gn, viewDir, gn);
  float3 shaded = f3(0.f);
  if (length(gn) > 1e-10f) {
    for (int li = 0; li < S.numLights; ++li) {
      Rng none;
      none.state = 0;
      const LightSample ls = sampleLight<true>(S.lights[li], P, none);
      const float3 lightDir = normalize(ls.dir);
      const float3 lightIntensity = ls.intensity * safeRcp(ls.dist2);
      const float NdotL = fmaxf(0.f, dot(gn, lightDir));
      shaded += rgb * kInvPi * lightIntensity * NdotL * safeRcp(ls.pdf);
    }
  }
  return shaded + rgb * ld3(R.ambientColor) * R.ambientRadiance;
}

// ----------------------------------------------------------------- volumes
// tex3D(normalized coords, linear, clamp) on the structured field,
// sampleField DeviceCopyableObjects.h:478-481; texel i is centred at
// (i+0.5)/N.
__device__ __forceinline__ float sampleField(const DVolume &V, float3 P) {
  const int nx = V.dims[0], ny = V.dims[1], nz = V.dims[2];
  const float x = P.x * nx - 0.5f, y = P.y * ny - 0.5f, z = P.z * nz - 0.5f;
  const float fx0 = floorf(x), fy0 = floorf(y), fz0 = floorf(z);
  const float fx = x - fx0, fy = y - fy0, fz = z - fz0;
  const int ix = (int)fminf(fmaxf(fx0, -1.f), (float)nx);
  const int iy = (int)fminf(fmaxf(fy0, -1.f), (float)ny);
  const int iz = (int)fminf(fmaxf(fz0, -1.f), (float)nz);
  const int x0 = min(max(ix, 0), nx - 1), x1 = min(max(ix + 1, 0), nx - 1);
  const int y0 = min(max(iy, 0), ny - 1), y1 = min(max(iy + 1, 0), ny - 1);
  const int z0 = min(max(iz, 0), nz - 1), z1 = min(max(iz + 1, 0), nz - 1);
  const float *d = V.data;
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  const size_t r00 = z0 * sz + y0 * sy, r10 = z0 * sz + y1 * sy;
  const size_t r01 = z1 * sz + y0 * sy, r11 = z1 * sz + y1 * sy;
  const float c00 = lerpf(__ldg(d + r00 + x0), __ldg(d + r00 + x1), fx);
  const float c10 = lerpf(__ldg(d + r10 + x0), __ldg(d + r10 + x1), fx);
  const float c01 = lerpf(__ldg(d + r01 + x0), __ldg(d + r01 + x1), fx);
  const float c11 = lerpf(__ldg(d + r11 + x0), __ldg(d + r11 + x1), fx);
  const float c0 = lerpf(c00, c10, fy);
  const float c1 = lerpf(c01, c11, fy);
  return lerpf(c0, c1, fz);
}

// Field sample in voxel space: the texture unit's trilinear filter (as
// tex3D in the reference's CUDA device) or the exact fp32 filter above.
__device__ __forceinline__ float fieldAt(const DVolume &V, float3 P, bool hw) {
  return hw ? tex3D<float>(V.tex, P.x, P.y, P.z) : sampleField(V, P);
}

// tex1D over the TF table (normalized, linear, clamp) after postClassify's
// value-range normalisation, DeviceCopyableObjects.h:614-619.
__device__ __forceinline__ float4 tfLookup(const float4 *tf, int n, float vrMin, float vrMax,
                                           float val) {
  val = (val - vrMin) / (vrMax - vrMin);
  const float x = val * n - 0.5f;
  const float f0 = floorf(x);
  const float f = x - f0;
  const int i = (int)fminf(fmaxf(f0, -1.f), (float)n);
  const int i0 = min(max(i, 0), n - 1), i1 = min(max(i + 1, 0), n - 1);
  const float4 a = tf[i0], b = tf[i1];
  return make_float4(lerpf(a.x, b.x, f), lerpf(a.y, b.y, f), lerpf(a.z, b.z, f), lerpf(a.w, b.w, f));
}

// Classification of a field value. The exact path divides by the value
// range as postClassify does; the hardware-filter path, already approximate,
// multiplies by the precomputed reciprocal.
__device__ __forceinline__ float4 classify(const DVolume &V, const float4 *tf, float val, bool hw) {
  if (!hw) return tfLookup(tf, V.tfSize, V.vrMin, V.vrMax, val);
  const int n = V.tfSize;
  const float x = (val - V.vrMin) * V.vrScale * n - 0.5f;
  const float f0 = floorf(x);
  const float f = x - f0;
  const int i = (int)fminf(fmaxf(f0, -1.f), (float)n);
  const int i0 = min(max(i, 0), n - 1), i1 = min(max(i + 1, 0), n - 1);
  const float4 a = tf[i0], b = tf[i1];
  return make_float4(lerpf(a.x, b.x, f), lerpf(a.y, b.y, f), lerpf(a.z, b.z, f), lerpf(a.w, b.w, f));
}

struct BoxHit {
  bool hit;
  float tnear, tfar;
};
__device__ __forceinline__ BoxHit intersectBox(float3 o, float3 d, const float *lo, const float *hi) {
  float3 inv = f3(1.f) / d;
  float3 t1 = (ld3(lo) - o) * inv, t2 = (ld3(hi) - o) * inv;
  BoxHit b;
  b.tnear = maxe(min3(t1, t2));
  b.tfar = mine(max3(t1, t2));
  b.hit = b.tnear <= b.tfar;
  return b;
}

__device__ __forceinline__ int projectOnGrid1(float v, float lo, float hi, int n) {
  float v01 = (v - lo) / (hi - lo);
  int c = (int)fminf(fmaxf(v01 * (float)n, -1.f), (float)n);
  return min(max(c, 0), n - 1);
}

// dda3, renderer/DDA.h:12-113, with projectOnGrid and linearIndex
// (scene/volume/spatial_field/GridAccel-common.h:9-25): walks the cells of
// a gx x gy x gz grid spanning [blo, bhi] that the ray o + t d crosses from
// tmin on, calling cell(id, t0, t1) with id = (z gy + y) gx + x for each
// until it returns false or the walk leaves the grid (t1 is clipped to
// tmax; the walk itself goes on past tmax, as the reference's does). A walk
// of more than 4 (gx + gy + gz) + 16 cells sets ERR_DDA_LIMIT and stops.
// The two products that a compiler would fuse into multiply-adds (the
// moved origin and the first cell boundaries) are rounded separately, as
// in the reference's own (uncontracted) arithmetic, so the walk visits the
// same cells at the same parameters bit for bit.
template <typename CellFn>
__device__ __forceinline__ void ddaWalk(float3 o, float3 d, float tmin, float tmax, float3 blo,
                                        float3 bhi, int gx, int gy, int gz, uint32_t &err,
                                        CellFn &&cell) {
  const float ray_tmin = tmin;
  const float3 ro = f3(__fadd_rn(o.x, __fmul_rn(tmin, d.x)), __fadd_rn(o.y, __fmul_rn(tmin, d.y)),
                       __fadd_rn(o.z, __fmul_rn(tmin, d.z)));
  const float rtmax = tmax - ray_tmin;
  const float3 rcp = f3(1.f) / d;
  const float3 lo = (blo - ro) * rcp;
  const float3 hi = (bhi - ro) * rcp;
  float3 tnear = min3(lo, hi);
  const float3 tfar = max3(lo, hi);
  if (d.x == 0.f) tnear.x = FLT_MAX;
  if (d.y == 0.f) tnear.y = FLT_MAX;
  if (d.z == 0.f) tnear.z = FLT_MAX;
  int cx = projectOnGrid1(ro.x, blo.x, bhi.x, gx);
  int cy = projectOnGrid1(ro.y, blo.y, bhi.y, gy);
  int cz = projectOnGrid1(ro.z, blo.z, bhi.z, gz);
  const float3 dist = max3(f3(0.f), (tfar - tnear) / f3((float)gx, (float)gy, (float)gz));
  const int stx = d.x > 0.f ? 1 : -1, sty = d.y > 0.f ? 1 : -1, stz = d.z > 0.f ? 1 : -1;
  const int spx = d.x > 0.f ? gx : -1, spy = d.y > 0.f ? gy : -1, spz = d.z > 0.f ? gz : -1;
  float3 tnext;
  tnext.x = __fadd_rn(tnear.x, __fmul_rn(float(d.x > 0.f ? cx + 1 : gx - cx), dist.x));
  tnext.y = __fadd_rn(tnear.y, __fmul_rn(float(d.y > 0.f ? cy + 1 : gy - cy), dist.y));
  tnext.z = __fadd_rn(tnear.z, __fmul_rn(float(d.z > 0.f ? cz + 1 : gz - cz), dist.z));
  float t0 = 0.f;
  int steps = 4 * (gx + gy + gz) + 16;
  while (true) {
    if (--steps < 0) { err |= ERR_DDA_LIMIT; break; }
    const float t1 = fminf(mine(tnext), rtmax);
    const int id = (cz * gy + cy) * gx + cx;
    if (!cell(id, ray_tmin + t0, ray_tmin + t1)) break;
    const float tc = mine(tnext);
    if (tnext.x == tc) {
      tnext.x += dist.x;
      cx += stx;
      if (cx == spx) break;
    }
    if (tnext.y == tc) {
      tnext.y += dist.y;
      cy += sty;
      if (cy == spy) break;
    }
    if (tnext.z == tc) {
      tnext.z += dist.z;
      cz += stz;
      if (cz == spz) break;
    }
    t0 = t1;
  }
}

// Delta tracking through one volume: intersect(Ray, Volume),
// DeviceCopyableObjects.h:680-796, with the DDA of renderer/DDA.h:12-113
// over the majorant grid (voxel-space bounds [0,1]^3). Returns true on a
// scattering event at object-space parameter tHit.
template <bool Count>
__device__ bool deltaTrack(const DVolume &V, float3 o, float3 d, float tmin, float tmax, Rng &rnd,
                           float &tHit, float3 &albedo, uint32_t &err, unsigned long long *cnt,
                           bool hw) {
  BoxHit bh = intersectBox(o, d, V.boundsLo, V.boundsHi);
  if (!bh.hit || bh.tfar < tmin || bh.tnear > tmax) return false;
  tmin = fmaxf(tmin, bh.tnear);
  tmax = fminf(tmax, bh.tfar);
  const float3 S = ld3(V.S);
  o = S * (o + ld3(V.T));
  d = S * d;
  const float dt_scale = length(d);
  d = normalize(d);
  tmin *= dt_scale;
  tmax *= dt_scale;
  const float unitDistance = V.unitDistance * dt_scale;
  const float invUnitDistance = 1.f / unitDistance;
  bool hit = false;
  float ht = tmax;
  unsigned samples = 0, cells = 0;
  int budget = 1 << 22;

  auto woodcock = [&](int leafID, float t0, float t1) -> bool {
    if (Count) ++cells;
    const float majorant = V.majorant ? __ldg(V.majorant + leafID) : 1.f;
    float t = t0;
    while (true) {
      if (majorant <= 0.f) break;
      t -= (logf(1.f - rnd()) / (majorant * invUnitDistance));
      if (t >= t1) break;
      if (Count) ++samples;
      if (--budget <= 0) { err |= ERR_TRACK_LIMIT; return false; }
      float3 P = o + d * t;
      float4 s = classify(V, V.tf, fieldAt(V, P, hw), hw);
      float u = rnd();
      if (s.w >= u * majorant) {
        albedo = f3(s.x, s.y, s.z);
        hit = true;
        ht = t;
        return false;
      }
    }
    return true;
  };

  if (V.majorant) {
    // dda3 with modelBounds = [0,1]^3 in voxel space
    ddaWalk(o, d, tmin, tmax, f3(0.f), f3(1.f), V.gdims[0], V.gdims[1], V.gdims[2], err, woodcock);
  } else {
    woodcock(-1, tmin, tmax);
  }
  if (Count) {
    atomicAdd(&cnt[4], (unsigned long long)samples);
    atomicAdd(&cnt[5], (unsigned long long)cells);
  }
  if (hit) tHit = ht / dt_scale;
  return hit;
}

// ------------------------------------------------------------------- frame
// dco::Frame::writeSample = fillGBuffer + accumSample + toneMap,
// DeviceCopyableObjects.h:2692-2781; cvt_uint32(_srgb), frame/common.h:31-48.
__device__ __forceinline__ float linearToSrgb(float x) {
  return x <= 0.0031308f ? 12.92f * x : 1.055f * powf(x, 1.f / 2.4f) - 0.055f;
}
__device__ __forceinline__ uint32_t cvtU8(float f) {
  return (uint32_t)(255.f * fminf(fmaxf(f, 0.f), 1.f));
}
// cvt_uint32 (srgb = false) / cvt_uint32_srgb (srgb = true) of one colour.
__device__ __forceinline__ uint32_t packRGBA8(float4 color, bool srgb) {
  float r = color.x, g = color.y, b = color.z;
  if (srgb) { r = linearToSrgb(r); g = linearToSrgb(g); b = linearToSrgb(b); }
  return cvtU8(r) | (cvtU8(g) << 8) | (cvtU8(b) << 16) | (cvtU8(color.w) << 24);
}

// Window position of a world point under a column-major view-projection
// matrix M (Visionaray's project, the gluProject convention: clip = M (p, 1),
// ndc = clip / w, win = size (ndc + 1) / 2), for motion vectors
// (Pathtrace_impl.cpp:290-297). Every product and sum is rounded on its own,
// in a fixed order, so the oracle's arithmetic gives the same bits.
__device__ __forceinline__ float2 projectWin(const float *M, float3 p, float W, float H) {
  auto row = [&](int r) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[r], p.x), __fmul_rn(M[4 + r], p.y)),
                               __fmul_rn(M[8 + r], p.z)),
                     M[12 + r]);
  };
  const float cx = row(0), cy = row(1), cw = row(3);
  const float nx = __fdiv_rn(cx, cw), ny = __fdiv_rn(cy, cw);
  return make_float2(__fmul_rn(__fmul_rn(W, __fadd_rn(nx, 1.f)), 0.5f),
                     __fmul_rn(__fmul_rn(H, __fadd_rn(ny, 1.f)), 0.5f));
}

// The path tracer's frame write with temporal anti-aliasing
// (dco::Frame::fillGBuffer, DeviceCopyableObjects.h:2745-2773): motion
// vector, this frame's colour and the closest sample's albedo for the
// resolve pass, then the depth-tested G-buffer; the accumulation buffer and
// the colour channel are left to the resolve pass.
__device__ __forceinline__ void fillGBufferTaa(const DFrame &F, int x, int y, float4 color,
                                               float depth, float3 Ng, float3 albedo, float2 mv) {
  const size_t idx = (size_t)y * F.width + x;
  F.motionVec[idx] = mv;
  F.taaCurr[idx] = color;
  F.taaCurrAlbedo[3 * idx] = albedo.x;
  F.taaCurrAlbedo[3 * idx + 1] = albedo.y;
  F.taaCurrAlbedo[3 * idx + 2] = albedo.z;
  if (F.depth && !(depth > F.depth[idx])) {
    F.depth[idx] = depth;
    if (F.normal) {
      F.normal[3 * idx] = Ng.x;
      F.normal[3 * idx + 1] = Ng.y;
      F.normal[3 * idx + 2] = Ng.z;
    }
    if (F.albedo) {
      F.albedo[3 * idx] = albedo.x;
      F.albedo[3 * idx + 1] = albedo.y;
      F.albedo[3 * idx + 2] = albedo.z;
    }
  }
}

// The TAA history: the previous resolved image read at normalised
// coordinates (u, v) with clamp addressing and a cardinal-spline (Catmull-
// Rom) filter over 4x4 texels, texel centres at (i + 0.5) / size, as the
// reference's history texture is set up (frame/Frame.cpp:541-545).
__device__ __forceinline__ void catmullRomWeights(float f, float w[4]) {
  const float f2 = f * f, f3 = f2 * f;
  w[0] = 0.5f * (-f3 + 2.f * f2 - f);
  w[1] = 0.5f * (3.f * f3 - 5.f * f2 + 2.f);
  w[2] = 0.5f * (-3.f * f3 + 4.f * f2 + f);
  w[3] = 0.5f * (f3 - f2);
}
__device__ __forceinline__ float4 historyAt(const float4 *img, int W, int H, float u, float v) {
  const float tx = u * (float)W - 0.5f, ty = v * (float)H - 0.5f;
  const float fx0 = floorf(tx), fy0 = floorf(ty);
  float wx[4], wy[4];
  catmullRomWeights(tx - fx0, wx);
  catmullRomWeights(ty - fy0, wy);
  const int x0 = (int)fx0 - 1, y0 = (int)fy0 - 1;
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int j = 0; j < 4; ++j) {
    const int yy = min(max(y0 + j, 0), H - 1);
    float4 row = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = 0; i < 4; ++i) {
      const int xx = min(max(x0 + i, 0), W - 1);
      const float4 t = img[(size_t)yy * W + xx];
      row.x += wx[i] * t.x; row.y += wx[i] * t.y; row.z += wx[i] * t.z; row.w += wx[i] * t.w;
    }
    r.x += wy[j] * row.x; r.y += wy[j] * row.y; r.z += wy[j] * row.z; r.w += wy[j] * row.w;
  }
  return r;
}

// lumSqMean: the mean over this frame's samples of the squared sample
// luminance (0.3 r + 0.59 g + 0.11 b), for the optional variance channel;
// negative when the caller does not track it.
__device__ __forceinline__ void writeSample(const DFrame &F, int x, int y, bool stochastic,
                                            float4 color, float depth, float3 Ng, float3 albedo,
                                            float lumSqMean = -1.f) {
  const size_t idx = (size_t)y * F.width + x;
  if (F.depth && !(depth > F.depth[idx])) {
    F.depth[idx] = depth;
    if (F.normal) {
      F.normal[3 * idx] = Ng.x;
      F.normal[3 * idx + 1] = Ng.y;
      F.normal[3 * idx + 2] = Ng.z;
    }
    if (F.albedo) {
      F.albedo[3 * idx] = albedo.x;
      F.albedo[3 * idx + 1] = albedo.y;
      F.albedo[3 * idx + 2] = albedo.z;
    }
  }
  if (stochastic) {
    int frames = F.accumID;  // frames already in this pixel's mean
    if (F.pixelFrames) {
      frames = (int)F.pixelFrames[idx];
      F.pixelFrames[idx] = (uint32_t)frames + 1u;
    }
    const float a = 1.f / (frames + 1);
    const float4 acc = F.accum[idx];
    color = make_float4((1 - a) * acc.x + a * color.x, (1 - a) * acc.y + a * color.y,
                        (1 - a) * acc.z + a * color.z, (1 - a) * acc.w + a * color.w);
    F.accum[idx] = color;
    if (F.accumSq && lumSqMean >= 0.f) {
      // variance of the mean luminance over all (accumID + 1) * spp samples
      const float m2 = (1 - a) * F.accumSq[idx] + a * lumSqMean;
      F.accumSq[idx] = m2;
      const float lm = 0.3f * color.x + 0.59f * color.y + 0.11f * color.z;
      const float n = (float)(frames + 1) * (float)F.pixelSamples;
      F.variance[idx] = n > 1.f ? fmaxf(m2 - lm * lm, 0.f) / (n - 1.f) : FLT_MAX;
    }
  }
  if (F.colorType == COLOR_FLOAT4) {
    reinterpret_cast<float4 *>(F.color)[idx] = color;
  } else if (F.colorType == COLOR_UFIXED8 || F.colorType == COLOR_SRGB8) {
    reinterpret_cast<uint32_t *>(F.color)[idx] = packRGBA8(color, F.colorType == COLOR_SRGB8);
  }
}

} // namespace vsr
