// CPU oracle: vector math and the sampling/shading conventions it restates.
//
// TEST INFRASTRUCTURE ONLY. This header belongs to the CPU restatement of the
// anari-visionaray CPU device that the tests and the CPU baseline use as the
// checker. Nothing in the product library includes or links it.
//
// Several helpers below live in the Visionaray library in the reference
// (not vendored, so not available to compare against). Each one is restated
// from its mathematical definition and the chosen convention is written next
// to it; these conventions are "parity unpinned".
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <algorithm>

namespace orc {

struct f2 { float x, y; };
struct f3 {
  float x, y, z;
  f3() : x(0), y(0), z(0) {}
  f3(float a) : x(a), y(a), z(a) {}
  f3(float a, float b, float c) : x(a), y(b), z(c) {}
  float &operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
};
struct f4 {
  float x, y, z, w;
  f4() : x(0), y(0), z(0), w(0) {}
  f4(float a) : x(a), y(a), z(a), w(a) {}
  f4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  f4(f3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  f3 xyz() const { return f3(x, y, z); }
};

inline f3 operator+(f3 a, f3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline f3 operator-(f3 a, f3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline f3 operator*(f3 a, f3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline f3 operator/(f3 a, f3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline f3 operator*(f3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
inline f3 operator*(float s, f3 a) { return f3(a.x * s, a.y * s, a.z * s); }
inline f3 operator/(f3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
inline f3 operator-(f3 a) { return f3(-a.x, -a.y, -a.z); }
inline f3 &operator+=(f3 &a, f3 b) { a = a + b; return a; }
inline f3 &operator*=(f3 &a, f3 b) { a = a * b; return a; }
inline f3 &operator*=(f3 &a, float s) { a = a * s; return a; }
inline f3 &operator/=(f3 &a, float s) { a = a / s; return a; }

inline f4 operator+(f4 a, f4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline f4 operator*(f4 a, float s) { return f4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline f4 operator*(float s, f4 a) { return a * s; }
inline f4 &operator+=(f4 &a, f4 b) { a = a + b; return a; }

inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline f3 cross(f3 a, f3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(f3 a) { return std::sqrt(dot(a, a)); }
// normalize(0) is 0/0 = NaN, as plain division gives.
inline f3 normalize(f3 a) { return a / length(a); }
inline f3 fabs3(f3 a) { return f3(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }
inline f3 min3(f3 a, f3 b) { return f3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
inline f3 max3(f3 a, f3 b) { return f3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
inline float max_element(f3 a) { return std::fmax(a.x, std::fmax(a.y, a.z)); }
inline float min_element(f3 a) { return std::fmin(a.x, std::fmin(a.y, a.z)); }

inline float lerpf(float a, float b, float t) { return a + t * (b - a); }
inline f3 lerp3(f3 a, f3 b, float t) { return a + t * (b - a); }

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 6.28318530717958647692f;
constexpr float kInvPi = 0.31830988618379067154f;

// faceforward(n, i, nref): n flipped onto the side of nref that i points to.
// Convention: the returned vector lies in the hemisphere of i (the reference
// calls it with i = view direction, pointing away from the surface).
inline f3 faceforward(f3 n, f3 i, f3 nref) { return dot(i, nref) < 0.f ? -n : n; }

// reflect(i, n): mirror of i about n, i pointing away from the surface;
// the result lies on the same side as i.
inline f3 reflect(f3 i, f3 n) { return 2.f * dot(n, i) * n - i; }

// refract(i, n, eta): i points away from the surface, eta = eta_t / eta_i.
// Returns 0 on total internal reflection.
inline f3 refract(f3 i, f3 n, float eta) {
  float r = 1.f / eta;
  float cosi = dot(i, n);
  float k = 1.f - r * r * (1.f - cosi * cosi);
  if (k < 0.f) return f3(0.f);
  return -r * i + (r * cosi - std::sqrt(k)) * n;
}

// Orthonormal basis around w, the construction the reference inlines in
// sampleMaterial (renderer/common.h:1296-1299).
inline void make_orthonormal_basis(f3 &u, f3 &v, f3 w) {
  v = std::fabs(w.x) > std::fabs(w.y) ? normalize(f3(-w.z, 0.f, w.x))
                                      : normalize(f3(0.f, w.z, -w.y));
  u = cross(v, w);
}

// cosine_sample_hemisphere(u1,u2): polar mapping (Malley), +z up.
inline f3 cosine_sample_hemisphere(float u1, float u2) {
  float r = std::sqrt(u1);
  float phi = kTwoPi * u2;
  return f3(r * std::cos(phi), r * std::sin(phi), std::sqrt(std::fmax(0.f, 1.f - u1)));
}

// uniform_sample_sphere(u1,u2): z = 1 - 2 u1, phi = 2 pi u2.
inline f3 uniform_sample_sphere(float u1, float u2) {
  float z = 1.f - 2.f * u1;
  float r = std::sqrt(std::fmax(0.f, 1.f - z * z));
  float phi = kTwoPi * u2;
  return f3(r * std::cos(phi), r * std::sin(phi), z);
}

inline float power_heuristic(float a, float b) {
  float a2 = a * a, b2 = b * b;
  return a2 / (a2 + b2);
}

// Luminance weights 0.3 / 0.59 / 0.11.
inline float rgb_to_luminance(f3 c) { return 0.3f * c.x + 0.59f * c.y + 0.11f * c.z; }

inline float linear_to_srgb1(float x) {
  return x <= 0.0031308f ? 12.92f * x : 1.055f * std::pow(x, 1.f / 2.4f) - 0.055f;
}

// LCG<4> from common.h:55-102 (in-reference code, so this part is exact):
// TEA-style 4-round seed mixing, then an LCG (A=1664525, C=1013904223)
// returning the low 24 bits as a float in [0,1).
struct LCG {
  uint32_t state;
  LCG() : state(0) {}
  LCG(uint32_t v0_in, uint32_t v1_in) { init(v0_in, v1_in); }
  void init(uint32_t v0, uint32_t v1) {
    uint32_t s0 = 0;
    for (unsigned n = 0; n < 4; n++) {
      s0 += 0x9e3779b9u;
      v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
      v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    state = v0;
  }
  float operator()() {
    state = 1664525u * state + 1013904223u;
    return (state & 0x00FFFFFFu) / (float)0x01000000;
  }
  float next() { return (*this)(); }
};

// epsilonFrom, renderer/common.h:14-18.
inline float epsilonFrom(f3 P, f3 dir, float t) {
  const float ulpEpsilon = 0x1.fp-18f;
  f3 aP = fabs3(P);
  float m = std::fmax(std::fmax(aP.x, aP.y), std::fmax(aP.z, max_element(fabs3(dir)) * t));
  return m * ulpEpsilon;
}

inline f4 over(f4 A, f4 B) { return A + (1.f - A.w) * B; }

} // namespace orc
