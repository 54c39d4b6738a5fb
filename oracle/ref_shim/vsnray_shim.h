// Test infrastructure: a minimal stand-in for the Visionaray math types
// (vector, box, component-wise min/max/clamp) that lets a few of the
// reference's own header-only functions compile without Visionaray, which
// is not available. Only what those functions use is defined. Visionaray's
// conventions assumed here: vector<3,int>(vector<3,float>) converts each
// component by static_cast (truncation toward zero); min/max on vectors are
// component-wise with std::min/std::max semantics; min_element is the
// smallest component.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>

#ifndef VSNRAY_FUNC
#define VSNRAY_FUNC
#endif

namespace visionaray {

template <typename T>
struct vec2t {
  T x, y;
};

template <typename T>
struct vec3t {
  T x, y, z;
  vec3t() = default;
  constexpr vec3t(T a, T b, T c) : x(a), y(b), z(c) {}
  constexpr explicit vec3t(T s) : x(s), y(s), z(s) {}
  template <typename U>
  constexpr explicit vec3t(const vec3t<U> &o)
      : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
  T &operator[](int i) { return (&x)[i]; }
  const T &operator[](int i) const { return (&x)[i]; }
};

template <typename T>
struct vec4t {
  T x, y, z, w;
  vec4t() = default;
  constexpr vec4t(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  constexpr vec4t(const vec3t<T> &v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec3t<T> xyz() const { return vec3t<T>(x, y, z); }
};

using vec2i = vec2t<int>;
using vec2ui = vec2t<unsigned>;
using vec3f = vec3t<float>;
using vec3 = vec3f;
using vec3i = vec3t<int>;
using vec4f = vec4t<float>;
using vec4 = vec4f;
using float3 = vec3f;
using float4 = vec4f;

#define VSR_SHIM_BINOP(op)                                                            \
  template <typename T>                                                              \
  inline vec3t<T> operator op(const vec3t<T> &a, const vec3t<T> &b) {               \
    return vec3t<T>(a.x op b.x, a.y op b.y, a.z op b.z);                             \
  }                                                                                  \
  template <typename T>                                                              \
  inline vec3t<T> operator op(T s, const vec3t<T> &b) {                              \
    return vec3t<T>(s op b.x, s op b.y, s op b.z);                                   \
  }                                                                                  \
  template <typename T>                                                              \
  inline vec3t<T> operator op(const vec3t<T> &a, T s) {                              \
    return vec3t<T>(a.x op s, a.y op s, a.z op s);                                   \
  }
VSR_SHIM_BINOP(+)
VSR_SHIM_BINOP(-)
VSR_SHIM_BINOP(*)
VSR_SHIM_BINOP(/)
#undef VSR_SHIM_BINOP

template <typename T>
inline vec3t<T> min(const vec3t<T> &a, const vec3t<T> &b) {
  return vec3t<T>(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z));
}
template <typename T>
inline vec3t<T> max(const vec3t<T> &a, const vec3t<T> &b) {
  return vec3t<T>(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z));
}
template <typename T>
inline vec3t<T> clamp(const vec3t<T> &v, const vec3t<T> &lo, const vec3t<T> &hi) {
  return min(max(v, lo), hi);
}
template <typename T>
inline T min_element(const vec3t<T> &v) {
  return std::min(std::min(v.x, v.y), v.z);
}
using std::min;
using std::max;

struct box3f {
  vec3f min, max;
};

// The ray type the reference's dda3 is instantiated with (basic_ray<float>).
struct ShimRay {
  vec3f ori, dir;
  float tmin, tmax;
};

} // namespace visionaray
