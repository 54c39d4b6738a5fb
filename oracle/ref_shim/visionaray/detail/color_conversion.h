// Test infrastructure: stands in for Visionaray's color_conversion.h, which
// is not available. linear_to_srgb is the sRGB encoding of IEC 61966-2-1
// (the published piecewise curve: 12.92 x up to 0.0031308, else
// 1.055 x^(1/2.4) - 0.055), applied per component. Visionaray's own code
// for it cannot be checked here, so conversions through it pin the
// reference's cvt_uint32_srgb only up to this definition.
#pragma once
#include "../../vsnray_shim.h"

namespace visionaray {

inline float linear_to_srgb(float x) {
  return x <= 0.0031308f ? 12.92f * x : 1.055f * std::pow(x, 1.f / 2.4f) - 0.055f;
}
inline vec3f linear_to_srgb(const vec3f &v) {
  return vec3f(linear_to_srgb(v.x), linear_to_srgb(v.y), linear_to_srgb(v.z));
}

} // namespace visionaray
