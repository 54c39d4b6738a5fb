// Test infrastructure: a C entry point around a few of the reference's own
// functions, compiled from the reference's sources (Visionaray replaced by
// the shim in ref_shim/), so that the oracle and the GPU kernels can be
// checked against reference code rather than against a restatement:
//
//   ref_lcg : LCG<4> (common.h:55-102), the struct taken verbatim from the
//             reference file by the build recipe (common.h itself needs the
//             ANARI SDK), seed mixing and the 24-bit uniform stream;
//   ref_dda : dda3 (renderer/DDA.h:12-113 with projectOnGrid / linearIndex
//             of scene/volume/spatial_field/GridAccel-common.h:9-25),
//             included unchanged, recording each visited cell and its
//             [t0, t1];
//   ref_cvt : cvt_uint32 / cvt_uint32_srgb (frame/common.h:31-48),
//             included unchanged (linear_to_srgb from the shim).
//
// Built by `make ref` in this directory into _ref/libref.so, only where the
// reference sources are present. Nothing in the product links this.
#include "ref_shim/vsnray_shim.h"

namespace visionaray {
#include "_ref/lcg_extract.h"
} // namespace visionaray

#include "renderer/DDA.h"
#include "frame/common.h"

using namespace visionaray;

extern "C" {

// n values of the stream seeded with (v0, v1); states[i] is the generator
// state after value i (may be null).
void ref_lcg(uint32_t v0, uint32_t v1, int n, float *values, uint32_t *states) {
  Random r(v0, v1);
  for (int i = 0; i < n; ++i) {
    values[i] = r();
    if (states) states[i] = r.state;
  }
}

// Cells visited by dda3 for the ray over a grid of dims cells spanning
// [lo, hi]: up to maxCells (cell id, t0, t1) records; returns the count.
int ref_dda(const float *ori, const float *dir, float tmin, float tmax, const int32_t *dims,
            const float *lo, const float *hi, int32_t *cells, float *t01, int maxCells) {
  ShimRay ray;
  ray.ori = vec3f(ori[0], ori[1], ori[2]);
  ray.dir = vec3f(dir[0], dir[1], dir[2]);
  ray.tmin = tmin;
  ray.tmax = tmax;
  const vec3i gd(dims[0], dims[1], dims[2]);
  box3f bounds;
  bounds.min = vec3f(lo[0], lo[1], lo[2]);
  bounds.max = vec3f(hi[0], hi[1], hi[2]);
  int n = 0;
  dda3(ray, gd, bounds, [&](size_t id, float t0, float t1) {
    if (n < maxCells) {
      cells[n] = (int32_t)id;
      t01[2 * n] = t0;
      t01[2 * n + 1] = t1;
    }
    ++n;
    return n < 1000000;
  });
  return n;
}

// rgba: n float4 colours; out: n packed RGBA8 words (srgb: colour through
// cvt_uint32_srgb, else cvt_uint32).
void ref_cvt(const float *rgba, int n, int srgb, uint32_t *out) {
  for (int i = 0; i < n; ++i) {
    const float4 v(rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2], rgba[4 * i + 3]);
    out[i] = srgb ? cvt_uint32_srgb(v) : cvt_uint32(v);
  }
}

} // extern "C"
