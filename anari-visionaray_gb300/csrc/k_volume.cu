// Volume and frame helper kernels: brick majorant grid and accumulation
// reset.
#include "kernels.h"

#include <float.h>

namespace vsr {
namespace {

// One warp per brick. Brick k along an axis covers normalized coordinates
// [k/G, (k+1)/G]; a trilinear sample there reads texels
// floor(k*N/G - 0.5) .. floor((k+1)*N/G - 0.5) + 1 (clamped), so their
// min/max bound every sample in the brick. The TF lookup is linear between
// bin centres, so the bins floor(lo*T-0.5) .. floor(hi*T-0.5)+1 bound its
// alpha. This keeps delta tracking unbiased (the majorant never undercuts
// the density) while replacing the reference's per-voxel rasterisation
// into a 16^3 grid (StructuredRegularField.cpp:95-127, GridAccel.cpp:69-108).
__global__ void kBrickMajorants(const float *__restrict__ field, int nx, int ny, int nz, int gx,
                                int gy, int gz, const float4 *__restrict__ tf, int tfSize,
                                float vrMin, float vrMax, float *out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int numBricks = gx * gy * gz;
  if (warp >= numBricks) return;
  const int kx = warp % gx, ky = (warp / gx) % gy, kz = warp / (gx * gy);
  auto range = [](int k, int n, int G, int &t0, int &t1) {
    double lo = floor(double(k) * n / G - 0.5);
    double hi = floor(double(k + 1) * n / G - 0.5) + 1.0;
    t0 = (int)fmin(fmax(lo, 0.0), double(n - 1));
    t1 = (int)fmin(fmax(hi, 0.0), double(n - 1));
  };
  int x0, x1, y0, y1, z0, z1;
  range(kx, nx, gx, x0, x1);
  range(ky, ny, gy, y0, y1);
  range(kz, nz, gz, z0, z1);
  const int ex = x1 - x0 + 1, ey = y1 - y0 + 1, ez = z1 - z0 + 1;
  const int total = ex * ey * ez;
  float mn = FLT_MAX, mx = -FLT_MAX;
  for (int i = lane; i < total; i += 32) {
    const int x = x0 + i % ex, y = y0 + (i / ex) % ey, z = z0 + i / (ex * ey);
    const float v = __ldg(field + ((size_t)z * ny + y) * nx + x);
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  const float lo = (mn - vrMin) / (vrMax - vrMin);
  const float hi = (mx - vrMin) / (vrMax - vrMin);
  int ilo = (int)fminf(fmaxf(floorf(lo * tfSize - 0.5f), -1.f), (float)tfSize);
  int ihi = (int)fminf(fmaxf(floorf(hi * tfSize - 0.5f), -1.f), (float)tfSize) + 1;
  ilo = min(max(ilo, 0), tfSize - 1);
  ihi = min(max(ihi, 0), tfSize - 1);
  float m = 0.f;
  for (int i = ilo + lane; i <= ihi; i += 32) m = fmaxf(m, tf[i].w);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) out[warp] = m;
}

__global__ void kFrameReset(float4 *accum, float *depth, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    if (accum) accum[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (depth) depth[i] = 1e31f;
  }
}

__global__ void kFillU32(uint32_t *p, uint32_t v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}

} // namespace

cudaError_t launchBrickMajorants(const float *field, const int dims[3], int brick,
                                 const float4 *tf, int tfSize, float vrMin, float vrMax,
                                 float *out, const int gdims[3], cudaStream_t stream) {
  (void)brick;
  const int numBricks = gdims[0] * gdims[1] * gdims[2];
  const int threads = 256;
  const int blocks = (numBricks * 32 + threads - 1) / threads;
  kBrickMajorants<<<blocks, threads, 0, stream>>>(field, dims[0], dims[1], dims[2], gdims[0],
                                                  gdims[1], gdims[2], tf, tfSize, vrMin, vrMax,
                                                  out);
  return cudaGetLastError();
}

cudaError_t launchFrameReset(float4 *accum, float *depth, size_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const int threads = 256;
  const int blocks = (int)((n + threads - 1) / threads < 152 * 16 ? (n + threads - 1) / threads
                                                                   : 152 * 16);
  kFrameReset<<<blocks, threads, 0, stream>>>(accum, depth, n);
  return cudaGetLastError();
}

cudaError_t launchFillU32(uint32_t *p, uint32_t value, size_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const int threads = 256;
  const size_t want = (n + threads - 1) / threads;
  const int blocks = (int)(want < 152 * 16 ? want : 152 * 16);
  kFillU32<<<blocks, threads, 0, stream>>>(p, value, n);
  return cudaGetLastError();
}

} // namespace vsr
