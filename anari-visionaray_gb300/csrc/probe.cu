// Probe entry points (libvsr_probe.so, a separate library that tests load):
// run single device functions of the renderer core on the GPU, so tests can
// compare them bit for bit with fixtures made from the reference's own code
// (LCG<4>, dda3, cvt_uint32). They call exactly the inline device functions
// the render kernels use (Rng, ddaWalk, packRGBA8 in render_common.cuh).
// Inputs and outputs are host arrays; each call allocates and frees its own
// device buffers and synchronizes. Every function returns a cudaError_t
// value (0 = success).
#include "render_common.cuh"

namespace {

using namespace vsr;

__global__ void kProbeLcg(uint32_t v0, uint32_t v1, int n, float *values, uint32_t *states) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  Rng r;
  r.init(v0, v1);
  for (int i = 0; i < n; ++i) {
    values[i] = r();
    states[i] = r.state;
  }
}

// One thread per ray: rays[8 i ..] = ori.xyz, dir.xyz, tmin, tmax.
__global__ void kProbeDda(const float *rays, int n, int gx, int gy, int gz, float3 blo, float3 bhi,
                          int maxCells, int *counts, int *cells, float *t01, uint32_t *errs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *r = rays + 8 * (size_t)i;
  int k = 0;
  uint32_t err = 0;
  int *c = cells + (size_t)i * maxCells;
  float *t = t01 + 2 * (size_t)i * maxCells;
  ddaWalk(f3(r[0], r[1], r[2]), f3(r[3], r[4], r[5]), r[6], r[7], blo, bhi, gx, gy, gz, err,
          [&](int id, float t0, float t1) -> bool {
            if (k < maxCells) {
              c[k] = id;
              t[2 * k] = t0;
              t[2 * k + 1] = t1;
            }
            ++k;
            return true;
          });
  counts[i] = k;
  errs[i] = err;
}

__global__ void kProbeCvt(const float4 *rgba, int n, int srgb, uint32_t *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = packRGBA8(rgba[i], srgb != 0);
}

// Streaming read of `bytes` (a multiple of 16) `repeats` times: every
// thread sums 16-byte loads of a grid-stride walk; one partial sum per block
// keeps the loads live. With a buffer that fits the L2 cache (e.g. 8 MiB)
// this measures the achievable L2 read bandwidth.
__global__ void kProbeRead(const float4 *buf, size_t n16, int repeats, float *sink) {
  float acc = 0.f;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int r = 0; r < repeats; ++r) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += 4 * stride) {
      float4 v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const size_t j = i + k * stride;
        v[k] = j < n16 ? __ldcg(buf + j) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) acc += v[k].x + v[k].y + v[k].z + v[k].w;
    }
  }
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    sink[blockIdx.x] = t;
  }
}

struct DevBuf {
  void *p = nullptr;
  cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes > 0 ? bytes : 4); }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

} // namespace

extern "C" {

// values[i] / states[i]: the i-th uniform of the stream seeded (v0, v1) and
// the generator state after it.
int vsrProbeLcg(uint32_t v0, uint32_t v1, int n, float *values, uint32_t *states) {
  if (n <= 0) return (int)cudaErrorInvalidValue;
  DevBuf dv, ds;
  cudaError_t e;
  if ((e = dv.alloc(n * sizeof(float))) || (e = ds.alloc(n * sizeof(uint32_t)))) return (int)e;
  kProbeLcg<<<1, 32>>>(v0, v1, n, (float *)dv.p, (uint32_t *)ds.p);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) return (int)e;
  if ((e = cudaMemcpy(values, dv.p, n * sizeof(float), cudaMemcpyDeviceToHost))) return (int)e;
  return (int)cudaMemcpy(states, ds.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
}

// n rays (8 floats each) walked over a grid of dims cells spanning [lo, hi];
// per ray: counts[i] cells visited, the first maxCells (id, t0, t1) records
// in cells[i * maxCells ..] and t01[2 i maxCells ..], errs[i] error bits.
int vsrProbeDda(const float *rays, int n, const int *dims, const float *lo, const float *hi,
                int maxCells, int *counts, int *cells, float *t01, uint32_t *errs) {
  if (n <= 0 || maxCells <= 0) return (int)cudaErrorInvalidValue;
  DevBuf dr, dc, dcl, dt, de;
  cudaError_t e;
  if ((e = dr.alloc(8 * sizeof(float) * n)) || (e = dc.alloc(sizeof(int) * n)) ||
      (e = dcl.alloc(sizeof(int) * (size_t)n * maxCells)) ||
      (e = dt.alloc(2 * sizeof(float) * (size_t)n * maxCells)) || (e = de.alloc(sizeof(uint32_t) * n)))
    return (int)e;
  if ((e = cudaMemcpy(dr.p, rays, 8 * sizeof(float) * n, cudaMemcpyHostToDevice))) return (int)e;
  kProbeDda<<<(n + 127) / 128, 128>>>((const float *)dr.p, n, dims[0], dims[1], dims[2],
                                      make_float3(lo[0], lo[1], lo[2]),
                                      make_float3(hi[0], hi[1], hi[2]), maxCells, (int *)dc.p,
                                      (int *)dcl.p, (float *)dt.p, (uint32_t *)de.p);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) return (int)e;
  if ((e = cudaMemcpy(counts, dc.p, sizeof(int) * n, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(cells, dcl.p, sizeof(int) * (size_t)n * maxCells, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(t01, dt.p, 2 * sizeof(float) * (size_t)n * maxCells, cudaMemcpyDeviceToHost)))
    return (int)e;
  return (int)cudaMemcpy(errs, de.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost);
}

// n float4 colours to packed RGBA8 words as the frame's UFIXED8 (srgb = 0)
// and sRGB8 (srgb = 1) colour formats store them.
int vsrProbeCvt(const float *rgba, int n, int srgb, uint32_t *out) {
  if (n <= 0) return (int)cudaErrorInvalidValue;
  DevBuf di, dout;
  cudaError_t e;
  if ((e = di.alloc(16 * (size_t)n)) || (e = dout.alloc(4 * (size_t)n))) return (int)e;
  if ((e = cudaMemcpy(di.p, rgba, 16 * (size_t)n, cudaMemcpyHostToDevice))) return (int)e;
  kProbeCvt<<<(n + 127) / 128, 128>>>((const float4 *)di.p, n, srgb, (uint32_t *)dout.p);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) return (int)e;
  return (int)cudaMemcpy(out, dout.p, 4 * (size_t)n, cudaMemcpyDeviceToHost);
}

// Enqueue kProbeRead on `stream` over the device buffer `buf` (`bytes`, a
// multiple of 16, 16-byte aligned) `repeats` times; `sink`: device floats,
// one per block of the grid (blocksPerSM x the SM count). Asynchronous.
int vsrProbeReadBandwidth(const void *buf, size_t bytes, int repeats, int blocksPerSM, float *sink,
                          void *stream) {
  if (!buf || !sink || bytes % 16 || ((uintptr_t)buf & 15) || repeats <= 0 || blocksPerSM <= 0)
    return (int)cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) ||
      (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)))
    return (int)e;
  kProbeRead<<<sms * blocksPerSM, 512, 0, (cudaStream_t)stream>>>((const float4 *)buf, bytes / 16,
                                                                   repeats, sink);
  return (int)cudaGetLastError();
}

// Bytes in use and reserved in the current device's default stream-ordered
// memory pool (the pool cudaMallocAsync draws from), for tests that check
// that an entry point allocates nothing.
int vsrProbeMemPoolUsage(uint64_t *used, uint64_t *reserved) {
  int dev = 0;
  cudaMemPool_t pool;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) || (e = cudaDeviceGetDefaultMemPool(&pool, dev))) return (int)e;
  unsigned long long u = 0, r = 0;  // the attributes are 64-bit counts
  if ((e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u)) ||
      (e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r)))
    return (int)e;
  *used = u;
  *reserved = r;
  return 0;
}

} // extern "C"
