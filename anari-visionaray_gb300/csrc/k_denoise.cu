// Denoiser kernels: a U-Net of 3x3 convolutions over bf16 activations in
// channel-blocked planes (actAt in kernels.h) with fp32 accumulation, its
// backward pass, and Adam.
//
// Convolutions are implicit GEMMs on the tensor cores (mma.sync m16n8k16
// bf16 -> fp32): the forward pass and the input gradient are one kernel
// (the input gradient is the forward convolution of the output gradient
// with the spatially flipped, channel-transposed weights), the weight
// gradient is a pixel-reduction GEMM split over pixel chunks. Tiles are
// staged in shared memory with cp.async (zero fill outside the image) and
// read into fragments with ldmatrix.
#include "kernels.h"

#include <cuda_bf16.h>
#include <stdint.h>

namespace vsr {
namespace {

typedef __nv_bfloat16 bf16;

// ------------------------------------------------------------ primitives
__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// 16-byte async copy; src_bytes = 0 fills the destination with zeros
__device__ __forceinline__ void cpAsync16(void *dst, const void *src, bool valid) {
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smemAddr(dst)),
               "l"(src), "r"(n));
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cpAsyncWait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void ldsm4(uint32_t (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smemAddr(p)));
}
__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smemAddr(p)));
}

// D (16x8 f32) += A (16x16 bf16, row) * B (16x8 bf16, col)
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ------------------------------------------------------ convolution (GEMM)
// CTA tile: 64 pixels x BN output channels (64, or 32 for layers of at most
// 32), k-step 16 (one tap, 16 input channels); 4 warps as 2 x 2, each 32 x
// BN/2 (2 x BN/16 mma tiles). Two stages.
constexpr int kBM = 64, kBK = 16;
constexpr int kRowA = kBK + 8;  // padded smem row (48 B): conflict-free ldmatrix

template <int BN>
__global__ void __launch_bounds__(128) kConv3x3(ConvArgs a) {
  constexpr int NT = BN / 16;  // n8 tiles per warp
  __shared__ __align__(128) bf16 As[2][kBM][kRowA];
  __shared__ __align__(128) bf16 Bs[2][BN][kRowA];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int P = a.N * a.H * a.W;
  const int pBase = blockIdx.x * kBM;
  const int nBase = blockIdx.y * BN;
  const int kChunks = a.Cin / kBK;  // per tap
  const int steps = 9 * kChunks;
  // this thread's loads: one 16-byte half-row of A and one of B
  const int lr = tid >> 1, lh = tid & 1;
  const int p = pBase + lr;
  int py = 0, px = 0, pn = 0;
  const bool pIn = p < P;
  if (pIn) {
    px = p % a.W;
    const int t = p / a.W;
    py = t % a.H;
    pn = t / a.H;
  }
  const int co = nBase + lr;
  auto load = [&](int stage, int step) {
    const int tap = step / kChunks, c0 = (step - tap * kChunks) * kBK + lh * 8;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int yy = py + dy, xx = px + dx;
    const bool ok = pIn && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
    const bf16 *src = a.x + (ok ? actAt(P, ((size_t)pn * a.H + yy) * a.W + xx, a.xOff + c0) : 0);
    cpAsync16(&As[stage][lr][lh * 8], src, ok);
    if (lr < BN) {
      const bool wok = co < a.Cout;
      const bf16 *wsrc = a.w + (wok ? ((size_t)co * 9 + tap) * a.Cin + c0 : 0);
      cpAsync16(&Bs[stage][lr][lh * 8], wsrc, wok);
    }
  };
  float acc[2][NT][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  load(0, 0);
  cpAsyncCommit();
  for (int s = 0; s < steps; ++s) {
    const int cur = s & 1;
    if (s + 1 < steps) load(cur ^ 1, s + 1);
    cpAsyncCommit();
    cpAsyncWait<1>();
    __syncthreads();
    uint32_t af[2][4], bfr[NT / 2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
      ldsm4(af[mt], &As[cur][wm * 32 + mt * 16 + (lane & 15)][(lane >> 4) * 8]);
#pragma unroll
    for (int np = 0; np < NT / 2; ++np)
      ldsm4(bfr[np], &Bs[cur][wn * (BN / 2) + np * 16 + (lane & 7) + (lane >> 4) * 8]
                        [((lane >> 3) & 1) * 8]);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
        mma16816(acc[mt][nt], af[mt], bfr[nt >> 1][(nt & 1) * 2], bfr[nt >> 1][(nt & 1) * 2 + 1]);
    __syncthreads();
  }
  // epilogue: bias, ReLU, mask of a previous ReLU, store; the biases of
  // this thread's columns are loaded once
  const int g = lane >> 2, t4 = lane & 3;
  float bias[NT][2];
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const int c = nBase + wn * (BN / 2) + nt * 8 + t4 * 2;
    bias[nt][0] = (a.bias && c < a.Cout) ? a.bias[c] : 0.f;
    bias[nt][1] = (a.bias && c + 1 < a.Cout) ? a.bias[c + 1] : 0.f;
  }
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int pp = pBase + wm * 32 + mt * 16 + g + half * 8;
      if (pp >= P) continue;
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int c = nBase + wn * (BN / 2) + nt * 8 + t4 * 2;
        float v0 = acc[mt][nt][half * 2] + bias[nt][0], v1 = acc[mt][nt][half * 2 + 1] + bias[nt][1];
        if (a.relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (a.resid) {
          const bf16 *r = a.resid + actAt(P, pp, c);  // c, c + 1 in one 8-channel block
          if (c < a.residN) v0 += __bfloat162float(r[0]);
          if (c + 1 < a.residN) v1 += __bfloat162float(r[1]);
        }
        if (a.mask) {
          const bf16 *m = a.mask + actAt(P, pp, a.maskOff + c);
          if (c < a.Cout && !(__bfloat162float(m[0]) > 0.f)) v0 = 0.f;
          if (c + 1 < a.Cout && !(__bfloat162float(m[1]) > 0.f)) v1 = 0.f;
        }
        if (a.yf) {  // fp32 output: NHWC
          const size_t o = (size_t)pp * a.yC + a.yOff + c;
          if (c < a.Cout) a.yf[o] = v0;
          if (c + 1 < a.Cout) a.yf[o + 1] = v1;
          continue;
        }
        const size_t o = actAt(P, pp, a.yOff + c);
        if (c + 1 < a.Cout) {
          *reinterpret_cast<__nv_bfloat162 *>(a.y + o) = __floats2bfloat162_rn(v0, v1);
        } else if (c < a.Cout) {
          a.y[o] = __float2bfloat16(v0);
        }
      }
    }
}

// ------------------------------------------------------- weight gradient
// dW[co][tap][ci] += sum over a chunk of pixels p of dY[p][co] * X[p + tap][ci]
// (M = 64 output channels, N = 64 input channels of one tap, K = pixels).
// Tiles are stored pixel-major as in memory; ldmatrix.trans turns them into
// the row-major A (co x p) and column-major B (p x ci) fragments.
constexpr int kRowW = 64 + 8;  // padded row of 64 channels (144 B)

__global__ void __launch_bounds__(128) kConvWgrad(WgradArgs a) {
  __shared__ __align__(128) bf16 Ds[2][kBK][kRowW];
  __shared__ __align__(128) bf16 Xs[2][kBK][kRowW];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int P = a.N * a.H * a.W;
  const int coBase = blockIdx.x * 64;
  const int tap = blockIdx.y % 9, ciBase = (blockIdx.y / 9) * 64;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int pStart = blockIdx.z * a.chunk;
  const int pEnd = min(P, pStart + a.chunk);
  const int steps = pEnd > pStart ? (pEnd - pStart + kBK - 1) / kBK : 0;
  // loads: 16 pixels x 64 channels = 128 x 16 B for each of Ds and Xs,
  // consecutive threads on consecutive pixels of one 8-channel block
  const int lr = tid & 15, lc = (tid >> 4) * 8;
  auto load = [&](int stage, int step) {
    const int p = pStart + step * kBK + lr;
    const bool pIn = p < pEnd;
    int px = 0, py = 0, pn = 0;
    if (pIn) {
      px = p % a.W;
      const int t = p / a.W;
      py = t % a.H;
      pn = t / a.H;
    }
    const bool dok = pIn && coBase + lc < a.Cout;
    cpAsync16(&Ds[stage][lr][lc], a.dy + (dok ? actAt(P, p, a.dyOff + coBase + lc) : 0), dok);
    const int yy = py + dy, xx = px + dx;
    const bool xok = pIn && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W && ciBase + lc < a.Cin;
    cpAsync16(&Xs[stage][lr][lc],
              a.x + (xok ? actAt(P, ((size_t)pn * a.H + yy) * a.W + xx, a.xOff + ciBase + lc) : 0),
              xok);
  };
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  if (steps > 0) {
    load(0, 0);
    cpAsyncCommit();
  }
  for (int s = 0; s < steps; ++s) {
    const int cur = s & 1;
    if (s + 1 < steps) load(cur ^ 1, s + 1);
    cpAsyncCommit();
    cpAsyncWait<1>();
    __syncthreads();
    uint32_t af[2][4], bfr[2][4];
    // A (m = co, k = pixel) from Ds[k][m]
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
      ldsm4t(af[mt],
             &Ds[cur][(lane & 7) + (lane >> 4) * 8][wm * 32 + mt * 16 + ((lane >> 3) & 1) * 8]);
    // B (k = pixel, n = ci) from Xs[k][n]
#pragma unroll
    for (int np = 0; np < 2; ++np)
      ldsm4t(bfr[np],
             &Xs[cur][(lane & 7) + ((lane >> 3) & 1) * 8][wn * 32 + np * 16 + (lane >> 4) * 8]);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < 4; ++nt)
        mma16816(acc[mt][nt], af[mt], bfr[nt >> 1][(nt & 1) * 2], bfr[nt >> 1][(nt & 1) * 2 + 1]);
    __syncthreads();
  }
  if (steps == 0) return;
  const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int c = coBase + wm * 32 + mt * 16 + g + half * 8;
      if (c >= a.Cout) continue;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int ci = ciBase + wn * 32 + nt * 8 + t4 * 2;
        float *dst = a.dw + ((size_t)c * 9 + tap) * a.Cin + ci;
        if (ci < a.Cin) atomicAdd(dst, acc[mt][nt][half * 2]);
        if (ci + 1 < a.Cin) atomicAdd(dst + 1, acc[mt][nt][half * 2 + 1]);
      }
    }
}

// db[c] += sum over pixels of dY[p][c]: one 8-channel block per blockIdx.y,
// 16 bytes per thread and pixel
__global__ void __launch_bounds__(256) kBiasGrad(const bf16 *dy, int dyOff, size_t P, float *db) {
  const int blk = blockIdx.y;
  const int c0 = dyOff + 8 * blk;
  float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < P;
       p += (size_t)gridDim.x * blockDim.x) {
    const uint4 v = *reinterpret_cast<const uint4 *>(dy + actAt(P, p, c0));
    const bf16 *e = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
    for (int k = 0; k < 8; ++k) s[k] += __bfloat162float(e[k]);
  }
  __shared__ float red[8][256];
#pragma unroll
  for (int k = 0; k < 8; ++k) red[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
#pragma unroll
      for (int k = 0; k < 8; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 8) atomicAdd(db + 8 * blk + threadIdx.x, red[threadIdx.x][0]);
}

// --------------------------------------------------- layout and elementwise
// Every thread below handles one 8-channel block of one pixel (16 bytes).
__device__ __forceinline__ uint4 ld16(const bf16 *p) { return *reinterpret_cast<const uint4 *>(p); }
__device__ __forceinline__ void st16(bf16 *p, uint4 v) { *reinterpret_cast<uint4 *>(p) = v; }
__device__ __forceinline__ float el(const uint4 &v, int k) {
  return __bfloat162float(reinterpret_cast<const bf16 *>(&v)[k]);
}
__device__ __forceinline__ void setEl(uint4 &v, int k, float f) {
  reinterpret_cast<bf16 *>(&v)[k] = __float2bfloat16(f);
}

// 2x2 max pooling (H, W even)
__global__ void kMaxPool(const bf16 *x, int C, int N, int H, int W, bf16 *y) {
  const int Ho = H / 2, Wo = W / 2;
  const size_t Pi = (size_t)N * H * W, Po = (size_t)N * Ho * Wo;
  const size_t n = Po * (C / 8);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / Po);
    const size_t po = i % Po;
    const int xo = (int)(po % Wo);
    const size_t q = po / Wo;
    const int yo = (int)(q % Ho);
    const int b = (int)(q / Ho);
    const size_t p0 = ((size_t)b * H + 2 * yo) * W + 2 * xo;
    const size_t pin[4] = {p0, p0 + 1, p0 + W, p0 + W + 1};
    uint4 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = ld16(x + actAt(Pi, pin[k], 8 * blk));
    uint4 o;
#pragma unroll
    for (int e = 0; e < 8; ++e)
      setEl(o, e, fmaxf(fmaxf(el(v[0], e), el(v[1], e)), fmaxf(el(v[2], e), el(v[3], e))));
    st16(y + actAt(Po, po, 8 * blk), o);
  }
}

// gradient of kMaxPool: to the first maximum of each 2x2 window, zero
// elsewhere; with mask, also zero where the mask is <= 0
__global__ void kMaxPoolGrad(const bf16 *x, const bf16 *dy, int C, int N, int H, int W,
                             const bf16 *mask, bf16 *dx) {
  const int Ho = H / 2, Wo = W / 2;
  const size_t Pi = (size_t)N * H * W, Po = (size_t)N * Ho * Wo;
  const size_t n = Po * (C / 8);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / Po);
    const size_t po = i % Po;
    const int xo = (int)(po % Wo);
    const size_t q = po / Wo;
    const int yo = (int)(q % Ho);
    const int b = (int)(q / Ho);
    const size_t p0 = ((size_t)b * H + 2 * yo) * W + 2 * xo;
    const size_t pin[4] = {p0, p0 + 1, p0 + W, p0 + W + 1};
    uint4 v[4], m[4], d[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = ld16(x + actAt(Pi, pin[k], 8 * blk));
      if (mask) m[k] = ld16(mask + actAt(Pi, pin[k], 8 * blk));
    }
    const uint4 g = ld16(dy + actAt(Po, po, 8 * blk));
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      int arg = 0;
      float mx = el(v[0], e);
      for (int k = 1; k < 4; ++k) {
        const float f = el(v[k], e);
        if (f > mx) {
          mx = f;
          arg = k;
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        float f = k == arg ? el(g, e) : 0.f;
        if (mask && !(el(m[k], e) > 0.f)) f = 0.f;
        setEl(d[k], e, f);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) st16(dx + actAt(Pi, pin[k], 8 * blk), d[k]);
  }
}

// nearest 2x upsampling of x (C channels, N x H x W) into channels
// [yOff, yOff + C) of y (N x 2H x 2W)
__global__ void kUpsample(const bf16 *x, int C, int N, int H, int W, bf16 *y, int yOff) {
  const size_t Pi = (size_t)N * H * W, Po = 4 * Pi;
  const size_t n = Po * (C / 8);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / Po);
    const size_t po = i % Po;
    const int xo = (int)(po % (2 * W));
    const size_t q = po / (2 * W);
    const int yo = (int)(q % (2 * H));
    const int b = (int)(q / (2 * H));
    const size_t pi = ((size_t)b * H + yo / 2) * W + xo / 2;
    st16(y + actAt(Po, po, yOff + 8 * blk), ld16(x + actAt(Pi, pi, 8 * blk)));
  }
}

// gradient of kUpsample: sum of the four children; with mask, zero where
// the mask (the upsampled input) is <= 0
__global__ void kUpsampleGrad(const bf16 *dy, int dyOff, int C, int N, int H, int W,
                              const bf16 *mask, bf16 *dx) {
  const size_t Pi = (size_t)N * H * W, Po = 4 * Pi;
  const size_t n = Pi * (C / 8);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / Pi);
    const size_t pi = i % Pi;
    const int x = (int)(pi % W);
    const size_t q = pi / W;
    const int yv = (int)(q % H);
    const int b = (int)(q / H);
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < 4; ++k) {
      const size_t po = ((size_t)b * 2 * H + 2 * yv + (k >> 1)) * 2 * W + 2 * x + (k & 1);
      const uint4 v = ld16(dy + actAt(Po, po, dyOff + 8 * blk));
#pragma unroll
      for (int e = 0; e < 8; ++e) s[e] += el(v, e);
    }
    uint4 m, o;
    if (mask) m = ld16(mask + actAt(Pi, pi, 8 * blk));
#pragma unroll
    for (int e = 0; e < 8; ++e) setEl(o, e, (mask && !(el(m, e) > 0.f)) ? 0.f : s[e]);
    st16(dx + actAt(Pi, pi, 8 * blk), o);
  }
}

// copy C channels: y[:, yOff:yOff+C] = x[:, xOff:xOff+C]; with add, y += x
__global__ void kCopyChannels(const bf16 *x, int xOff, bf16 *y, int yOff, int C, size_t P,
                              int add) {
  const size_t n = P * (C / 8);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / P);
    const size_t p = i % P;
    uint4 v = ld16(x + actAt(P, p, xOff + 8 * blk));
    bf16 *d = y + actAt(P, p, yOff + 8 * blk);
    if (add) {
      const uint4 w = ld16(d);
#pragma unroll
      for (int e = 0; e < 8; ++e) setEl(v, e, el(v, e) + el(w, e));
    }
    st16(d, v);
  }
}

// ReLU backward in place: d *= (post > 0)
__global__ void kReluMask(bf16 *d, int dOff, const bf16 *post, int pOff, int C, size_t P) {
  const size_t n = P * (C / 8);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / P);
    const size_t p = i % P;
    bf16 *dp = d + actAt(P, p, dOff + 8 * blk);
    uint4 v = ld16(dp);
    const uint4 m = ld16(post + actAt(P, p, pOff + 8 * blk));
#pragma unroll
    for (int e = 0; e < 8; ++e)
      if (!(el(m, e) > 0.f)) setEl(v, e, 0.f);
    st16(dp, v);
  }
}

// NHWC (C channels per pixel) -> channel-blocked planes
__global__ void kToBlocked(const bf16 *x, int C, size_t P, bf16 *y) {
  const size_t n = P * (C / 8);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / P);
    const size_t p = i % P;
    st16(y + actAt(P, p, 8 * blk), ld16(x + p * C + 8 * blk));
  }
}

// packed weights for kConv3x3Ws: [nTile][stage][tap][chunk 4][N][8]
__global__ void kPackConvWeights(const bf16 *w, int Cin, int Cout, int N, int stages, size_t n,
                                 bf16 *out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(i & 7);
    size_t q = i >> 3;
    const int co = (int)(q % N);
    q /= N;
    const int chunk = (int)(q % 4);
    q /= 4;
    const int tap = (int)(q % 9);
    q /= 9;
    const int st = (int)(q % stages);
    const int nt = (int)(q / stages);
    const int cog = nt * N + co, ci = st * 32 + chunk * 8 + e;
    out[i] = (cog < Cout && ci < Cin) ? w[((size_t)cog * 9 + tap) * Cin + ci] : __float2bfloat16(0.f);
  }
}

// L1 loss between the first C channels of the output (fp32 log(1 + colour),
// oC channels per pixel) and log(1 + target colour) (tC floats per pixel,
// linear colour), and its gradient (sign / count) in bf16 in blocked planes
// of gC channels (the others are left as they are)
__global__ void kL1(const float *out, int oC, const float *target, int tC, int C, size_t P,
                    bf16 *grad, int gC, float *loss) {
  __shared__ float red[256];
  const size_t n = P * C;
  float s = 0.f;
  const float inv = 1.f / (float)n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t p = i / C;
    const int c = (int)(i % C);
    const float d = out[p * oC + c] - log1pf(fmaxf(target[p * tC + c], 0.f));
    s += fabsf(d);
    grad[actAt(P, p, c)] = __float2bfloat16(d > 0.f ? inv : (d < 0.f ? -inv : 0.f));
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0 && loss) atomicAdd(loss, red[0] * inv);
}

// Adam (Kingma & Ba 2015) on fp32 master weights; writes the bf16 copy, and
// for convolution weights the flipped, transposed copy the input gradient
// uses: wt[ci][tap'][co] = w[co][8 - tap'][ci].
__global__ void kAdam(float *w, float *m, float *v, const float *g, size_t n, float lr, float b1,
                      float b2, float eps, float c1, float c2, bf16 *wb, bf16 *wt, int Cin,
                      int CoutT) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
    if (wt) {
      const int ci = (int)(i % Cin);
      const int tap = (int)((i / Cin) % 9);
      const int co = (int)(i / ((size_t)Cin * 9));
      wt[((size_t)ci * 9 + (8 - tap)) * CoutT + co] = __float2bfloat16(wi);
    }
  }
}

// Network input from a frame: log(1 + colour), albedo, normal (as stored),
// depth mapped to [0, 1) by d / (1 + d) (0 for "no hit"), the noise level:
// log(1 + standard error of the mean luminance) from the variance channel
// (0 without it) and 1 / sqrt(samples per pixel), zero padding to xC
// channels. The network image is Wp x Hp (multiples of 8); pixels outside
// the frame are zero.
__global__ void kDenoiseInput(const float4 *color, const float *albedo, const float *normal,
                              const float *depth, const float *var, float invSqrtN, int W, int H,
                              int Wp, int Hp, bf16 *x, int xC) {
  const size_t np = (size_t)Wp * Hp;
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < np;
       j += (size_t)gridDim.x * blockDim.x) {
    const int px = (int)(j % Wp), py = (int)(j / Wp);
    if (px >= W || py >= H) {
      for (int k = 0; k < xC; k += 8) *reinterpret_cast<uint4 *>(x + j * xC + k) = make_uint4(0, 0, 0, 0);
      continue;
    }
    const size_t i = (size_t)py * W + px;
    float f[16];
    const float4 c = color[i];
    f[0] = log1pf(fmaxf(c.x, 0.f));
    f[1] = log1pf(fmaxf(c.y, 0.f));
    f[2] = log1pf(fmaxf(c.z, 0.f));
    for (int k = 0; k < 3; ++k) f[3 + k] = albedo ? albedo[3 * i + k] : 0.f;
    for (int k = 0; k < 3; ++k) f[6 + k] = normal ? normal[3 * i + k] : 0.f;
    const float d = depth ? depth[i] : 1e31f;
    f[9] = d < 1e30f ? d / (1.f + d) : 0.f;
    const float v = var ? var[i] : 0.f;
    f[10] = v > 0.f && v < 1e30f ? log1pf(sqrtf(v)) : 0.f;
    f[11] = invSqrtN;
    for (int k = 12; k < 16; ++k) f[k] = 0.f;
    // 16-byte stores of 8 channels
    for (int k = 0; k < xC; k += 8) {
      __nv_bfloat162 h[4];
#pragma unroll
      for (int e = 0; e < 4; ++e)
        h[e] = k < 16 ? __floats2bfloat162_rn(f[k + 2 * e], f[k + 2 * e + 1])
                      : __floats2bfloat162_rn(0.f, 0.f);
      *reinterpret_cast<uint4 *>(x + j * xC + k) = *reinterpret_cast<const uint4 *>(h);
    }
  }
}

// Denoised colour = exp(output) - 1, and the variance gate: a pixel keeps
// the denoised value if its residual to the accumulated mean is within
// `k` standard errors of that mean (plus an absolute floor), else it keeps
// the mean and is marked for more samples.
__global__ void kDenoiseOutput(const float *out, int oC, int W, int H, int Wp, const float4 *mean,
                               const float *var, float k, float floorAbs, float4 *result,
                               uint8_t *retry, unsigned *numRetry) {
  const int n = W * H;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float *o = out + ((size_t)(i / W) * Wp + i % W) * oC;
    float4 d = make_float4(fmaxf(expm1f(o[0]), 0.f), fmaxf(expm1f(o[1]), 0.f),
                           fmaxf(expm1f(o[2]), 0.f), 1.f);
    bool keep = true;
    if (var && mean) {
      const float4 m = mean[i];
      const float lm = 0.3f * m.x + 0.59f * m.y + 0.11f * m.z;
      const float ld = 0.3f * d.x + 0.59f * d.y + 0.11f * d.z;
      keep = fabsf(ld - lm) <= k * sqrtf(fmaxf(var[i], 0.f)) + floorAbs;
    }
    if (result) result[i] = keep ? d : (mean ? mean[i] : d);
    if (retry) retry[i] = keep ? 0 : 1;
    if (!keep && numRetry) atomicAdd(numRetry, 1u);
  }
}

int gridFor(size_t n, int threads = 256) {
  const size_t b = (n + threads - 1) / threads;
  return (int)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

}  // namespace

cudaError_t launchConv3x3(const ConvArgs &a, cudaStream_t s) {
  if (a.Cin % 16 || a.Cout <= 0 || a.xC % 8 || a.xOff % 8 || a.x2 || a.split || a.up)
    return cudaErrorInvalidValue;
  const int P = a.N * a.H * a.W;
  if (a.Cout <= 32) {
    kConv3x3<32><<<dim3((P + kBM - 1) / kBM, 1), 128, 0, s>>>(a);
  } else {
    kConv3x3<64><<<dim3((P + kBM - 1) / kBM, (a.Cout + 63) / 64), 128, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launchConvWgrad(const WgradArgs &a, cudaStream_t s) {
  if (a.Cin % 8 || a.Cout % 8 || a.chunk <= 0 || a.dyC % 8 || a.dyOff % 8 || a.xC % 8 || a.xOff % 8)
    return cudaErrorInvalidValue;
  const int P = a.N * a.H * a.W;
  dim3 grid((a.Cout + 63) / 64, 9 * ((a.Cin + 63) / 64), (P + a.chunk - 1) / a.chunk);
  kConvWgrad<<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// The channel-count arguments of views (dyC, yC, ...) only take part in the
// checks: in blocked planes a view's address depends on its pixel count and
// first channel.
static bool blocks8(int C, int off) { return C > 0 && C % 8 == 0 && off % 8 == 0; }

cudaError_t launchBiasGrad(const __nv_bfloat16 *dy, int dyC, int dyOff, int C, int P, float *db,
                           cudaStream_t s) {
  if (!blocks8(C, dyOff) || dyOff + C > dyC) return cudaErrorInvalidValue;
  dim3 grid(min(256, (P + 255) / 256), C / 8);
  kBiasGrad<<<grid, 256, 0, s>>>(dy, dyOff, (size_t)P, db);
  return cudaGetLastError();
}

cudaError_t launchMaxPool(const __nv_bfloat16 *x, int C, int N, int H, int W, __nv_bfloat16 *y,
                          cudaStream_t s) {
  if (!blocks8(C, 0) || H % 2 || W % 2) return cudaErrorInvalidValue;
  kMaxPool<<<gridFor((size_t)N * (H / 2) * (W / 2) * (C / 8)), 256, 0, s>>>(x, C, N, H, W, y);
  return cudaGetLastError();
}

cudaError_t launchMaxPoolGrad(const __nv_bfloat16 *x, const __nv_bfloat16 *dy, int C, int N, int H,
                              int W, const __nv_bfloat16 *mask, __nv_bfloat16 *dx, cudaStream_t s) {
  if (!blocks8(C, 0) || H % 2 || W % 2) return cudaErrorInvalidValue;
  kMaxPoolGrad<<<gridFor((size_t)N * (H / 2) * (W / 2) * (C / 8)), 256, 0, s>>>(x, dy, C, N, H, W,
                                                                              mask, dx);
  return cudaGetLastError();
}

cudaError_t launchUpsample(const __nv_bfloat16 *x, int C, int N, int H, int W, __nv_bfloat16 *y,
                           int yC, int yOff, cudaStream_t s) {
  if (!blocks8(C, yOff) || yOff + C > yC) return cudaErrorInvalidValue;
  kUpsample<<<gridFor((size_t)N * 4 * H * W * (C / 8)), 256, 0, s>>>(x, C, N, H, W, y, yOff);
  return cudaGetLastError();
}

cudaError_t launchUpsampleGrad(const __nv_bfloat16 *dy, int dyC, int dyOff, int C, int N, int H,
                               int W, const __nv_bfloat16 *mask, __nv_bfloat16 *dx, cudaStream_t s) {
  if (!blocks8(C, dyOff) || dyOff + C > dyC) return cudaErrorInvalidValue;
  kUpsampleGrad<<<gridFor((size_t)N * H * W * (C / 8)), 256, 0, s>>>(dy, dyOff, C, N, H, W, mask,
                                                                   dx);
  return cudaGetLastError();
}

cudaError_t launchCopyChannels(const __nv_bfloat16 *x, int xC, int xOff, __nv_bfloat16 *y, int yC,
                               int yOff, int C, size_t P, int add, cudaStream_t s) {
  if (!blocks8(C, xOff) || !blocks8(C, yOff) || xOff + C > xC || yOff + C > yC)
    return cudaErrorInvalidValue;
  kCopyChannels<<<gridFor(P * (C / 8)), 256, 0, s>>>(x, xOff, y, yOff, C, P, add);
  return cudaGetLastError();
}

cudaError_t launchReluMask(__nv_bfloat16 *d, int dC, int dOff, const __nv_bfloat16 *post, int pC,
                           int pOff, int C, size_t P, cudaStream_t s) {
  if (!blocks8(C, dOff) || !blocks8(C, pOff) || dOff + C > dC || pOff + C > pC)
    return cudaErrorInvalidValue;
  kReluMask<<<gridFor(P * (C / 8)), 256, 0, s>>>(d, dOff, post, pOff, C, P);
  return cudaGetLastError();
}

cudaError_t launchToBlocked(const __nv_bfloat16 *x, int C, size_t P, __nv_bfloat16 *y,
                            cudaStream_t s) {
  if (!blocks8(C, 0)) return cudaErrorInvalidValue;
  kToBlocked<<<gridFor(P * (C / 8)), 256, 0, s>>>(x, C, P, y);
  return cudaGetLastError();
}

size_t packedConvWeights(int Cin, int Cout) {
  const int N = Cout <= 32 ? 32 : 64;
  const size_t nTiles = (size_t)(Cout + N - 1) / N, stages = (size_t)(Cin + 31) / 32;
  return nTiles * stages * 9 * 4 * N * 8;
}

cudaError_t launchPackConvWeights(const __nv_bfloat16 *w, int Cin, int Cout, __nv_bfloat16 *packed,
                                  cudaStream_t s) {
  if (Cin <= 0 || Cout <= 0 || Cin % 16) return cudaErrorInvalidValue;
  const int N = Cout <= 32 ? 32 : 64;
  const size_t n = packedConvWeights(Cin, Cout);
  kPackConvWeights<<<gridFor(n), 256, 0, s>>>(w, Cin, Cout, N, (Cin + 31) / 32, n, packed);
  return cudaGetLastError();
}

cudaError_t launchL1(const float *out, int oC, const float *target, int tC, int C, size_t P,
                     __nv_bfloat16 *grad, int gC, float *loss, cudaStream_t s) {
  kL1<<<gridFor(P * C), 256, 0, s>>>(out, oC, target, tC, C, P, grad, gC, loss);
  return cudaGetLastError();
}

cudaError_t launchAdam(float *w, float *m, float *v, const float *g, size_t n, float lr, float b1,
                       float b2, float eps, int step, __nv_bfloat16 *wb, __nv_bfloat16 *wt, int Cin,
                       int CoutT, cudaStream_t s) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  kAdam<<<gridFor(n), 256, 0, s>>>(w, m, v, g, n, lr, b1, b2, eps, c1, c2, wb, wt, Cin, CoutT);
  return cudaGetLastError();
}

cudaError_t launchDenoiseInput(const float4 *color, const float *albedo, const float *normal,
                               const float *depth, const float *var, float invSqrtN, int W, int H,
                               int Wp, int Hp, __nv_bfloat16 *x, int xC, cudaStream_t s) {
  kDenoiseInput<<<gridFor((size_t)Wp * Hp), 256, 0, s>>>(color, albedo, normal, depth, var,
                                                         invSqrtN, W, H, Wp, Hp, x, xC);
  return cudaGetLastError();
}

cudaError_t launchDenoiseOutput(const float *out, int oC, int W, int H, int Wp, const float4 *mean,
                                const float *var, float k, float floorAbs, float4 *result,
                                uint8_t *retry, unsigned *numRetry, cudaStream_t s) {
  kDenoiseOutput<<<gridFor((size_t)W * H), 256, 0, s>>>(out, oC, W, H, Wp, mean, var, k, floorAbs,
                                                        result, retry, numRetry);
  return cudaGetLastError();
}

}  // namespace vsr
