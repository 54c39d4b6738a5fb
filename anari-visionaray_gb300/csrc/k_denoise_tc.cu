// The denoiser's 3x3 convolution on the 5th-generation tensor cores:
// tcgen05.mma (kind::f16, bf16 x bf16 -> fp32) with the accumulators in
// tensor memory.
//
// A CTA computes a tile of kR = 4 image rows x 128 pixels (tensor-core M =
// the 128 pixels of one row) x N output channels (64, or 32 for narrow
// layers), with one accumulator of 128 lanes x N columns per row. It walks
// the input channels in groups of 32 (the stage). For each stage it stages
// the group's input halo, (kR + 2) rows x 130 pixels, once in shared memory,
// plus the weights of all nine taps for the N output channels. Each tap is
// then a shifted view of the halo. The A operand of output row r and tap
// (dy, dx) starts at halo row r + dy + 1, column dx + 1. The MMAs read each
// staged input value up to 9 x kR times, while global memory and L2 deliver
// it (kR + 2) / kR times.
//
// Shared-memory layout (the tensor core's no-swizzle K-major form, 16-byte
// rows, core matrices of 8 rows):
//   halo     [chunk (8 channels)][halo row][halo column, padded to kHX][16 B]
//            8 consecutive pixels of a row form a core matrix (128 B);
//            stride between 8-pixel groups (SBO) 128 B, between the two
//            channel chunks of a K = 16 step (LBO) one chunk plane
//   weights  [tap][chunk][output channel][16 B]
//            SBO 128 B (8 output channels), LBO N x 16 B (next chunk)
// The halo row is padded to kHX = 131 entries so that the four chunk planes
// start in different banks, which keeps the staging writes conflict-free.
//
// One thread issues a stage's MMAs (kR x 9 x 2) and commits them to an
// mbarrier. The next stage's loads wait for that commit. Two or three CTAs
// share an SM, so one CTA's loads overlap another's MMAs. The epilogue reads
// the accumulators with tcgen05.ld (warp w: pixels 32w..32w+31 of the tile
// row, one pixel per thread) and applies bias, ReLU, the residual and the
// mask of a previous ReLU, in the same order and with the same results as
// kConv3x3. Activations are channel-blocked planes (actAt, kernels.h): a
// warp's halo loads and output stores cover contiguous rows of one block.
//
// The input can be the concatenation of two tensors, the first one at half
// resolution (a U-Net decoder's upsampled coarse level and its skip
// connection): each 32-channel group is read from the tensor that holds it,
// so neither the upsampled tensor nor the concatenation is written out.
//
// Every mbarrier wait is bounded (one second); a wait that runs out sets the
// error word, and the CTA still waits (bounded) for its MMAs and releases its
// tensor memory before it returns.
#include "kernels.h"

#include <cuda_bf16.h>
#include <stdint.h>

namespace vsr {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kR = 4;          // output rows per CTA
constexpr int kTX = 128;       // output pixels per row (tensor-core M)
constexpr int kHY = kR + 2;    // halo rows
constexpr int kHXUsed = kTX + 2;
constexpr int kHX = 131;       // halo row pitch in 16-byte entries
constexpr int kChunks = 4;     // 8-channel chunks per stage (32 channels)
constexpr int kPlane = kHY * kHX * 16;  // bytes of one chunk plane of the halo
constexpr int kHaloBytes = kChunks * kPlane;
constexpr uint32_t kSpinLimit = 1u << 26;
constexpr uint64_t kWaitNs = 1000000000ull;  // one second

template <int N>
__host__ __device__ constexpr int weightBytes() {
  return 9 * kChunks * N * 16;
}
template <int N>
__host__ __device__ constexpr int smemBytes() {
  return kHaloBytes + weightBytes<N>() + 128;
}

__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cpAsync16(uint32_t dst, const void *src, bool valid) {
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}

// shared-memory matrix descriptor: start, leading and stride byte offsets
// (all in 16-byte units), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3fff);
  d |= (uint64_t)((lbo >> 4) & 0x3fff) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3fff) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N and M
__host__ __device__ constexpr uint32_t instrDesc(int n, int m) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint64_t globalNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

// true once the phase of the given parity has completed; false after a
// second (or kSpinLimit polls)
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = globalNs();
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 255) == 255 && globalNs() - t0 > kWaitNs) return false;
  }
  return false;
}

// Thread 0 waits; the outcome reaches the whole block through shared
// memory, so that every thread takes the same path around the barriers.
__device__ __forceinline__ bool blockWait(uint32_t bar, uint32_t parity, volatile int *flag) {
  if (threadIdx.x == 0) *flag = mbarWait(bar, parity) ? 1 : 0;
  __syncthreads();
  const bool ok = *flag != 0;
  __syncthreads();  // the flag is written again by the next wait
  return ok;
}

template <int N>
__global__ void __launch_bounds__(128) kConv3x3Tc(ConvArgs a, int tilesX, int tilesY, unsigned *error) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *sHalo = smem;
  uint8_t *sW = smem + kHaloBytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(sW + weightBytes<N>());
  uint32_t &tmemBase = *reinterpret_cast<uint32_t *>(bar + 1);
  volatile int *waitFlag = reinterpret_cast<volatile int *>(bar + 2);
  constexpr int kCols = kR * N;  // tensor-memory columns: 128 or 256
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int t = blockIdx.x;
  const int tx = t % tilesX;
  t /= tilesX;
  const int ty = t % tilesY;
  const int n = t / tilesY;
  const int x0 = tx * kTX, y0 = ty * kR;
  const int nBase = blockIdx.y * N;
  const int stages = (a.Cin + 8 * kChunks - 1) / (8 * kChunks);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smemAddr(&tmemBase)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smemAddr(bar)));
    // a barrier nothing arrives on, waited on only by the timeout test
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smemAddr(bar + 3)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = tmemBase;
  const uint32_t haloBase = smemAddr(sHalo), wBase = smemAddr(sW);
  bool ok = true;
  int issued = 0;  // stages whose MMAs were committed
  // timeout test: nothing is in flight yet when this wait runs out
  if (a.testStall) ok = blockWait(smemAddr(bar + 3), 0, waitFlag);

  for (int s = 0; ok && s < stages; ++s) {
    if (s > 0) {
      ok = blockWait(smemAddr(bar), (s - 1) & 1, waitFlag);  // the MMAs of stage s - 1
      if (!ok) break;
    }
    const int c0 = s * 8 * kChunks;
    const int chunks = min(kChunks, (a.Cin - c0) / 8);  // 4, or 2 for a last group of 16
    // this group's source: x (upsampled or not) or the second input x2
    const bool second = a.split > 0 && c0 >= a.split;
    const bf16 *srcBase = second ? a.x2 : a.x;
    const int srcC = second ? a.x2C : a.xC;
    const int srcOff = second ? a.x2Off + c0 - a.split : a.xOff + c0;
    const int sh = (!second && a.up) ? 1 : 0;
    const int srcH = a.H >> sh, srcW = a.W >> sh;
    const size_t srcP = (size_t)a.N * srcH * srcW;
    // the halo: pixel fastest, so that a warp reads a row of one 8-channel
    // block (contiguous in blocked planes)
    const int haloEntries = chunks * kHY * kHXUsed;
    for (int i = tid; i < haloEntries; i += 128) {
      const int hx = i % kHXUsed;
      const int r = i / kHXUsed;
      const int c = r % chunks, hy = r / chunks;
      const int y = y0 - 1 + hy, x = x0 - 1 + hx;
      const bool in = y >= 0 && y < a.H && x >= 0 && x < a.W;
      const size_t pix = ((size_t)n * srcH + (y >> sh)) * srcW + (x >> sh);
      const bf16 *src = srcBase + (in ? actAt(srcP, pix, srcOff + 8 * c) : 0);
      cpAsync16(haloBase + (uint32_t)(c * kPlane + (hy * kHX + hx) * 16), src, in);
    }
    // the weights of the nine taps
    const int wEntries = 9 * chunks * N;
    for (int i = tid; i < wEntries; i += 128) {
      const int c = i % chunks;
      const int r = i / chunks;
      const int tap = r % 9, co = r / 9;
      const bool in = nBase + co < a.Cout;
      const bf16 *src = a.w + (in ? ((size_t)(nBase + co) * 9 + tap) * a.Cin + c0 + 8 * c : 0);
      cpAsync16(wBase + (uint32_t)(((tap * chunks + c) * N + co) * 16), src, in);
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
    // the staged operands, written through the generic proxy, become
    // visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;\n" ::);
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      constexpr uint32_t idesc = instrDesc(N, kTX);
#pragma unroll 1
      for (int r = 0; r < kR; ++r) {
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap) {
          const uint32_t aRow = haloBase + (uint32_t)(((r + tap / 3) * kHX + tap % 3) * 16);
#pragma unroll 2
          for (int k = 0; k < chunks; k += 2) {
            const uint64_t da = smemDesc(aRow + (uint32_t)(k * kPlane), kPlane, 128);
            const uint64_t db = smemDesc(wBase + (uint32_t)((tap * chunks + k) * N * 16), N * 16, 128);
            const uint32_t accum = (s > 0 || tap > 0 || k > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                    tmem + (uint32_t)(r * N)),
                "l"(da), "l"(db), "r"(idesc), "r"(accum));
          }
        }
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              smemAddr(bar)));
    }
    issued = s + 1;
  }
  // the last commit covers all earlier MMAs
  if (ok && issued > 0) ok = blockWait(smemAddr(bar), (issued - 1) & 1, waitFlag);
  if (!ok) {
    if (tid == 0) atomicOr(error, 1u);
    // before the tensor memory is released: wait (bounded) for the last
    // commit once more
    if (issued > 0) blockWait(smemAddr(bar), (issued - 1) & 1, waitFlag);
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (ok) {
    const int x = x0 + warp * 32 + lane;
    const size_t P = (size_t)a.N * a.H * a.W;
    // columns outside, rows inside: a column group's biases are loaded once
#pragma unroll
    for (int c32 = 0; c32 < N / 32; ++c32) {
      float bias[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const int c = nBase + c32 * 32 + k;
        bias[k] = (a.bias && c < a.Cout) ? __ldg(a.bias + c) : 0.f;
      }
#pragma unroll 1
      for (int r = 0; r < kR; ++r) {
        const int y = y0 + r;
        const bool pixIn = x < a.W && y < a.H;
        const size_t pp = ((size_t)n * a.H + y) * a.W + x;
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
            "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
              "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
              "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
              "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(r * N + c32 * 32)));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
        if (!pixIn) continue;
#pragma unroll
        for (int g = 0; g < 32; g += 8) {
          const int cb = nBase + c32 * 32 + g;
          if (cb >= a.Cout) break;
          float o[8];
          // 16-byte blocks of the residual and the mask (blocked planes)
          uint4 rv = make_uint4(0, 0, 0, 0), mv = make_uint4(0, 0, 0, 0);
          if (a.resid && cb < a.residN) rv = *reinterpret_cast<const uint4 *>(a.resid + actAt(P, pp, cb));
          if (a.mask) mv = *reinterpret_cast<const uint4 *>(a.mask + actAt(P, pp, a.maskOff + cb));
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int c = cb + k;
            float val = __uint_as_float(v[g + k]);
            val += bias[g + k];
            if (a.relu) val = fmaxf(val, 0.f);
            if (a.resid && c < a.residN)
              val += __bfloat162float(reinterpret_cast<const bf16 *>(&rv)[k]);
            if (a.mask && !(__bfloat162float(reinterpret_cast<const bf16 *>(&mv)[k]) > 0.f))
              val = 0.f;
            o[k] = val;
          }
          if (a.yf) {  // fp32 output: NHWC
            const size_t ob = pp * a.yC + a.yOff + cb;
#pragma unroll
            for (int k = 0; k < 8; ++k)
              if (cb + k < a.Cout) a.yf[ob + k] = o[k];
          } else {
            // Cout is a multiple of 16: whole 8-channel blocks
            __nv_bfloat162 h[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(o[2 * k], o[2 * k + 1]);
            *reinterpret_cast<uint4 *>(a.y + actAt(P, pp, a.yOff + cb)) = *reinterpret_cast<const uint4 *>(h);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kCols));
}

template <int N>
cudaError_t launchTc(const ConvArgs &a, unsigned *error, cudaStream_t s) {
  const int tilesX = (a.W + kTX - 1) / kTX, tilesY = (a.H + kR - 1) / kR;
  const size_t tiles = (size_t)a.N * tilesX * tilesY;
  if (tiles > 0x7fffffff) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(kConv3x3Tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       smemBytes<N>());
  if (e != cudaSuccess) return e;
  kConv3x3Tc<N><<<dim3((unsigned)tiles, (a.Cout + N - 1) / N), 128, smemBytes<N>(), s>>>(
      a, tilesX, tilesY, error);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launchConv3x3Tc(const ConvArgs &a, unsigned *error, cudaStream_t s) {
  if (a.Cin <= 0 || a.Cin % 16 || a.Cout <= 0 || a.xC % 8 || a.xOff % 8 || !error)
    return cudaErrorInvalidValue;
  // bf16 outputs, masks and residuals in whole 8-channel blocks
  if ((!a.yf && (a.Cout % 8 || a.yOff % 8)) || (a.mask && a.maskOff % 8) ||
      (a.resid && a.residN > 8 * ((a.residC + 7) / 8)))
    return cudaErrorInvalidValue;
  if (a.split && (a.split < 0 || a.split % 32 || a.split >= a.Cin || !a.x2 || a.x2C % 8 ||
                  a.x2Off % 8 || a.x2Off + a.Cin - a.split > a.x2C))
    return cudaErrorInvalidValue;
  if (a.up && (a.H % 2 || a.W % 2)) return cudaErrorInvalidValue;
  if (a.N <= 0 || a.H <= 0 || a.W <= 0) return cudaSuccess;
  return a.Cout <= 32 ? launchTc<32>(a, error, s) : launchTc<64>(a, error, s);
}

}  // namespace vsr
