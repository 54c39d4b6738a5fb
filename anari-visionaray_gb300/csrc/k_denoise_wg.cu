// The denoiser's weight gradient on tcgen05: dW[co][tap][ci] = sum over
// pixels p of dY[p][co] * X[p + tap][ci] (tap = (dy, dx) of the 3x3 stencil,
// X zero outside the image), a GEMM per tap with M = output channels,
// N = input channels and the pixels as the reduction (K) dimension.
//
// One CTA owns 128 output channels (M, zero rows past Cout), 32 input
// channels (N) and a contiguous range of pixels, taken in chunks of 64. The
// nine taps' accumulators (9 x 32 fp32 columns) stay in tensor memory for
// the whole range. The activations are channel-blocked (16 bytes = 8
// channels per pixel, actAt), so a chunk's operands arrive pixel-major:
// cp.async copies (consecutive threads on consecutive pixels) stage dY's
// 64 pixels and X's three stencil rows (64 + 2 pixels each, at p + dy W - 1)
// per 8-channel block, one chunk ahead. ldmatrix.trans then reads 8 x 8
// blocks (8 pixels x 8 channels) transposed and the warps store them as
// core-matrix rows (8 pixels of one channel, 16 bytes) of the tensor core's
// no-swizzle K-major layout, zeroing taps' pixels outside the image (the
// staged rows are contiguous in memory, not in the image). One thread then issues the chunk's 9 taps x 4 tcgen05.mma (K = 16
// pixels each) and commits them to the slot's barrier; the gathers of the
// next chunks proceed into the other slots meanwhile. At the end the
// accumulators are read with tcgen05.ld and written as the CTA's partial
// sums; kWgradReduce adds the partials of all pixel ranges into dW in a
// fixed order (no atomics).
//
// Layouts (bytes): A (dY, M x K) as [kg 0..7][co 0..127][8 pixels], LBO
// (next 8 pixels along K) 2048, SBO (next 8 channels along M) 128; B (X,
// N x K) per tap as [kg][ci 0..31][8 pixels], LBO 512, SBO 128.
//
// Every wait is bounded (one second): a wait that runs out sets the error
// word and the CTA stops issuing work; before the tensor memory is released
// the issuing thread waits (bounded) for the MMAs it committed.
#include "kernels.h"

#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>

namespace vsr {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kM = 128;          // output channels per CTA (tensor-core M)
constexpr int kN = 32;           // input channels per CTA (N per tap)
constexpr int kChunkPx = 64;     // pixels per chunk (4 MMAs of K = 16)
constexpr int kKg = kChunkPx / 8;
constexpr int kABytes = kKg * kM * 16;        // 16384
constexpr int kBTapBytes = kKg * kN * 16;     // 4096
constexpr int kBBytes = 9 * kBTapBytes;       // 36864
constexpr int kSlotBytes = kABytes + kBBytes; // 53248 (a multiple of 1024)
constexpr int kSlots = 3;
// raw staging (pixel-major, 16 bytes per pixel and 8-channel block), two
// chunks: dY [16 blocks][64 pixels], X [3 rows][4 blocks][66 pixels]
constexpr int kRowPx = kChunkPx + 2;
constexpr int kRawA = (kM / 8) * kChunkPx * 16;        // 16384
constexpr int kRawB = 3 * (kN / 8) * kRowPx * 16;      // 12672
constexpr int kRawBytes = kRawA + kRawB;
constexpr int kRawOff = kSlots * kSlotBytes;
constexpr int kPixOff = kRawOff + 2 * kRawBytes;       // x, y of the chunk's pixels, two chunks
constexpr int kBarOff = kPixOff + 2 * 2 * kChunkPx * 4;
constexpr int kSmem = kBarOff + 64;           // empty[3], done, tensor-memory slot, abort
constexpr int kThreads = 512;
constexpr int kTmemCols = 512;                // 9 x 32 = 288 used
constexpr uint32_t kSpinLimit = 1u << 26;
constexpr uint64_t kWaitNs = 1000000000ull;
static_assert(kSmem <= 227 * 1024, "shared memory");

__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globalNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbarTry(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// true once the phase of the given parity has completed; false after a
// second, or at once when the CTA is aborting
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity, volatile int *abort) {
  const uint64_t t0 = globalNs();
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (mbarTry(bar, parity)) return true;
    if ((i & 63) == 63) {
      if (abort && *abort) return false;
      if (globalNs() - t0 > kWaitNs) return false;
    }
  }
  return false;
}

__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3fff);
  d |= (uint64_t)((lbo >> 4) & 0x3fff) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3fff) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// kind::f16: fp32 accumulator, bf16 A and B, both K-major; N, M
__host__ __device__ constexpr uint32_t instrDesc(int n, int m) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void cpAsync16(uint32_t dst, const void *src, bool valid) {
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}

// four 8 x 8 blocks of 16-bit elements, transposed: lane t gets, of block
// m, the elements (2 (t % 4), t / 4) and (2 (t % 4) + 1, t / 4) of the
// stored block (rows: the addresses lanes 8 m .. 8 m + 7 give)
__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

__global__ void __launch_bounds__(kThreads, 1)
    kConvWgradTc(WgradArgs a, int ciBlocks, int splits, int nChunks, float *part, unsigned *error) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kBarOff);
  const uint32_t emptyBar = smemAddr(bars), doneBar = emptyBar + 8 * kSlots;
  uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(bars + kSlots + 1);
  volatile int *abort = reinterpret_cast<volatile int *>(bars + kSlots + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int coBlock = blockIdx.x / ciBlocks, ciBlock = blockIdx.x % ciBlocks;
  const int co0 = coBlock * kM, ci0 = ciBlock * kN;
  const int split = blockIdx.y;
  const int cBegin = (int)((long long)split * nChunks / splits);
  const int cEnd = (int)((long long)(split + 1) * nChunks / splits);
  const int P = a.N * a.H * a.W;
  const uint32_t slot0 = smemAddr(smem);

  if (tid == 0) {
    for (int s = 0; s < kSlots; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(emptyBar + 8 * s));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(doneBar));
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smemAddr(tmemSlot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *tmemSlot;

  const int aBlocks = min(kM / 8, max(0, (a.Cout - co0 + 7) / 8));  // 8-channel blocks of dY
  // the K-major A rows of output channels past Cout stay zero: written once
  for (int i = tid; i < kSlots * kKg * (kM / 8 - aBlocks) * 32; i += kThreads) {
    const int w = i % 32, r = i / 32;
    const int cb = aBlocks + r % (kM / 8 - aBlocks), rest = r / (kM / 8 - aBlocks);
    const int kg = rest % kKg, sl = rest / kKg;
    reinterpret_cast<uint32_t *>(smem + sl * kSlotBytes + kg * (kM * 16) + cb * 128)[w] = 0u;
  }
  int *pixXY = reinterpret_cast<int *>(smem + kPixOff);
  // stage chunk c (raw buffer rb): dY, X's three rows, the pixels' x, y
  auto stage = [&](int c, int rb) {
    const uint32_t rawA = slot0 + kRawOff + rb * kRawBytes, rawB = rawA + kRawA;
    const int p0 = c * kChunkPx;
    for (int i = tid; i < aBlocks * kChunkPx; i += kThreads) {
      const int px = i % kChunkPx, cb = i / kChunkPx, p = p0 + px;
      const bool ok = p < P;
      cpAsync16(rawA + (cb * kChunkPx + px) * 16,
                a.dy + (ok ? actAt((size_t)P, (size_t)p, a.dyOff + co0 + cb * 8) : 0), ok);
    }
    for (int i = tid; i < 3 * (kN / 8) * kRowPx; i += kThreads) {
      const int px = i % kRowPx, r = i / kRowPx, cb = r % (kN / 8), dyi = r / (kN / 8);
      const long long q = (long long)p0 + (long long)(dyi - 1) * a.W + px - 1;
      const bool ok = q >= 0 && q < P && ci0 + cb * 8 < a.Cin;
      cpAsync16(rawB + ((dyi * (kN / 8) + cb) * kRowPx + px) * 16,
                a.x + (ok ? actAt((size_t)P, (size_t)q, a.xOff + ci0 + cb * 8) : 0), ok);
    }
    if (tid < kChunkPx) {
      const int p = p0 + tid;
      int x = -1000000, y = -1000000;
      if (p < P) {
        x = p % a.W;
        y = (p / a.W) % a.H;
      }
      pixXY[(rb * 2 + 0) * kChunkPx + tid] = x;
      pixXY[(rb * 2 + 1) * kChunkPx + tid] = y;
    }
    asm volatile("cp.async.commit_group;\n" ::);
  };
  int issued = 0;  // chunks whose MMAs were committed
  if (cBegin < cEnd) stage(cBegin, 0);
  for (int c = cBegin; c < cEnd; ++c) {
    const int k = c - cBegin, slot = k % kSlots, rb = k & 1;
    // the next chunk's copies go out before this one is transposed
    if (c + 1 < cEnd) stage(c + 1, rb ^ 1);
    else asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    if (k >= kSlots && !mbarWait(emptyBar + 8 * slot, ((k / kSlots) & 1) ^ 1, abort)) {
      atomicOr(error, 1u);
      *abort = 1;
    }
    __syncthreads();
    if (*abort) break;
    const uint32_t sA = slot0 + slot * kSlotBytes, sB = sA + kABytes;
    const uint32_t rawA = slot0 + kRawOff + rb * kRawBytes, rawB = rawA + kRawA;
    const int *xs = pixXY + (rb * 2) * kChunkPx, *ys = xs + kChunkPx;
    // 8 x 8 blocks: A (aBlocks x 8 pixel groups), then B (9 taps x 4 x 8);
    // a warp takes four blocks per ldmatrix.x4
    const int nA = aBlocks * kKg, nBlocks = nA + 9 * (kN / 8) * kKg;
    const int warps = kThreads / 32;
    for (int b0 = warp * 4; b0 < nBlocks; b0 += warps * 4) {
      // lane l addresses row l % 8 of block b0 + l / 8
      const int bl = b0 + (lane >> 3), row = lane & 7;
      uint32_t src = rawA;  // a valid address for lanes past the end
      if (bl < nA) {
        const int cb = bl / kKg, kg = bl % kKg;
        src = rawA + (cb * kChunkPx + kg * 8 + row) * 16;
      } else if (bl < nBlocks) {
        const int m = bl - nA, kg = m % kKg, r = m / kKg, cb = r % (kN / 8), tap = r / (kN / 8);
        src = rawB + (((tap / 3) * (kN / 8) + cb) * kRowPx + kg * 8 + row + tap % 3) * 16;
      }
      uint32_t v[4];
      ldsm4t(v, src);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int b = b0 + j;
        if (b >= nBlocks) break;
        const int ch = lane >> 2, pp = 2 * (lane & 3);  // channel row, first of two pixels
        uint32_t val = v[j], dst;
        if (b < nA) {
          const int cb = b / kKg, kg = b % kKg;
          dst = sA + kg * (kM * 16) + cb * 128;
        } else {
          const int m = b - nA, kg = m % kKg, r = m / kKg, cb = r % (kN / 8), tap = r / (kN / 8);
          const int dy = tap / 3 - 1, dx = tap % 3 - 1;
          dst = sB + tap * kBTapBytes + kg * (kN * 16) + cb * 128;
          // pixels kg * 8 + pp, + 1: zero where the tap leaves the image
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int px = kg * 8 + pp + h;
            const int xx = xs[px] + dx, yy = ys[px] + dy;
            if (!(xx >= 0 && xx < a.W && yy >= 0 && yy < a.H)) val &= h ? 0x0000ffffu : 0xffff0000u;
          }
        }
        asm volatile("st.shared.b32 [%0], %1;\n" ::"r"(dst + ch * 16 + (lane & 3) * 4), "r"(val));
      }
    }
    // the generic-proxy writes become visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      constexpr uint32_t idesc = instrDesc(kN, kM);
      const uint32_t aBase = slot0 + slot * kSlotBytes, bBase = aBase + kABytes;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
        for (int j = 0; j < kKg / 2; ++j) {
          const uint64_t da = smemDesc(aBase + 2 * j * (kM * 16), kM * 16, 128);
          const uint64_t db = smemDesc(bBase + tap * kBTapBytes + 2 * j * (kN * 16), kN * 16, 128);
          const uint32_t accum = (k > 0 || j > 0) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                  tmem + (uint32_t)(tap * kN)),
              "l"(da), "l"(db), "r"(idesc), "r"(accum));
        }
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              emptyBar + 8 * slot));
    }
    ++issued;
  }
  // all committed MMAs done (tcgen05.commit tracks every earlier MMA)
  __syncthreads();
  const bool aborted = *abort != 0;
  if (tid == 0 && issued > 0)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
        doneBar));
  bool okLocal = issued > 0 && !aborted;
  if (issued > 0 && !mbarWait(doneBar, 0, nullptr)) {
    atomicOr(error, 1u);
    okLocal = false;
  }
  // the tensor-memory reads below are warp-collective: one outcome for all
  const bool ok = __syncthreads_and(okLocal ? 1 : 0) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  // epilogue: warp w reads tensor-memory lane quarter w % 4 (output
  // channels 32 (w % 4) ..), taps w / 4, w / 4 + 4, ...
  const int co = co0 + (warp & 3) * 32 + lane;
#pragma unroll 1
  for (int tap = warp >> 2; tap < 9; tap += kThreads / 128) {
    uint32_t v[32];
    if (ok) {
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
          "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
            "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
            "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
            "=r"(v[31])
          : "r"(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(tap * kN)));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = 0u;
    }
    if (co >= a.Cout) continue;
    float *dst = part + (((size_t)split * a.Cout + co) * 9 + tap) * a.Cin + ci0;
#pragma unroll
    for (int i = 0; i < kN; i += 4) {
      if (ci0 + i >= a.Cin) break;  // Cin is a multiple of 8, the partial rows 16-byte aligned
      reinterpret_cast<float4 *>(dst)[i / 4] =
          make_float4(__uint_as_float(v[i]), __uint_as_float(v[i + 1]), __uint_as_float(v[i + 2]),
                      __uint_as_float(v[i + 3]));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(kTmemCols));
}

// dW[i] += sum over s of part[s][i], in order of s
__global__ void kWgradReduce(const float *part, int splits, size_t n, float *dw) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += part[(size_t)k * n + i];
    dw[i] += s;
  }
}

}  // namespace

// The grid: (output-channel blocks x input-channel blocks, pixel ranges),
// about two CTAs' worth of work per SM; the partial buffer needs
// wgradPartFloats(...) floats.
static void wgradGrid(int Cout, int Cin, int P, int &ciBlocks, int &splits, int &nChunks) {
  ciBlocks = (Cin + kN - 1) / kN;
  const int tiles = ((Cout + kM - 1) / kM) * ciBlocks;
  nChunks = (P + kChunkPx - 1) / kChunkPx;
  splits = std::max(1, std::min(nChunks, (304 + tiles - 1) / tiles));
}

size_t wgradPartFloats(int Cout, int Cin, int P) {
  int ciBlocks, splits, nChunks;
  wgradGrid(Cout, Cin, P, ciBlocks, splits, nChunks);
  return (size_t)splits * Cout * 9 * Cin;
}

cudaError_t launchConvWgradTc(const WgradArgs &a, float *part, unsigned *error, cudaStream_t s) {
  if (a.Cin % 8 || a.Cout % 8 || a.dyC % 8 || a.dyOff % 8 || a.xC % 8 || a.xOff % 8 || !part)
    return cudaErrorInvalidValue;
  const int P = a.N * a.H * a.W;
  if (P <= 0) return cudaSuccess;
  int ciBlocks, splits, nChunks;
  wgradGrid(a.Cout, a.Cin, P, ciBlocks, splits, nChunks);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(kConvWgradTc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const dim3 grid((unsigned)(((a.Cout + kM - 1) / kM) * ciBlocks), (unsigned)splits);
  kConvWgradTc<<<grid, kThreads, kSmem, s>>>(a, ciBlocks, splits, nChunks, part, error);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const size_t n = (size_t)a.Cout * 9 * a.Cin;
  kWgradReduce<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>(part, splits, n, a.dw);
  return cudaGetLastError();
}

}  // namespace vsr
