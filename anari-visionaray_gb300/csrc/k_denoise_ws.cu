// The denoiser's 3x3 convolution as a persistent, warp-specialised tcgen05
// kernel with TMA loads.
//
// Work: the same tiles as kConv3x3Tc (k_denoise_tc.cu): 4 image rows x 128
// pixels x N output channels (64, or 32 for narrow layers), the input
// channels in stages of 32. One CTA per SM walks its share of the tiles.
// Three roles run concurrently, linked by mbarriers:
//
//   warps 9-12 producer: for each stage they wait for a free slot of a 2- or
//              3-slot shared-memory ring; one thread loads the stage's
//              weights (one bulk copy of their packed shared-memory image,
//              packConvWeights) and its input halo: activations are
//              channel-blocked planes (actAt, kernels.h), so 4 blocks x 6
//              rows x 130 pixels x 8 channels is one 5-d TMA box whose rows
//              are contiguous; the tensor map zero-fills outside the image.
//              A decoder's upsampled input (read at (y / 2, x / 2) of the
//              coarser level) is not a box: for those stages the 128
//              producer threads gather the halo with cp.async instead. The
//              slot's "full" barrier counts the TMA bytes and the threads'
//              cp.async completions.
//   warp 8     MMA: one thread waits for a full slot, issues the stage's
//              4 x 9 x 2 tcgen05.mma (bf16 x bf16 -> fp32; descriptors are
//              the slot's base descriptor plus constant offsets) into one of
//              two accumulator sets in tensor memory, and commits them to
//              the slot's "empty" barrier, and after a tile's last stage to
//              the set's "full" barrier.
//   warps 0-7  epilogue: wait for an accumulator set, read it with
//              tcgen05.ld (warp w reads lanes 32 (w % 4) .. and rows
//              2 (w / 4), 2 (w / 4) + 1 of the tile), apply bias,
//              ReLU, residual and mask like kConv3x3, store 16-byte blocks,
//              and release the set; meanwhile the MMA thread fills the other.
//
// Shared-memory operands use the tensor core's no-swizzle K-major layout
// (core matrices of 8 rows x 16 bytes): the halo as [block][row][130
// pixels][16 B] (the TMA box image; blocks 12480 bytes apart = the LBO of
// A, 8-pixel groups 128 bytes apart = SBO); the weights as
// [tap][block][N][16 B] (LBO N x 16 B, SBO 128 B). Tap (dy, dx) of output
// row r is the halo view that starts at row r + dy + 1, pixel dx + 1.
//
// Every wait is bounded (one second). A role whose wait runs out sets the
// error word and the CTA's abort flag, which ends the other roles' loops;
// before the tensor memory is released the producer waits (bounded) for
// the loads it issued and the MMA thread for the MMAs it committed.
#include "kernels.h"

#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <mutex>

namespace vsr {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kR = 4;             // output rows per tile
constexpr int kTX = 128;          // output pixels per tile row (tensor-core M)
constexpr int kHY = kR + 2;       // halo rows
constexpr int kHX = kTX + 2;      // halo pixels per row
constexpr int kChunks = 4;        // 8-channel chunks per stage
constexpr int kPlane = kHY * kHX * 16;  // one 8-channel block of the halo: 12480 bytes
constexpr int kHaloBytes = kChunks * kPlane;
constexpr int kEpiWarps = 8;      // two per tensor-memory lane quarter, two rows each
constexpr int kThreads = 32 * (kEpiWarps + 1 + 4);  // + 1 MMA warp + 4 producer warps
constexpr int kMmaWarp = kEpiWarps, kProdWarp0 = kEpiWarps + 1, kProducers = 128;
constexpr uint32_t kSpinLimit = 1u << 26;
constexpr uint64_t kWaitNs = 1000000000ull;  // one second

template <int N>
struct Cfg {
  static constexpr int kSlots = N == 64 ? 2 : 3;
  static constexpr int kWBytes = 9 * kChunks * N * 16;
  static constexpr int kSlotBytes = (kHaloBytes + kWBytes + 1023) / 1024 * 1024;
  static constexpr int kBarOff = kSlots * kSlotBytes;
  static constexpr int kSmem = kBarOff + 256;
  // barriers (2 kSlots + 4), tensor-memory slot, abort flag, timeout-test barrier
  static_assert(8 * (2 * kSlots + 7) <= 256, "barrier area");
  static constexpr int kCols = 2 * kR * N;  // two accumulator sets: 512 or 256 columns
};
static_assert(Cfg<64>::kSmem <= 227 * 1024 && Cfg<32>::kSmem <= 227 * 1024, "shared memory");

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

// a warp-uniform wait: lane 0 polls, the warp takes its outcome
__device__ __forceinline__ bool warpWait(uint32_t bar, uint32_t parity, volatile int *abort) {
  bool ok = false;
  if ((threadIdx.x & 31) == 0) ok = mbarWait(bar, parity, abort);
  return __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
}

__device__ __forceinline__ void fail(unsigned *error, volatile int *abort) {
  atomicOr(error, 1u);
  *abort = 1;
}

__device__ __forceinline__ void cpAsync16(uint32_t dst, const void *src, bool valid) {
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}

// one bulk copy of `bytes` (a multiple of 16) from global to shared memory
__device__ __forceinline__ void bulkCopy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tma5(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                     int c3, int c4, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3, %4, %5, %6}], [%7];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3fff);
  d |= (uint64_t)((lbo >> 4) & 0x3fff) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3fff) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__host__ __device__ constexpr uint32_t instrDesc(int n, int m) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

struct Tile {
  int n, x0, y0, nBase;
};

__device__ __forceinline__ Tile tileOf(int u, int tilesX, int tilesY, int nTiles, int N) {
  Tile t;
  const int nt = u % nTiles;
  int r = u / nTiles;
  const int tx = r % tilesX;
  r /= tilesX;
  const int ty = r % tilesY;
  t.n = r / tilesY;
  t.x0 = tx * kTX;
  t.y0 = ty * kR;
  t.nBase = nt * N;
  return t;
}

// Stall = true is the instantiation the wait-timeout test launches (its MMA
// thread first waits on a barrier nothing completes); kept apart because
// the test branch in the production kernel cost 13 % of a 1080p pass.
template <int N, bool Stall>
__global__ void __launch_bounds__(kThreads, 1)
    kConv3x3Ws(const __grid_constant__ CUtensorMap mapX, ConvArgs a, int tilesX, int tilesY,
               int nTiles, int units, unsigned *error) {
  typedef Cfg<N> C;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + C::kBarOff);
  // barriers: full[kSlots], empty[kSlots], accFull[2], accEmpty[2]
  const uint32_t fullBar = smemAddr(bars), emptyBar = fullBar + 8 * C::kSlots;
  const uint32_t accFullBar = emptyBar + 8 * C::kSlots, accEmptyBar = accFullBar + 16;
  uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(bars + 2 * C::kSlots + 4);
  volatile int *abort = reinterpret_cast<volatile int *>(bars + 2 * C::kSlots + 5);
  const uint32_t stallBar = smemAddr(bars + 2 * C::kSlots + 6);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int stages = (a.Cin + 8 * kChunks - 1) / (8 * kChunks);
  const uint32_t slot0 = smemAddr(smem);

  if (threadIdx.x == 0) {
    for (int s = 0; s < C::kSlots; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(fullBar + 8 * s),
                   "r"(1 + kProducers));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(emptyBar + 8 * s));
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(accFullBar + 8 * b));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(accEmptyBar + 8 * b),
                   "r"(32 * kEpiWarps));
    }
    // a barrier nothing arrives on, waited on only by the timeout test
    if (Stall) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(stallBar));
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smemAddr(tmemSlot)),
                 "r"(C::kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *tmemSlot;

  if (warp >= kProdWarp0) {
    // ------------------------------------------------------------ producer
    const int pt = threadIdx.x - kProdWarp0 * 32;  // 0..127
    const bool leader = pt == 0;
    int g = 0;  // stages issued
    const bool up = a.split > 0;
    const size_t Pc = (size_t)a.N * (a.H >> 1) * (a.W >> 1);  // pixels of an upsampled source
    for (int u = blockIdx.x; u < units && !*abort; u += gridDim.x) {
      const Tile T = tileOf(u, tilesX, tilesY, nTiles, N);
      for (int s = 0; s < stages; ++s, ++g) {
        const int slot = g % C::kSlots, round = g / C::kSlots;
        if (!warpWait(emptyBar + 8 * slot, (round & 1) ^ 1, abort)) {
          if (lane == 0) fail(error, abort);
          break;
        }
        const uint32_t sHalo = slot0 + slot * C::kSlotBytes, sW = sHalo + kHaloBytes;
        const uint32_t full = fullBar + 8 * slot;
        const int c0 = s * 8 * kChunks;
        const int chunks = min(kChunks, (a.Cin - c0) / 8);
        const bool gather = up && c0 < a.split;
        if (leader) {
          const uint32_t bytes = (uint32_t)(C::kWBytes + (gather ? 0 : kHaloBytes));
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(full),
                       "r"(bytes)
                       : "memory");
          bulkCopy(sW, a.wPacked + ((size_t)(T.nBase / N) * stages + s) * (C::kWBytes / 2),
                   (uint32_t)C::kWBytes, full);
          if (!gather) {
            const int blk = (up ? a.x2Off + c0 - a.split : a.xOff + c0) / 8;
            tma5(sHalo, &mapX, 0, T.x0 - 1, T.y0 - 1, T.n, blk, full);
          }
        }
        if (gather) {
          // the upsampled coarse level, zero outside the image; pixel
          // fastest, so that a warp reads a row of one 8-channel block
          const int Hc = a.H >> 1, Wc = a.W >> 1;
          const int entries = chunks * kHY * kHX;
          for (int i = pt; i < entries; i += kProducers) {
            const int hx = i % kHX;
            const int r = i / kHX;
            const int c = r % chunks, hy = r / chunks;
            const int y = T.y0 - 1 + hy, x = T.x0 - 1 + hx;
            const bool in = y >= 0 && y < a.H && x >= 0 && x < a.W;
            const size_t pix = ((size_t)T.n * Hc + (y >> 1)) * Wc + (x >> 1);
            const bf16 *src = a.x + (in ? actAt(Pc, pix, a.xOff + c0 + 8 * c) : 0);
            cpAsync16(sHalo + (uint32_t)(c * kPlane + (hy * kHX + hx) * 16), src, in);
          }
        }
        // each thread's cp.async (none outside gather stages) completes one arrival
        asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" ::"r"(full) : "memory");
      }
      if (*abort) break;
    }
    // before the CTA ends: the loads issued complete
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (leader)
      for (int k = max(0, g - C::kSlots); k < g; ++k)
        mbarWait(fullBar + 8 * (k % C::kSlots), (k / C::kSlots) & 1, nullptr);
    __syncwarp();
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------ MMA
    if (lane == 0) {
      int g = 0, j = 0;
      int lastSlot = -1, lastRound = 0;
      constexpr uint32_t idesc = instrDesc(N, kTX);
      // timeout test: the MMA thread has issued nothing when this wait runs
      // out; the producer drains the loads it started before the CTA ends
      if (Stall && !mbarWait(stallBar, 0, abort)) fail(error, abort);
      for (int u = blockIdx.x; u < units && !*abort; u += gridDim.x, ++j) {
        const int b = j & 1;
        if (!mbarWait(accEmptyBar + 8 * b, ((j >> 1) & 1) ^ 1, abort)) {
          fail(error, abort);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        const uint32_t dBase = tmem + (uint32_t)(b * kR * N);
        bool ok = true;
        for (int s = 0; s < stages; ++s, ++g) {
          const int slot = g % C::kSlots, round = g / C::kSlots;
          if (!mbarWait(fullBar + 8 * slot, round & 1, abort)) {
            fail(error, abort);
            ok = false;
            break;
          }
          const int c0 = s * 8 * kChunks;
          const int chunks = min(kChunks, (a.Cin - c0) / 8);
          // a gathered halo was written through the generic proxy
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
          const uint32_t sHalo = slot0 + slot * C::kSlotBytes, sW = sHalo + kHaloBytes;
          // descriptors: the slot's base plus constant offsets in 16-byte units
          const uint64_t da0 = smemDesc(sHalo, kPlane, 128), db0 = smemDesc(sW, N * 16, 128);
#pragma unroll
          for (int r = 0; r < kR; ++r) {
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
              for (int k = 0; k < kChunks; k += 2) {
                if (k >= chunks) break;
                const uint64_t da =
                    da0 + (uint64_t)((((r + tap / 3) * kHX + tap % 3) * 16 + k * kPlane) >> 4);
                const uint64_t db = db0 + (uint64_t)(((tap * kChunks + k) * N * 16) >> 4);
                const uint32_t accum = (s > 0 || tap > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                        dBase + (uint32_t)(r * N)),
                    "l"(da), "l"(db), "r"(idesc), "r"(accum));
              }
            }
          }
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                  emptyBar + 8 * slot));
          lastSlot = slot;
          lastRound = round;
        }
        if (!ok) break;
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                accFullBar + 8 * b));
      }
      // before the CTA ends: the MMAs committed complete
      if (lastSlot >= 0) mbarWait(emptyBar + 8 * lastSlot, lastRound & 1, nullptr);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    // warp w reads tensor-memory lane quarter w % 4 (the only one it may
    // access) and rows 2 (w / 4), 2 (w / 4) + 1 of the tile
    const int q = warp & 3, rowBase = 2 * (warp >> 2);
    const size_t P = (size_t)a.N * a.H * a.W;
    int j = 0;
    for (int u = blockIdx.x; u < units && !*abort; u += gridDim.x, ++j) {
      const int b = j & 1;
      if (!warpWait(accFullBar + 8 * b, (j >> 1) & 1, abort)) {
        if (lane == 0) fail(error, abort);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      const Tile T = tileOf(u, tilesX, tilesY, nTiles, N);
      const int x = T.x0 + q * 32 + lane;
      // columns outside, rows inside: the 32 biases of a column group are
      // loaded once per tile (loading them per element and row made the
      // epilogue the pipeline's bottleneck)
#pragma unroll
      for (int c32 = 0; c32 < N / 32; ++c32) {
        float bias[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) {
          const int c = T.nBase + c32 * 32 + k;
          bias[k] = (a.bias && c < a.Cout) ? __ldg(a.bias + c) : 0.f;
        }
#pragma unroll 1
        for (int r = rowBase; r < rowBase + 2; ++r) {
          const int y = T.y0 + r;
          const bool pixIn = x < a.W && y < a.H;
          const size_t pp = ((size_t)T.n * a.H + y) * a.W + x;
          uint32_t v[32];
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
              "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
                "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
                "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
                "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
                "=r"(v[31])
              : "r"(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kR * N + r * N + c32 * 32)));
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
          if (!pixIn) continue;
#pragma unroll
          for (int g8 = 0; g8 < 32; g8 += 8) {
            const int cb = T.nBase + c32 * 32 + g8;
            if (cb >= a.Cout) break;
            float o[8];
            uint4 rv = make_uint4(0, 0, 0, 0), mv = make_uint4(0, 0, 0, 0);
            if (a.resid && cb < a.residN)
              rv = *reinterpret_cast<const uint4 *>(a.resid + actAt(P, pp, cb));
            if (a.mask) mv = *reinterpret_cast<const uint4 *>(a.mask + actAt(P, pp, a.maskOff + cb));
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int c = cb + k;
              float val = __uint_as_float(v[g8 + k]);
              val += bias[g8 + k];
              if (a.relu) val = fmaxf(val, 0.f);
              if (a.resid && c < a.residN)
                val += __bfloat162float(reinterpret_cast<const bf16 *>(&rv)[k]);
              if (a.mask && !(__bfloat162float(reinterpret_cast<const bf16 *>(&mv)[k]) > 0.f))
                val = 0.f;
              o[k] = val;
            }
            if (a.yf) {  // fp32 output: NHWC, two 16-byte stores per 8 channels
              const size_t ob = pp * a.yC + a.yOff + cb;
              if (cb + 8 <= a.Cout && (ob & 3) == 0) {
                reinterpret_cast<float4 *>(a.yf + ob)[0] = make_float4(o[0], o[1], o[2], o[3]);
                reinterpret_cast<float4 *>(a.yf + ob)[1] = make_float4(o[4], o[5], o[6], o[7]);
              } else {
#pragma unroll
                for (int k = 0; k < 8; ++k)
                  if (cb + k < a.Cout) a.yf[ob + k] = o[k];
              }
            } else {
              __nv_bfloat162 h[4];
#pragma unroll
              for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(o[2 * k], o[2 * k + 1]);
              *reinterpret_cast<uint4 *>(a.y + actAt(P, pp, a.yOff + cb)) =
                  *reinterpret_cast<const uint4 *>(h);
            }
          }
        }
      }
      // this set is read: the MMA thread may overwrite it
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(accEmptyBar + 8 * b) : "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == kMmaWarp)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(C::kCols));
}

// cuTensorMapEncodeTiled through the runtime's driver entry point
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

bool encodeBf16(CUtensorMap *map, const void *base, int rank, const cuuint64_t *dims,
                const cuuint64_t *strides, const cuuint32_t *box) {
  EncodeTiledFn fn = encodeTiled();
  if (!fn) return false;
  const cuuint32_t ones[5] = {1, 1, 1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void *>(base), dims,
            strides, box, ones, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int N>
cudaError_t launchWs(const ConvArgs &a, unsigned *error, cudaStream_t s) {
  typedef Cfg<N> C;
  // the full-resolution input read by boxes: the skip connection of a
  // decoder, else x
  const bool up = a.split > 0;
  const bf16 *src = up ? a.x2 : a.x;
  const int srcC = up ? a.x2C : a.xC;
  // blocked planes as a 5-d tensor: [block][n][y][x][8 channels]
  CUtensorMap mapX;
  const cuuint64_t P = (cuuint64_t)a.N * a.H * a.W;
  const cuuint64_t xd[5] = {8, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.N,
                            (cuuint64_t)(srcC / 8)};
  const cuuint64_t xs[4] = {16, (cuuint64_t)a.W * 16, (cuuint64_t)a.H * a.W * 16, P * 16};
  const cuuint32_t xb[5] = {8, (cuuint32_t)kHX, (cuuint32_t)kHY, 1, (cuuint32_t)kChunks};
  if (!encodeBf16(&mapX, src, 5, xd, xs, xb)) return cudaErrorInvalidValue;
  const int tilesX = (a.W + kTX - 1) / kTX, tilesY = (a.H + kR - 1) / kR;
  const int nTiles = (a.Cout + N - 1) / N;
  const long long units = (long long)a.N * tilesX * tilesY * nTiles;
  if (units > 0x7fffffff) return cudaErrorInvalidValue;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    sms = sms > 0 ? sms : 1;
  }
  auto kernel = a.testStall ? kConv3x3Ws<N, true> : kConv3x3Ws<N, false>;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       C::kSmem);
  if (e != cudaSuccess) return e;
  const int grid = (int)std::min<long long>(units, sms);
  kernel<<<grid, kThreads, C::kSmem, s>>>(mapX, a, tilesX, tilesY, nTiles, (int)units, error);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launchConv3x3Ws(const ConvArgs &a, unsigned *error, cudaStream_t s) {
  if (a.Cin <= 0 || a.Cin % 16 || a.Cout <= 0 || a.xC % 8 || a.xOff % 8 || !error || !a.x ||
      !a.wPacked)
    return cudaErrorInvalidValue;
  if ((!a.yf && (a.Cout % 8 || a.yOff % 8)) || (a.mask && a.maskOff % 8) ||
      (a.resid && a.residN > 8 * ((a.residC + 7) / 8)))
    return cudaErrorInvalidValue;
  if (a.split && (a.split < 0 || a.split % 32 || a.split >= a.Cin || !a.x2 || a.x2C % 8 ||
                  a.x2Off % 8 || a.x2Off + a.Cin - a.split > a.x2C || !a.up))
    return cudaErrorInvalidValue;
  if (!a.split && a.up) return cudaErrorInvalidValue;
  if (a.up && (a.H % 2 || a.W % 2)) return cudaErrorInvalidValue;
  if (a.N <= 0 || a.H <= 0 || a.W <= 0) return cudaSuccess;
  return a.Cout <= 32 ? launchWs<32>(a, error, s) : launchWs<64>(a, error, s);
}

}  // namespace vsr
