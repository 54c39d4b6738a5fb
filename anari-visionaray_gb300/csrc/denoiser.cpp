// Host side of the learned denoiser (denoiser.h): parameter layout, the
// forward pass, the backward pass and Adam, as launches of the kernels in
// k_denoise.cu on the caller's stream.
#include "denoiser.h"

#include "kernels.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace vsr {
namespace {

// (cin, cout) of the 15 convolutions, in execution order
const int kLayerIO[15][2] = {{16, 32},   {32, 32},   {32, 64},  {64, 64},  {64, 128},
                             {128, 128}, {128, 256}, {256, 256}, {384, 128}, {128, 128},
                             {192, 64},  {64, 64},   {96, 32},  {32, 32},  {32, 16}};
enum {
  L_E0A, L_E0B, L_E1A, L_E1B, L_E2A, L_E2B, L_E3A, L_E3B,
  L_D2A, L_D2B, L_D1A, L_D1B, L_D0A, L_D0B, L_OUT
};

// splitmix64 + Box-Muller: a normal stream that is the same on every host
struct Normal {
  uint64_t s;
  double next01() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  }
  double operator()() {
    const double u = next01(), v = next01();
    return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
  }
};

// keeps the first error of a sequence of launches (argument checks return
// errors without setting CUDA's last error)
struct FirstError {
  cudaError_t e = cudaSuccess;
  void operator()(cudaError_t r) {
    if (e == cudaSuccess) e = r;
  }
};

template <typename T>
cudaError_t alloc(T *&p, size_t n, std::vector<void *> *track = nullptr) {
  cudaError_t e = cudaMalloc((void **)&p, std::max<size_t>(n, 1) * sizeof(T));
  if (e == cudaSuccess && track) track->push_back(p);
  return e;
}

}  // namespace

Denoiser::Denoiser(uint64_t seed) {
  size_t off = 0, offT = 0, offP = 0;
  for (auto &io : kLayerIO) {
    DenoiseLayer L;
    L.cin = io[0];
    L.cout = io[1];
    L.w = off;
    off += (size_t)L.cout * 9 * L.cin;
    L.b = off;
    off += L.cout;
    L.wt = offT;
    offT += (size_t)L.cout * 9 * L.cin;
    L.wp = offP;
    offP += packedConvWeights(L.cin, L.cout);
    L.wtp = offP;
    offP += packedConvWeights(L.cout, L.cin);
    layers_.push_back(L);
  }
  numParams_ = off;
  numWt_ = offT;
  numPacked_ = offP;
  ok_ = alloc(params_, off) == cudaSuccess && alloc(m_, off) == cudaSuccess &&
        alloc(v_, off) == cudaSuccess && alloc(grad_, off) == cudaSuccess &&
        alloc(wbf_, off) == cudaSuccess && alloc(wt_, offT) == cudaSuccess &&
        alloc(wpk_, offP) == cudaSuccess &&
        alloc(loss_, 1) == cudaSuccess && alloc(err_, 1) == cudaSuccess &&
        cudaMemset(err_, 0, sizeof(unsigned)) == cudaSuccess;
  if (!ok_) return;
  // He-normal weights (std sqrt(2 / fan_in)), zero biases. The output layer
  // starts at zero: the network begins as the identity on the input's
  // colour and grows its correction from there (a random correction at the
  // start drives the first steps to switch the ReLUs off instead).
  std::vector<float> h(off, 0.f);
  Normal rng{seed};
  for (size_t li = 0; li < layers_.size(); ++li) {
    const DenoiseLayer &L = layers_[li];
    const double sd = std::sqrt(2.0 / (9.0 * L.cin));
    const int used = li + 1 == layers_.size() ? 0 : L.cout;
    for (int co = 0; co < used; ++co)
      for (int k = 0; k < 9 * L.cin; ++k) h[L.w + (size_t)co * 9 * L.cin + k] = (float)(sd * rng());
  }
  ok_ = setParams(h.data(), 0) == cudaSuccess;
}

Denoiser::~Denoiser() {
  for (void *p : {(void *)params_, (void *)m_, (void *)v_, (void *)grad_, (void *)wbf_, (void *)wt_,
                  (void *)wpk_, (void *)loss_, (void *)err_})
    if (p) cudaFree(p);
  for (void *p : bufs_) cudaFree(p);
}

cudaError_t Denoiser::getParams(float *host, cudaStream_t s) {
  cudaError_t e =
      cudaMemcpyAsync(host, params_, numParams_ * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

cudaError_t Denoiser::setParams(const float *host, cudaStream_t s) {
  cudaError_t e =
      cudaMemcpyAsync(params_, host, numParams_ * sizeof(float), cudaMemcpyHostToDevice, s);
  // Adam state restarts; the bf16 copies are refreshed by a zero-rate step
  // on zero gradients, which leaves the weights and m, v (zero) unchanged
  if (e == cudaSuccess) e = cudaMemsetAsync(m_, 0, numParams_ * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(v_, 0, numParams_ * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(grad_, 0, numParams_ * sizeof(float), s);
  step_ = 0;
  for (const DenoiseLayer &L : layers_) {
    if (e != cudaSuccess) break;
    e = launchAdam(params_ + L.w, m_ + L.w, v_ + L.w, grad_ + L.w, (size_t)L.cout * 9 * L.cin, 0.f,
                   0.9f, 0.999f, 1e-8f, 1, wbf_ + L.w, wt_ + L.wt, L.cin, L.cout, s);
  }
  if (e == cudaSuccess) e = pack(s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

cudaError_t Denoiser::pack(cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  for (const DenoiseLayer &L : layers_) {
    if (e == cudaSuccess) e = launchPackConvWeights(wbf_ + L.w, L.cin, L.cout, wpk_ + L.wp, s);
    // the input gradient's weights: cout input channels, cin output channels
    if (e == cudaSuccess) e = launchPackConvWeights(wt_ + L.wt, L.cout, L.cin, wpk_ + L.wtp, s);
  }
  return e;
}

cudaError_t Denoiser::ensure(int N, int H, int W, bool train) {
  if (N == n_ && H == h_ && W == w_ && (train_ || !train)) return cudaSuccess;
  for (void *p : bufs_) cudaFree(p);
  bufs_.clear();
  act_ = Act{};
  grd_ = Act{};
  out_ = nullptr;
  gout_ = nullptr;
  n_ = h_ = w_ = 0;
  const size_t P0 = (size_t)N * H * W, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
  struct Sz {
    __nv_bfloat16 *Act::*f;
    size_t n;
  } sizes[] = {{&Act::x0, P0 * kInC}, {&Act::a0, P0 * 32},   {&Act::e0, P0 * 32},   {&Act::p0, P1 * 32},
               {&Act::a1, P1 * 64},   {&Act::e1, P1 * 64},   {&Act::p1, P2 * 64},
               {&Act::a2, P2 * 128},  {&Act::e2, P2 * 128},  {&Act::p2, P3 * 128},
               {&Act::a3, P3 * 256},  {&Act::e3, P3 * 256},  {&Act::cat2, P2 * 384},
               {&Act::b2, P2 * 128},  {&Act::d2, P2 * 128},  {&Act::cat1, P1 * 192},
               {&Act::b1, P1 * 64},   {&Act::d1, P1 * 64},   {&Act::cat0, P0 * 96},
               {&Act::b0, P0 * 32},   {&Act::d0, P0 * 32}};
  cudaError_t e = cudaSuccess;
  for (auto &z : sizes) {
    if (e == cudaSuccess) e = alloc(act_.*z.f, z.n, &bufs_);
    if (train && e == cudaSuccess) e = alloc(grd_.*z.f, z.n, &bufs_);
  }
  if (e == cudaSuccess) e = alloc(out_, P0 * kOutC, &bufs_);
  // the tcgen05 weight gradient's partial sums (tensor path 4; allocated at
  // its first use): the largest layer's
  wgradPart_ = nullptr;
  wgradPartFloats_ = 0;
  const int levelOf[15] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
  for (size_t li = 0; li < layers_.size(); ++li) {
    const int Pl = (int)(P0 >> (2 * levelOf[li]));
    wgradPartFloats_ =
        std::max(wgradPartFloats_, wgradPartFloats(layers_[li].cout, layers_[li].cin, Pl));
  }
  if (train && e == cudaSuccess) {
    e = alloc(gout_, P0 * kOutC, &bufs_);
    if (e == cudaSuccess) e = cudaMemset(gout_, 0, P0 * kOutC * sizeof(__nv_bfloat16));
  }
  if (e != cudaSuccess) return e;
  n_ = N;
  h_ = H;
  w_ = W;
  train_ = train;
  return cudaSuccess;
}

cudaError_t Denoiser::conv(int li, const __nv_bfloat16 *x, int xC, __nv_bfloat16 *y, float *yf, int yC,
                    int N, int H, int W, bool relu, cudaStream_t s, const __nv_bfloat16 *resid) {
  const DenoiseLayer &L = layers_[li];
  ConvArgs a{};
  a.x = x;
  a.xC = xC;
  a.Cin = L.cin;
  a.w = wbf_ + L.w;
  a.wPacked = wpk_ + L.wp;
  a.bias = params_ + L.b;
  a.Cout = L.cout;
  a.y = y;
  a.yf = yf;
  a.yC = yC;
  a.relu = relu ? 1 : 0;
  a.N = N;
  a.H = H;
  a.W = W;
  a.resid = resid;
  a.residC = kInC;
  a.residN = kColorC;
  return useTc(W) ? launchTc(a, s) : launchConv3x3(a, s);
}

cudaError_t Denoiser::launchTc(const ConvArgs &args, cudaStream_t s) const {
  ConvArgs a = args;
  a.testStall = stallNext_ ? 1 : 0;
  stallNext_ = false;
  return tensorPath_ == 3 ? launchConv3x3Tc(a, err_, s) : launchConv3x3Ws(a, err_, s);
}

// a decoder convolution on [upsampled coarse level | skip connection],
// read in place (tcgen05 path)
cudaError_t Denoiser::convCat(int li, const __nv_bfloat16 *coarse, int coarseC, const __nv_bfloat16 *skip,
                       int skipC, __nv_bfloat16 *y, int yC, int N, int H, int W, cudaStream_t s) {
  const DenoiseLayer &L = layers_[li];
  ConvArgs a{};
  a.x = coarse;
  a.xC = coarseC;
  a.up = 1;
  a.x2 = skip;
  a.x2C = skipC;
  a.split = coarseC;
  a.Cin = L.cin;
  a.w = wbf_ + L.w;
  a.wPacked = wpk_ + L.wp;
  a.bias = params_ + L.b;
  a.Cout = L.cout;
  a.y = y;
  a.yC = yC;
  a.relu = 1;
  a.N = N;
  a.H = H;
  a.W = W;
  return launchTc(a, s);
}

// Weight and bias gradients of layer li from its pre-activation gradient dy
// (cout channels) and its input x; with dx, also the gradient of the
// layer's input, zeroed where `mask` (the input itself, a ReLU output) is
// not positive, which makes it the pre-activation gradient of the layer
// that produced the input.
cudaError_t Denoiser::convBack(int li, const __nv_bfloat16 *x, int xC, const __nv_bfloat16 *dy,
                        __nv_bfloat16 *dx, const __nv_bfloat16 *mask, int N, int H, int W,
                        cudaStream_t s) {
  const DenoiseLayer &L = layers_[li];
  const int P = N * H * W;
  WgradArgs g{};
  g.dy = dy;
  g.dyC = L.cout;
  g.Cout = L.cout;
  g.x = x;
  g.xC = xC;
  g.Cin = L.cin;
  g.dw = grad_ + L.w;
  g.N = N;
  g.H = H;
  g.W = W;
  cudaError_t e = cudaSuccess;
  if (tensorPath_ == 4 && !wgradPart_) e = alloc(wgradPart_, wgradPartFloats_, &bufs_);
  if (tensorPath_ == 4) {
    // tcgen05: accumulators in tensor memory, partial sums per pixel range
    if (e == cudaSuccess) e = launchConvWgradTc(g, wgradPart_, err_, s);
  } else {
    // mma.sync: split the pixel reduction so that about 2048 CTAs run
    const int tiles = ((L.cout + 63) / 64) * 9 * ((L.cin + 63) / 64);
    const int chunks = std::max(1, std::min(2048 / tiles, P / 256));
    const int chunk = (P + chunks - 1) / chunks;
    g.chunk = (chunk + 15) / 16 * 16;
    e = launchConvWgrad(g, s);
  }
  if (e == cudaSuccess) e = launchBiasGrad(dy, L.cout, 0, L.cout, P, grad_ + L.b, s);
  if (dx) {
    ConvArgs a{};
    a.x = dy;
    a.xC = L.cout;
    a.Cin = L.cout;
    a.w = wt_ + L.wt;
    a.wPacked = wpk_ + L.wtp;
    a.Cout = L.cin;
    a.y = dx;
    a.yC = L.cin;
    a.mask = mask;
    a.maskC = L.cin;
    a.N = N;
    a.H = H;
    a.W = W;
    if (e == cudaSuccess) e = useTc(W) ? launchTc(a, s) : launchConv3x3(a, s);
  }
  return e;
}

cudaError_t Denoiser::run(const __nv_bfloat16 *x, int N, int H, int W, float *out, cudaStream_t s,
                          bool catOut) {
  FirstError E;
  const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
  const size_t P0 = (size_t)N * H * W, P1 = P0 / 4, P2 = P0 / 16;
  Act &A = act_;
  E(launchToBlocked(x, kInC, P0, A.x0, s));
  E(conv(L_E0A, A.x0, kInC, A.a0, nullptr, 32, N, H, W, true, s));
  E(conv(L_E0B, A.a0, 32, A.e0, nullptr, 32, N, H, W, true, s));
  E(launchMaxPool(A.e0, 32, N, H, W, A.p0, s));
  E(conv(L_E1A, A.p0, 32, A.a1, nullptr, 64, N, H1, W1, true, s));
  E(conv(L_E1B, A.a1, 64, A.e1, nullptr, 64, N, H1, W1, true, s));
  E(launchMaxPool(A.e1, 64, N, H1, W1, A.p1, s));
  E(conv(L_E2A, A.p1, 64, A.a2, nullptr, 128, N, H2, W2, true, s));
  E(conv(L_E2B, A.a2, 128, A.e2, nullptr, 128, N, H2, W2, true, s));
  E(launchMaxPool(A.e2, 128, N, H2, W2, A.p2, s));
  E(conv(L_E3A, A.p2, 128, A.a3, nullptr, 256, N, H3, W3, true, s));
  E(conv(L_E3B, A.a3, 256, A.e3, nullptr, 256, N, H3, W3, true, s));
  if (!catOut && useTc(W2)) {
    E(convCat(L_D2A, A.e3, 256, A.e2, 128, A.b2, 128, N, H2, W2, s));
  } else {
    E(launchUpsample(A.e3, 256, N, H3, W3, A.cat2, 384, 0, s));
    E(launchCopyChannels(A.e2, 128, 0, A.cat2, 384, 256, 128, P2, 0, s));
    E(conv(L_D2A, A.cat2, 384, A.b2, nullptr, 128, N, H2, W2, true, s));
  }
  E(conv(L_D2B, A.b2, 128, A.d2, nullptr, 128, N, H2, W2, true, s));
  if (!catOut && useTc(W1)) {
    E(convCat(L_D1A, A.d2, 128, A.e1, 64, A.b1, 64, N, H1, W1, s));
  } else {
    E(launchUpsample(A.d2, 128, N, H2, W2, A.cat1, 192, 0, s));
    E(launchCopyChannels(A.e1, 64, 0, A.cat1, 192, 128, 64, P1, 0, s));
    E(conv(L_D1A, A.cat1, 192, A.b1, nullptr, 64, N, H1, W1, true, s));
  }
  E(conv(L_D1B, A.b1, 64, A.d1, nullptr, 64, N, H1, W1, true, s));
  if (!catOut && useTc(W)) {
    E(convCat(L_D0A, A.d1, 64, A.e0, 32, A.b0, 32, N, H, W, s));
  } else {
    E(launchUpsample(A.d1, 64, N, H1, W1, A.cat0, 96, 0, s));
    E(launchCopyChannels(A.e0, 32, 0, A.cat0, 96, 64, 32, P0, 0, s));
    E(conv(L_D0A, A.cat0, 96, A.b0, nullptr, 32, N, H, W, true, s));
  }
  E(conv(L_D0B, A.b0, 32, A.d0, nullptr, 32, N, H, W, true, s));
  // the output is a correction of the input's log(1 + colour)
  E(conv(L_OUT, A.d0, 32, nullptr, out, kOutC, N, H, W, false, s, A.x0));
  E(cudaGetLastError());
  return E.e;
}

cudaError_t Denoiser::forward(const __nv_bfloat16 *x, int N, int H, int W, float *out,
                              cudaStream_t s) {
  if (!ok_ || !x || N <= 0 || H <= 0 || W <= 0 || H % 8 || W % 8) return cudaErrorInvalidValue;
  cudaError_t e = ensure(N, H, W, false);
  if (e != cudaSuccess) return e;
  return run(x, N, H, W, out ? out : out_, s, false);
}

cudaError_t Denoiser::backward(const __nv_bfloat16 *x, const float *target, int tC, int N, int H,
                               int W, float *lossDevice, cudaStream_t s) {
  if (!ok_ || !x || !target || N <= 0 || H <= 0 || W <= 0 || H % 8 || W % 8 || tC < kColorC)
    return cudaErrorInvalidValue;
  cudaError_t e = ensure(N, H, W, true);
  if (e != cudaSuccess) return e;
  if ((e = run(x, N, H, W, out_, s, true)) != cudaSuccess) return e;
  FirstError E;
  const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
  const size_t P0 = (size_t)N * H * W, P1 = P0 / 4, P2 = P0 / 16;
  Act &A = act_, &G = grd_;
  E(cudaMemsetAsync(grad_, 0, numParams_ * sizeof(float), s));
  if (lossDevice) E(cudaMemsetAsync(lossDevice, 0, sizeof(float), s));
  E(launchL1(out_, kOutC, target, tC, kColorC, P0, gout_, kOutC, lossDevice, s));
  // decoder, level 0
  E(convBack(L_OUT, A.d0, 32, gout_, G.d0, A.d0, N, H, W, s));
  E(convBack(L_D0B, A.b0, 32, G.d0, G.b0, A.b0, N, H, W, s));
  E(convBack(L_D0A, A.cat0, 96, G.b0, G.cat0, A.cat0, N, H, W, s));
  E(launchUpsampleGrad(G.cat0, 96, 0, 64, N, H1, W1, nullptr, G.d1, s));
  // level 1
  E(convBack(L_D1B, A.b1, 64, G.d1, G.b1, A.b1, N, H1, W1, s));
  E(convBack(L_D1A, A.cat1, 192, G.b1, G.cat1, A.cat1, N, H1, W1, s));
  E(launchUpsampleGrad(G.cat1, 192, 0, 128, N, H2, W2, nullptr, G.d2, s));
  // level 2
  E(convBack(L_D2B, A.b2, 128, G.d2, G.b2, A.b2, N, H2, W2, s));
  E(convBack(L_D2A, A.cat2, 384, G.b2, G.cat2, A.cat2, N, H2, W2, s));
  E(launchUpsampleGrad(G.cat2, 384, 0, 256, N, H3, W3, nullptr, G.e3, s));
  // bottleneck, then the encoder: a pooled level gets its gradient from the
  // pooling and from its skip connection
  E(convBack(L_E3B, A.a3, 256, G.e3, G.a3, A.a3, N, H3, W3, s));
  E(convBack(L_E3A, A.p2, 128, G.a3, G.p2, A.p2, N, H3, W3, s));
  E(launchMaxPoolGrad(A.e2, G.p2, 128, N, H2, W2, nullptr, G.e2, s));
  E(launchCopyChannels(G.cat2, 384, 256, G.e2, 128, 0, 128, P2, 1, s));
  E(convBack(L_E2B, A.a2, 128, G.e2, G.a2, A.a2, N, H2, W2, s));
  E(convBack(L_E2A, A.p1, 64, G.a2, G.p1, A.p1, N, H2, W2, s));
  E(launchMaxPoolGrad(A.e1, G.p1, 64, N, H1, W1, nullptr, G.e1, s));
  E(launchCopyChannels(G.cat1, 192, 128, G.e1, 64, 0, 64, P1, 1, s));
  E(convBack(L_E1B, A.a1, 64, G.e1, G.a1, A.a1, N, H1, W1, s));
  E(convBack(L_E1A, A.p0, 32, G.a1, G.p0, A.p0, N, H1, W1, s));
  E(launchMaxPoolGrad(A.e0, G.p0, 32, N, H, W, nullptr, G.e0, s));
  E(launchCopyChannels(G.cat0, 96, 64, G.e0, 32, 0, 32, P0, 1, s));
  E(convBack(L_E0B, A.a0, 32, G.e0, G.a0, A.a0, N, H, W, s));
  E(convBack(L_E0A, A.x0, kInC, G.a0, nullptr, nullptr, N, H, W, s));
  E(cudaGetLastError());
  return E.e;
}

cudaError_t Denoiser::adam(float lr, cudaStream_t s) {
  ++step_;
  cudaError_t e = cudaSuccess;
  for (const DenoiseLayer &L : layers_) {
    if (e == cudaSuccess)
      e = launchAdam(params_ + L.w, m_ + L.w, v_ + L.w, grad_ + L.w, (size_t)L.cout * 9 * L.cin, lr,
                     0.9f, 0.999f, 1e-8f, step_, wbf_ + L.w, wt_ + L.wt, L.cin, L.cout, s);
    if (e == cudaSuccess)
      e = launchAdam(params_ + L.b, m_ + L.b, v_ + L.b, grad_ + L.b, L.cout, lr, 0.9f, 0.999f,
                     1e-8f, step_, nullptr, nullptr, 1, 1, s);
  }
  if (e == cudaSuccess) e = pack(s);
  return e;
}

}  // namespace vsr
