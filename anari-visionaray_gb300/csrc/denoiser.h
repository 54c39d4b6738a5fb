// The learned denoiser: a 4-level U-Net of 3x3 convolutions (channels
// 32 -> 64 -> 128 -> 256, two convolutions per level, 2x2 max pooling,
// nearest 2x upsampling, skip connections by channel concatenation, ReLU),
// bf16 weights and activations with fp32 accumulation, trained with L1 on
// log(1 + colour) and Adam. Inputs: 16 channels per pixel (log(1 + colour),
// albedo, normal, depth / (1 + depth), log(1 + standard error of the mean
// luminance), 1 / sqrt(samples), four zeros); output: log(1 + colour)
// in the first 3 of 16 fp32 channels, as the input's log(1 + colour) plus
// the last convolution (a residual).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>

namespace vsr {

struct ConvArgs;

struct DenoiseLayer {
  int cin, cout;
  size_t w, b;  // offsets of weights [cout][9][cin] and bias [cout] in the parameter array
  size_t wt;    // offset of the flipped, transposed bf16 copy [cin][9][cout]
  size_t wp, wtp;  // offsets of the two copies packed for kConv3x3Ws (packConvWeights)
};

class Denoiser {
 public:
  static constexpr int kInC = 16, kOutC = 16, kColorC = 3;
  explicit Denoiser(uint64_t seed);
  ~Denoiser();
  bool ok() const { return ok_; }
  size_t numParams() const { return numParams_; }
  const std::vector<DenoiseLayer> &layers() const { return layers_; }

  // parameters in the canonical order (per layer: weights, then bias), fp32
  cudaError_t getParams(float *host, cudaStream_t s);
  cudaError_t setParams(const float *host, cudaStream_t s);

  // x: N x H x W x 16 bf16 (device), out: N x H x W x 16 fp32 (device);
  // H and W multiples of 8
  cudaError_t forward(const __nv_bfloat16 *x, int N, int H, int W, float *out, cudaStream_t s);
  // forward + backward: fp32 gradients into grad() (zeroed first), L1 loss
  // against the linear target colour (tC floats per pixel, first 3 used)
  cudaError_t backward(const __nv_bfloat16 *x, const float *target, int tC, int N, int H, int W,
                       float *lossDevice, cudaStream_t s);
  // one Adam step (beta 0.9 / 0.999, eps 1e-8) with the current gradients
  cudaError_t adam(float lr, cudaStream_t s);
  const float *grad() const { return grad_; }
  float *lossDevice() const { return loss_; }  // one device float for the loss
  // 0: convolutions on mma.sync (kConv3x3); 1: on tcgen05 (the
  // warp-specialised kConv3x3Ws with TMA loads) for images at least one
  // 128-pixel tile wide, mma.sync below that; 2: kConv3x3Ws at every width;
  // 3: as 1 with the one-tile-per-CTA kConv3x3Tc
  void setTensorPath(int path) { tensorPath_ = path; }
  int tensorPath() const { return tensorPath_; }
  unsigned *errorWord() const { return err_; }
  // timeout test: the next tcgen05 convolution launch runs with
  // ConvArgs::testStall set (one launch only)
  void armWaitTimeoutTest() { stallNext_ = true; }
  int steps() const { return step_; }

 private:
  // activations in channel-blocked planes (actAt, kernels.h); x0 is the
  // network input, converted from the caller's NHWC
  struct Act {
    __nv_bfloat16 *x0, *a0, *e0, *p0, *a1, *e1, *p1, *a2, *e2, *p2, *a3, *e3, *cat2, *b2, *d2,
        *cat1, *b1, *d1, *cat0, *b0, *d0;
  };
  cudaError_t ensure(int N, int H, int W, bool train);
  // catOut: write the decoders' concatenated inputs (the backward reads
  // them); without it the tcgen05 path reads the two parts directly
  cudaError_t run(const __nv_bfloat16 *x, int N, int H, int W, float *out, cudaStream_t s,
                  bool catOut);
  bool useTc(int W) const {
    return tensorPath_ == 2 || tensorPath_ == 4 ||
           ((tensorPath_ == 1 || tensorPath_ == 3) && W >= 128);
  }
  // the tcgen05 convolution: the persistent warp-specialised kernel with
  // TMA loads (kConv3x3Ws), or on path 3 one tile per CTA (kConv3x3Tc)
  cudaError_t launchTc(const ConvArgs &a, cudaStream_t s) const;
  cudaError_t convCat(int layer, const __nv_bfloat16 *coarse, int coarseC, const __nv_bfloat16 *skip,
               int skipC, __nv_bfloat16 *y, int yC, int N, int H, int W, cudaStream_t s);
  cudaError_t conv(int layer, const __nv_bfloat16 *x, int xC, __nv_bfloat16 *y, float *yf, int yC, int N,
            int H, int W, bool relu, cudaStream_t s, const __nv_bfloat16 *resid = nullptr);
  cudaError_t convBack(int layer, const __nv_bfloat16 *x, int xC, const __nv_bfloat16 *dy,
                __nv_bfloat16 *dx, const __nv_bfloat16 *mask, int N, int H, int W,
                cudaStream_t s);

  bool ok_ = false;
  std::vector<DenoiseLayer> layers_;
  size_t numParams_ = 0, numWt_ = 0;
  float *params_ = nullptr, *m_ = nullptr, *v_ = nullptr, *grad_ = nullptr, *loss_ = nullptr;
  unsigned *err_ = nullptr;
  float *wgradPart_ = nullptr;  // tcgen05 weight gradient: partial sums (tensor path 4)
  size_t wgradPartFloats_ = 0;
  int tensorPath_ = 2;  // tcgen05 at every level width (training crops reach 16 wide)
  mutable bool stallNext_ = false;
  __nv_bfloat16 *wbf_ = nullptr, *wt_ = nullptr, *wpk_ = nullptr;
  size_t numPacked_ = 0;
  // refresh the packed weight copies from wbf_ and wt_
  cudaError_t pack(cudaStream_t s);
  int step_ = 0;
  // activations (and, for training, their gradients), sized for (N, H, W)
  int n_ = 0, h_ = 0, w_ = 0;
  bool train_ = false;
  std::vector<void *> bufs_;
  Act act_{}, grd_{};
  float *out_ = nullptr;
  __nv_bfloat16 *gout_ = nullptr;
};

}  // namespace vsr
