// Per-frame render kernels: raycast (surfaces + emission-absorption ray
// marching) and pathtrace (NEE + AO + bounce state machine with Russian
// roulette), one thread per pixel in 16x8 pixel tiles for coherent primary
// rays. The per-pixel bodies are in render_pixel.cuh.
#include "render_pixel.cuh"
#include "kernels.h"

namespace vsr {

// Surfaces = false is the volume-only specialization (no traversal code,
// fewer registers); the launcher picks it for worlds without surfaces.
// Full = true adds the optional features (gradient shading, point and spot
// lights).
template <bool Count, bool Surfaces, bool Full>
__global__ void __launch_bounds__(VSR_RAYCAST_BLOCK_X * VSR_RAYCAST_BLOCK_Y,
                                 Full ? VSR_RAYCAST_FULL_MIN_BLOCKS : VSR_RAYCAST_MIN_BLOCKS)
    kRaycast(DScene S, DCamera C, DRenderer R, DFrame F, int stageTF) {
  extern __shared__ float4 sTF[];
  if (stageTF) {
    const DVolume &V = S.volumes[0];
    for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < V.tfSize; i += blockDim.x * blockDim.y)
      sTF[i] = V.tf[i];
    __syncthreads();
  }
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= F.width || y >= F.height) return;
  raycastPixel<Count, Surfaces, Full>(S, C, R, F, x, y, stageTF ? sTF : nullptr);
}

// Two register budgets of the same body: worlds with volumes keep more path
// state live during delta tracking and run faster with fewer resident
// blocks and fewer spills (64 registers); surface-only worlds with more
// blocks at 32 registers. Full = true adds the optional features (gradient
// shading of volume scatter events, point and spot lights).
template <bool Count, bool Volumes, bool Full>
__global__ void __launch_bounds__(16 * VSR_MEGA_BLOCK_Y,
                                 Volumes ? VSR_MEGA_MIN_BLOCKS_VOLUMES : VSR_MEGA_MIN_BLOCKS)
    kPathtrace(DScene S, DCamera C, DRenderer R, DFrame F) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= F.width || y >= F.height) return;
  if (F.sampleMask && !F.sampleMask[(size_t)y * F.width + x]) return;
  // grid z: the frame's sample chunks (1: the whole frame in one stream)
  pathtracePixel<Count, Full>(S, C, R, F, x, y, R.sampleChunks > 1 ? (int)blockIdx.z : -1);
}

__global__ void __launch_bounds__(256) kTaaResolve(DRenderer R, DFrame F) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= F.width || y >= F.height) return;
  taaResolvePixel(R, F, x, y);
}

__global__ void __launch_bounds__(256) kCombineChunks(DRenderer R, DFrame F) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= F.width || y >= F.height) return;
  if (F.sampleMask && !F.sampleMask[(size_t)y * F.width + x]) return;
  combineChunks(R, F, x, y);
}

static dim3 tileGrid(const DFrame &F, dim3 block) {
  return dim3((F.width + block.x - 1) / block.x, (F.height + block.y - 1) / block.y);
}

cudaError_t launchRaycast(const DScene &S, const DCamera &C, const DRenderer &R, const DFrame &F,
                          int stageTFSize, bool count, const MarchScratch *scratch,
                          cudaStream_t stream) {
  dim3 block(VSR_RAYCAST_BLOCK_X, VSR_RAYCAST_BLOCK_Y);
  size_t smem = stageTFSize > 0 ? sizeof(float4) * (size_t)stageTFSize : 0;
  const int stage = stageTFSize > 0;
  const dim3 grid = tileGrid(F, block);
  auto launch = [&](auto kernel) {
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kernel<<<grid, block, smem, stream>>>(S, C, R, F, stage);
  };
  // the full variant for gradient shading, and for point / spot lights,
  // spheres, cones, cylinders, quads or iso-surfaces on surfaces (volume-only worlds light nothing without gradient
  // shading)
  if (R.gradientShading || S.areaLights || S.attributes ||
      (S.hasSurfaces && (S.positionalLights || S.numAnalytic || S.quadGroups || S.numIso))) {
    if (count) launch(kRaycast<true, true, true>);
    else launch(kRaycast<false, true, true>);
  } else if (S.hasSurfaces) {
    if (count) launch(kRaycast<true, true, false>);
    else launch(kRaycast<false, true, false>);
  } else if (R.pixelSamples == 1 && scratch && !S.areaLights && !S.attributes) {
    // volume-only world: set-up, segments, combination (k_volume_march.cu)
    return launchVolumeMarch(S, C, R, F, stageTFSize, count, *scratch, stream);
  } else {
    if (count) launch(kRaycast<true, false, false>);
    else launch(kRaycast<false, false, false>);
  }
  return cudaGetLastError();
}

cudaError_t launchPathtrace(const DScene &S, const DCamera &C, const DRenderer &R, const DFrame &F,
                            bool count, cudaStream_t stream) {
  dim3 block(16, VSR_MEGA_BLOCK_Y);
  dim3 grid = tileGrid(F, block);
  const int chunks = R.sampleChunks > 1 ? R.sampleChunks : 1;
  if (chunks > 1 && !F.chunkOut) return cudaErrorInvalidValue;
  // chunked frames: every chunk of every pixel is a thread of one launch, so
  // the grid is chunks times longer and each thread's path loop chunks
  // times shorter (a shorter tail when the last blocks finish)
  grid.z = (unsigned)chunks;
  const bool full = S.positionalLights || S.numAnalytic || S.quadGroups || S.numIso ||
                    (S.numVolumes > 0 && R.gradientShading) || R.taa || S.attributes;
  if (R.taa && (!F.taaCurr || !F.taaPrev || !F.motionVec || chunks > 1))
    return cudaErrorInvalidValue;
  auto launch = [&](auto kernel) { kernel<<<grid, block, 0, stream>>>(S, C, R, F); };
  if (S.numVolumes > 0) {
    if (full) count ? launch(kPathtrace<true, true, true>) : launch(kPathtrace<false, true, true>);
    else count ? launch(kPathtrace<true, true, false>) : launch(kPathtrace<false, true, false>);
  } else {
    if (full) count ? launch(kPathtrace<true, false, true>) : launch(kPathtrace<false, false, true>);
    else count ? launch(kPathtrace<true, false, false>) : launch(kPathtrace<false, false, false>);
  }
  if (chunks > 1) {
    const dim3 cb(32, 8);
    kCombineChunks<<<tileGrid(F, cb), cb, 0, stream>>>(R, F);
  }
  if (R.taa) {
    // resolve, then this frame becomes the next one's history
    const dim3 cb(32, 8);
    kTaaResolve<<<tileGrid(F, cb), cb, 0, stream>>>(R, F);
    const size_t np = (size_t)F.width * F.height;
    cudaError_t e = cudaMemcpyAsync(F.taaPrev, F.taaCurr, np * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(F.taaPrevAlbedo, F.taaCurrAlbedo, np * 3 * sizeof(float),
                          cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

} // namespace vsr
