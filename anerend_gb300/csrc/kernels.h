// Launch wrappers of the device kernels (trace.cu, conv.cu, translate.cu).
#pragma once
#include "ddgi_common.cuh"

namespace ddgi {

constexpr int kTraceThreads = 128;

struct Mat3 {
  float m[9];
};

cudaError_t launchLattice(int n, const float rot[9], float4* out, cudaStream_t stream);
cudaError_t launchTraceShade(const SceneGPU& s, const GridGPU& g, const FrameGPU& f, const float4* lattice,
                             const int* order, const void* atlasPrev, float4* rayRad, float4* rayDir, int* rayHit,
                             uint32_t* err, cudaStream_t stream);

// probe_conv.comp: weights table (N x 64, transposed) and per-texel weight sums from the lattice.
cudaError_t launchConvWeights(int n, const float4* dirs, float* wt, float* wsum, cudaStream_t stream);
// Convolution + hysteresis (or bake accumulation) of layers [layerBegin, layerEnd) into `atlas`.
cudaError_t launchConvFp32(const GridGPU& g, const float4* rayRad, const float* wt, const float* wsum,
                           void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags,
                           cudaStream_t stream);

// Tensor-core convolution (conv_tc.cu). rad16: planar 16-bit radiance (elemFmt 0 FP16, 1 BF16), row
// c * pTotal + p; N a multiple of 64. scratch: tcScratchBytes(N) bytes (16-bit weights + two sum rows).
size_t tcScratchBytes(int n);
cudaError_t launchConvTc(const GridGPU& g, int elemFmt, const void* rad16, int pTotal, const float4* dirs,
                         void* scratch, void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags,
                         uint32_t* err, cudaStream_t stream);
cudaError_t launchPackRays16(const GridGPU& g, int elemFmt, const float4* rayRad, void* out16, int layerBegin,
                             int layerEnd, int pTotal, cudaStream_t stream);

// Translation copy (IrradianceProbeTranslationPass.cpp:83-168): out = in shifted by (sx, sz) probes.
cudaError_t launchTranslate(const GridGPU& g, const void* in, void* out, int sx, int sz, cudaStream_t stream);
// Fill every texel of the atlas with (0,0,0,1) (clearConvTex, IrradianceProbeConvolvePass.cpp:9-47).
cudaError_t launchClearAtlas(const GridGPU& g, void* atlas, cudaStream_t stream);

}  // namespace ddgi
