// Probe translation (IrradianceProbeTranslationPass.cpp:56-186) as one integer-indexed gather.
//
// The reference copies the atlas into TempProbeTex and then copies, per layer plane, the rectangle that
// survives the camera step back with a shift of sign(dx), sign(dz) probes (10 texels):
//   dx > 0: src x + 10 -> dst x, dst x in [0, W - 10)      dx < 0: src x -> dst x + 10, dst x in [10, W)
//   dz > 0: src y + 10 -> dst y, dst y in [0, H_p - 10)    dz < 0: src y -> dst y + 10, dst y in [10, H_p)
// Texels outside the destination rectangle keep their old value. Here each output texel reads its source
// directly (out-of-place), which moves exactly 2 x atlas bytes. The plane height H_p is 10*Z; the reference
// writes `width` (10*X) there, which is the same value for the square planes it supports.
#include "ddgi_common.cuh"
#include "kernels.h"

namespace ddgi {

namespace {

template <typename T>
__global__ void k_translate(const T* __restrict__ in, T* __restrict__ out, int W, int H, int planeH, int sx,
                            int sz) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)W * H;
  for (; i < total; i += (long long)gridDim.x * blockDim.x) {
    int x = (int)(i % W), y = (int)(i / W);
    int yy = y % planeH;
    bool inX = sx > 0 ? (x < W - kProbePix) : (sx < 0 ? (x >= kProbePix) : true);
    bool inY = sz > 0 ? (yy < planeH - kProbePix) : (sz < 0 ? (yy >= kProbePix) : true);
    long long src = i;
    if (inX && inY) src = (long long)(y + sz * kProbePix) * W + (x + sx * kProbePix);
    out[i] = in[src];
  }
}

template <typename T>
__global__ void k_fill(T* __restrict__ out, long long total, T v) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i < total; i += (long long)gridDim.x * blockDim.x) out[i] = v;
}

int gridFor(long long total) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long b = (total + 255) / 256;
  long long cap = (long long)sms * 8;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

}  // namespace

cudaError_t launchTranslate(const GridGPU& g, const void* in, void* out, int sx, int sz, cudaStream_t stream) {
  long long total = (long long)g.atlasW * g.atlasH;
  int planeH = kProbePix * g.Z;
  if (g.atlasFmt == DDGI_FORMAT_RGBA32F)
    k_translate<float4><<<gridFor(total), 256, 0, stream>>>((const float4*)in, (float4*)out, g.atlasW, g.atlasH,
                                                            planeH, sx, sz);
  else
    k_translate<uint2><<<gridFor(total), 256, 0, stream>>>((const uint2*)in, (uint2*)out, g.atlasW, g.atlasH,
                                                           planeH, sx, sz);
  return cudaGetLastError();
}

cudaError_t launchClearAtlas(const GridGPU& g, void* atlas, cudaStream_t stream) {
  long long total = (long long)g.atlasW * g.atlasH;
  if (g.atlasFmt == DDGI_FORMAT_RGBA32F) {
    k_fill<float4><<<gridFor(total), 256, 0, stream>>>((float4*)atlas, total, make_float4(0.f, 0.f, 0.f, 1.f));
  } else {
    // half 1.0 = 0x3C00: (0,0) in .x, (0, 1.0) in .y
    uint2 v;
    v.x = 0u;
    v.y = 0x3C000000u;
    k_fill<uint2><<<gridFor(total), 256, 0, stream>>>((uint2*)atlas, total, v);
  }
  return cudaGetLastError();
}

// RGBA32F <-> RGBA16F atlas texels (round to nearest even), for persistence in the reference's layout.
__global__ void k_atlas_to_half(const float4* __restrict__ in, uint2* __restrict__ out, long long total) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const float4 v = in[i];
    __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
    out[i] = make_uint2(*reinterpret_cast<uint32_t*>(&a), *reinterpret_cast<uint32_t*>(&b));
  }
}
__global__ void k_atlas_from_half(const uint2* __restrict__ in, float4* __restrict__ out, long long total) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const uint2 u = in[i];
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    out[i] = make_float4(a.x, a.y, b.x, b.y);
  }
}

cudaError_t launchAtlasToHalf(const float4* in, void* out, long long texels, cudaStream_t stream) {
  k_atlas_to_half<<<gridFor(texels), 256, 0, stream>>>(in, (uint2*)out, texels);
  return cudaGetLastError();
}
cudaError_t launchAtlasFromHalf(const void* in, float4* out, long long texels, cudaStream_t stream) {
  k_atlas_from_half<<<gridFor(texels), 256, 0, stream>>>((const uint2*)in, out, texels);
  return cudaGetLastError();
}

}  // namespace ddgi
