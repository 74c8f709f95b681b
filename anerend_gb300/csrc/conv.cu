// Probe convolution + hysteresis on CUDA cores in FP32 (probe_conv.comp:21-90).
//
// Every probe of a dispatch uses the same N ray directions, so the cosine weights are one table
// W[t][j] = max(0, dot(d_j, omega_t)) (0 where <= 1e-6, probe_conv.comp:296-299) shared by all probes, and
// the weight sum s_t = sum_j W[t][j] is shared too. The kernel stages W^T (N x 64) in shared memory once per
// CTA, then walks groups of four probes: their ray radiance is staged in shared memory and each thread
// accumulates one (probe, texel) pair, normalises by s_t and blends with the old atlas texel.
#include "ddgi_common.cuh"
#include "kernels.h"

namespace ddgi {

namespace {

constexpr int kConvProbes = 4;                       // probes per group
constexpr int kConvThreads = kConvProbes * kOctTexels;  // 256

__global__ void __launch_bounds__(256) k_conv_weights(int n, const float4* __restrict__ dirs, float* __restrict__ wt,
                                                      float* __restrict__ wsum) {
  // one block per texel, threads over the rays, the weight sum through a shared-memory tree
  __shared__ float part[256];
  int t = blockIdx.x;
  float3 omega = texelDirection(t % kOct, t / kOct);
  float s = 0.0f;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    float w = fmaxf(0.0f, dot3(xyz(dirs[j]), omega));
    if (!(w > 1e-6f)) w = 0.0f;
    wt[j * kOctTexels + t] = w;
    s += w;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) wsum[t] = part[0];
}

// kSmemW: the N x 64 weight table is staged in shared memory (N <= 512); otherwise it is read from global
// memory, where it stays L1/L2-resident (256 KB at N = 1024).
template <bool kSmemW>
__global__ void __launch_bounds__(kConvThreads) k_conv_fp32(GridGPU g, const float4* __restrict__ rayRad,
                                                            const float* __restrict__ wt,
                                                            const float* __restrict__ wsum,
                                                            void* __restrict__ atlas, int layerBegin,
                                                            int layerEnd, float hysteresis, uint32_t flags) {
  extern __shared__ float4 smem4[];
  const int N = g.N;
  const float* sW = wt;
  float4* sR = smem4;  // kConvProbes * N
  if (kSmemW) {
    float* w = reinterpret_cast<float*>(smem4);  // N * 64
    for (int i = threadIdx.x; i < N * kOctTexels; i += blockDim.x) w[i] = wt[i];
    sW = w;
    sR = smem4 + (N * kOctTexels) / 4;
  }
  const int t = threadIdx.x % kOctTexels;
  const int q = threadIdx.x / kOctTexels;
  const float ws = wsum[t];
  const int probesPerLayer = g.X * g.Z;
  const long long total = (long long)(layerEnd - layerBegin) * probesPerLayer;
  const long long groups = (total + kConvProbes - 1) / kConvProbes;
  const bool bake = (flags & DDGI_UBO_BAKE_MODE_ON_FLAG) != 0;
  for (long long grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    __syncthreads();  // sW ready / previous group's sR consumed
    // stage the radiance of the group's probes
    for (int i = threadIdx.x; i < kConvProbes * N; i += blockDim.x) {
      int qq = i / N, j = i % N;
      long long pl = grp * kConvProbes + qq;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (pl < total) {
        int layer = layerBegin + (int)(pl / probesPerLayer);
        int p = (int)(pl % probesPerLayer);
        int px = p % g.X, pz = p / g.X;
        int rx = px * g.bw + (j % g.bw);
        int ry = (layer * g.Z + pz) * g.bh + (j / g.bw);
        v = rayRad[(size_t)ry * g.rayW + rx];
      }
      sR[qq * N + j] = v;
    }
    __syncthreads();
    long long pl = grp * kConvProbes + q;
    if (pl >= total) continue;
    float ax = 0.f, ay = 0.f, az = 0.f;
    const float4* r = sR + q * N;
#pragma unroll 8
    for (int j = 0; j < N; ++j) {
      float w = sW[j * kOctTexels + t];
      float4 L = r[j];
      ax = fmaf(w, L.x, ax);
      ay = fmaf(w, L.y, ay);
      az = fmaf(w, L.z, az);
    }
    int layer = layerBegin + (int)(pl / probesPerLayer);
    int p = (int)(pl % probesPerLayer);
    int px = p % g.X, pz = p / g.X;
    int tx = t % kOct, ty = t / kOct;
    size_t ai = (size_t)(kProbePix * (layer * g.Z + pz) + 1 + ty) * g.atlasW + (kProbePix * px + 1 + tx);
    float4 old = loadTexel(atlas, g.atlasFmt, ai);
    float4 out;
    if (bake) {
      // probe_conv.comp:307-319: weighted accumulation with the stored weight in .w
      float tw = old.w + ws;
      float3 tot = f3(ax, ay, az) + xyz(old) * old.w;
      if (tw > 1e-6f) tot = tot / tw;
      out = make_float4(tot.x, tot.y, tot.z, tw);
    } else {
      // probe_conv.comp:321-326
      float3 res = f3(ax, ay, az);
      if (ws > 1e-6f) res = res / ws;
      float a = 1.0f - hysteresis;
      out = make_float4(res.x * a + old.x * hysteresis, res.y * a + old.y * hysteresis,
                        res.z * a + old.z * hysteresis, ws * a + old.w * hysteresis);
    }
    storeTexel(atlas, g.atlasFmt, ai, out);
  }
}

// ---- many grids in one launch -------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_conv_weights_batch(const ConvItem* __restrict__ items) {
  __shared__ float part[256];
  const ConvItem& it = items[blockIdx.y];
  const int n = it.g.N;
  int t = blockIdx.x;
  float3 omega = texelDirection(t % kOct, t / kOct);
  float s = 0.0f;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    float w = fmaxf(0.0f, dot3(xyz(it.dirs[j]), omega));
    if (!(w > 1e-6f)) w = 0.0f;
    it.wt[j * kOctTexels + t] = w;
    s += w;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) it.wsum[t] = part[0];
}

// Each block takes a contiguous range of probe groups (4 probes x 64 texels), so a block mostly stays
// inside one item; the item's N x 64 weight table is read through L1.
__global__ void __launch_bounds__(kConvThreads) k_conv_fp32_batch(const ConvItem* __restrict__ items, int numItems,
                                                                  long long totalGroups) {
  const int t = threadIdx.x % kOctTexels;
  const int q = threadIdx.x / kOctTexels;
  long long per = (totalGroups + gridDim.x - 1) / gridDim.x;
  long long g0 = (long long)blockIdx.x * per, g1 = min(totalGroups, g0 + per);
  for (long long grp = g0; grp < g1; ++grp) {
    int lo = 0, hi = numItems - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (items[mid].groupBegin <= grp) lo = mid; else hi = mid - 1;
    }
    const ConvItem& it = items[lo];
    const GridGPU& g = it.g;
    const int probesPerLayer = g.X * g.Z;
    long long pl = (grp - it.groupBegin) * kConvProbes + q;
    long long total = (long long)(it.layerEnd - it.layerBegin) * probesPerLayer;
    if (pl >= total) continue;
    int layer = it.layerBegin + (int)(pl / probesPerLayer);
    int p = (int)(pl % probesPerLayer);
    int px = p % g.X, pz = p / g.X;
    float ax = 0.f, ay = 0.f, az = 0.f;
    const float* W = it.wt;
    for (int j = 0; j < g.N; ++j) {
      int rx = px * g.bw + (j % g.bw);
      int ry = (layer * g.Z + pz) * g.bh + (j / g.bw);
      float4 L = __ldg(&it.rayRad[(size_t)ry * g.rayW + rx]);
      float w = __ldg(&W[j * kOctTexels + t]);
      ax = fmaf(w, L.x, ax);
      ay = fmaf(w, L.y, ay);
      az = fmaf(w, L.z, az);
    }
    const float ws = __ldg(&it.wsum[t]);
    int tx = t % kOct, ty = t / kOct;
    size_t ai = (size_t)(kProbePix * (layer * g.Z + pz) + 1 + ty) * g.atlasW + (kProbePix * px + 1 + tx);
    float4 old = loadTexel(it.atlas, g.atlasFmt, ai);
    float4 out;
    if (it.flags & DDGI_UBO_BAKE_MODE_ON_FLAG) {
      float tw = old.w + ws;
      float3 tot = f3(ax, ay, az) + xyz(old) * old.w;
      if (tw > 1e-6f) tot = tot / tw;
      out = make_float4(tot.x, tot.y, tot.z, tw);
    } else {
      float3 res = f3(ax, ay, az);
      if (ws > 1e-6f) res = res / ws;
      float h = it.hysteresis, a = 1.0f - h;
      out = make_float4(res.x * a + old.x * h, res.y * a + old.y * h, res.z * a + old.z * h, ws * a + old.w * h);
    }
    storeTexel(it.atlas, g.atlasFmt, ai, out);
  }
}

}  // namespace

long long convGroups(const GridGPU& g, int layerBegin, int layerEnd) {
  return ((long long)(layerEnd - layerBegin) * g.X * g.Z + kConvProbes - 1) / kConvProbes;
}

cudaError_t launchConvFp32Batch(const ConvItem* dItems, int numItems, long long totalGroups, cudaStream_t stream) {
  if (numItems <= 0 || totalGroups <= 0) return cudaSuccess;
  k_conv_weights_batch<<<dim3(kOctTexels, numItems), 256, 0, stream>>>(dItems);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long grid = (long long)sms * 8;
  if (grid > totalGroups) grid = totalGroups;
  k_conv_fp32_batch<<<(unsigned)grid, kConvThreads, 0, stream>>>(dItems, numItems, totalGroups);
  return cudaGetLastError();
}

cudaError_t launchConvWeights(int n, const float4* dirs, float* wt, float* wsum, cudaStream_t stream) {
  k_conv_weights<<<kOctTexels, 256, 0, stream>>>(n, dirs, wt, wsum);
  return cudaGetLastError();
}

cudaError_t launchConvFp32(const GridGPU& g, const float4* rayRad, const float* wt, const float* wsum,
                           void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags,
                           cudaStream_t stream) {
  if (layerEnd <= layerBegin) return cudaSuccess;
  const bool smemW = g.N <= 512;
  size_t smem = sizeof(float4) * (size_t)kConvProbes * g.N;
  if (smemW) smem += sizeof(float) * (size_t)g.N * kOctTexels;
  auto kern = smemW ? k_conv_fp32<true> : k_conv_fp32<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long groups = ((long long)(layerEnd - layerBegin) * g.X * g.Z + kConvProbes - 1) / kConvProbes;
  int perSm = smem <= 100 * 1024 ? 2 : 1;
  long long grid = (long long)sms * perSm;
  if (grid > groups) grid = groups;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, kConvThreads, smem, stream>>>(g, rayRad, wt, wsum, atlas, layerBegin, layerEnd, hysteresis,
                                                      flags);
  return cudaGetLastError();
}

}  // namespace ddgi
