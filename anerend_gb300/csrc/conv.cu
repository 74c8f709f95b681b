// Probe convolution + hysteresis on CUDA cores in FP32 (probe_conv.comp:21-90).
//
// Every probe of a dispatch uses the same N ray directions, so the cosine weights are one table
// W[t][j] = max(0, dot(d_j, omega_t)) (0 where <= 1e-6, probe_conv.comp:296-299) shared by all probes, and
// the weight sum s_t = sum_j W[t][j] is shared too. A weights kernel writes W^T (N x 64) and s; the
// convolution kernel then works on tiles of 32 probes with a 4-probe x 4-texel register tile per thread,
// streaming the rays through shared memory in chunks of 16 (k_conv_fp32_batch). One launch covers many
// grids (a record per grid) or one grid passed by value (the raw entry points).
#include "ddgi_common.cuh"
#include "kernels.h"

namespace ddgi {

namespace {


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

// Many grids in one launch. The unit of work is a tile of 8 kPT probes of one item; a block of 128 threads
// computes the 8 kPT x 64 (probe, texel) block of a tile with a kPT-probe x 4-texel register tile per thread,
// so one shared-memory float4 of weights and kPT float4s of radiance feed 12 kPT FMAs. The rays are walked
// in chunks of 16: the next chunk's radiance and weights are fetched into registers while the current chunk
// is consumed from shared memory. Every (probe, texel) sum runs over j in order with fmaf, whatever the tile
// shape. kPT = 4 reads shared memory least per FMA; kPT = 2 keeps twice the warps resident when a launch has
// few tiles (an 8192-probe grid: 512 tiles of 16 probes instead of 256 of 32), which the latency of the
// shared-memory loads needs. convTileProbes picks one per launch.
constexpr int kTileThreads = 128;
constexpr int kChunk = 16;  // rays per chunk (the smallest raysPerProbe)
constexpr int kRStride = kChunk + 1;  // padded probe stride of the radiance chunk (bank spread)
constexpr int kWLoads = kChunk * kOctTexels / 4 / kTileThreads;       // 2 float4 per thread

// kSingle: one item, passed by value in `single` (the raw entry points, which own no device records).
// kPT: probes per thread (tiles of 8 kPT probes).
template <bool kSingle, int kPT>
__global__ void __launch_bounds__(kTileThreads, 4) k_conv_fp32_batch(const ConvItem* __restrict__ items, int numItems,
                                                                     long long totalTiles,
                                                                     const __grid_constant__ ConvItem single) {
  constexpr int kTileProbes = 8 * kPT;
  constexpr int kRLoads = kTileProbes * kChunk / kTileThreads;  // kPT float4 per thread
  __shared__ float4 sR[kTileProbes * kRStride];
  __shared__ float4 sW[kChunk * kOctTexels / 4];
  const int tg = threadIdx.x & 15;  // texels 4tg .. 4tg+3
  const int pg = threadIdx.x >> 4;  // probes kPT pg .. kPT pg + kPT - 1 of the tile
  for (long long tile = blockIdx.x; tile < totalTiles; tile += gridDim.x) {
    int lo = 0, hi = kSingle ? 0 : numItems - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (items[mid].groupBegin <= tile) lo = mid; else hi = mid - 1;
    }
    const ConvItem& it = kSingle ? single : items[lo];
    const GridGPU& g = it.g;
    const int probesPerLayer = g.X * g.Z;
    const long long total = (long long)(it.layerEnd - it.layerBegin) * probesPerLayer;
    const long long base = (tile - it.groupBegin) * kTileProbes;
    const int N = g.N;
    // this thread stages ray (j0 + tg) of probes pg + 8k of the tile (k < kRLoads): the texel index of each
    // probe's ray block in the ray image, -1 past the tile's probes
    long long rsrc[kRLoads];
#pragma unroll
    for (int k = 0; k < kRLoads; ++k) {
      long long pl = base + pg + 8 * k;
      rsrc[k] = -1;
      if (pl < total) {
        int layer = it.layerBegin + (int)(pl / probesPerLayer);
        int p = (int)(pl % probesPerLayer);
        int px = p % g.X, pz = p / g.X;
        rsrc[k] = (long long)((layer * g.Z + pz) * g.bh) * g.rayW + (long long)px * g.bw;
      }
    }
    const float4* W4 = reinterpret_cast<const float4*>(it.wt);
    const bool rays16 = g.rayFmt == DDGI_FORMAT_RGBA16F;  // the same for the whole item
    float4 rn[kRLoads], wn[kWLoads];
    auto fetch = [&](int j0) {
      const int j = j0 + tg;
      const long long off = (long long)(j >> (__ffs(g.bw) - 1)) * g.rayW + (j & (g.bw - 1));  // bw: a power of two
#pragma unroll
      for (int k = 0; k < kRLoads; ++k) {
        if (rsrc[k] < 0) {
          rn[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else if (rays16) {
          const uint2 raw = __ldg(reinterpret_cast<const uint2*>(it.rayRad) + rsrc[k] + off);
          const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
          const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&raw.y));
          rn[k] = make_float4(a.x, a.y, b.x, b.y);
        } else {
          rn[k] = __ldg(reinterpret_cast<const float4*>(it.rayRad) + rsrc[k] + off);
        }
      }
#pragma unroll
      for (int k = 0; k < kWLoads; ++k) wn[k] = __ldg(W4 + (size_t)j0 * (kOctTexels / 4) + threadIdx.x + k * kTileThreads);
    };
    float acc[kPT][4][3];
#pragma unroll
    for (int a = 0; a < kPT; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = acc[a][b][2] = 0.0f;
    fetch(0);
    for (int j0 = 0; j0 < N; j0 += kChunk) {
      __syncthreads();  // the previous chunk is consumed
#pragma unroll
      for (int k = 0; k < kRLoads; ++k) sR[(pg + 8 * k) * kRStride + tg] = rn[k];
#pragma unroll
      for (int k = 0; k < kWLoads; ++k) sW[threadIdx.x + k * kTileThreads] = wn[k];
      __syncthreads();
      if (j0 + kChunk < N) fetch(j0 + kChunk);
#pragma unroll 4
      for (int jj = 0; jj < kChunk; ++jj) {
        float4 w = sW[jj * (kOctTexels / 4) + tg];
        float wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int a = 0; a < kPT; ++a) {
          float4 L = sR[(kPT * pg + a) * kRStride + jj];
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            acc[a][b][0] = fmaf(wv[b], L.x, acc[a][b][0]);
            acc[a][b][1] = fmaf(wv[b], L.y, acc[a][b][1]);
            acc[a][b][2] = fmaf(wv[b], L.z, acc[a][b][2]);
          }
        }
      }
    }
    const bool bake = (it.flags & DDGI_UBO_BAKE_MODE_ON_FLAG) != 0;
    const float h = it.hysteresis, ha = 1.0f - h;
#pragma unroll
    for (int a = 0; a < kPT; ++a) {
      long long pl = base + kPT * pg + a;
      if (pl >= total) break;
      int layer = it.layerBegin + (int)(pl / probesPerLayer);
      int p = (int)(pl % probesPerLayer);
      int px = p % g.X, pz = p / g.X;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int t = 4 * tg + b;
        const float ws = __ldg(&it.wsum[t]);
        int tx = t % kOct, ty = t / kOct;
        size_t ai = (size_t)(kProbePix * (layer * g.Z + pz) + 1 + ty) * g.atlasW + (kProbePix * px + 1 + tx);
        float4 old = loadTexel(it.atlas, g.atlasFmt, ai);
        float4 out;
        if (bake) {
          // probe_conv.comp:307-319
          float tw = old.w + ws;
          float3 tot = f3(acc[a][b][0], acc[a][b][1], acc[a][b][2]) + xyz(old) * old.w;
          if (tw > 1e-6f) tot = tot / tw;
          out = make_float4(tot.x, tot.y, tot.z, tw);
        } else {
          // probe_conv.comp:321-326
          float3 res = f3(acc[a][b][0], acc[a][b][1], acc[a][b][2]);
          if (ws > 1e-6f) res = res / ws;
          out = make_float4(res.x * ha + old.x * h, res.y * ha + old.y * h, res.z * ha + old.z * h,
                            ws * ha + old.w * h);
        }
        storeTexel(it.atlas, g.atlasFmt, ai, out);
      }
    }
  }
}

}  // namespace

long long convGroups(const GridGPU& g, int layerBegin, int layerEnd, int tileProbes) {
  return ((long long)(layerEnd - layerBegin) * g.X * g.Z + tileProbes - 1) / tileProbes;
}

int convTileProbes(long long probes) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // 32-probe tiles once they fill two waves of 4 blocks per SM, else 16-probe tiles
  return probes >= 2LL * 4 * sms * 32 ? 32 : 16;
}

namespace {
template <bool kSingle, int kPT>
void launchTiles(const ConvItem* dItems, int numItems, long long tiles, const ConvItem& single, cudaStream_t stream) {
  int dev = 0, sms = 0, perSm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_conv_fp32_batch<kSingle, kPT>, kTileThreads, 0);
  long long grid = (long long)sms * (perSm > 0 ? perSm : 1);
  if (grid > tiles) grid = tiles;
  k_conv_fp32_batch<kSingle, kPT><<<(unsigned)grid, kTileThreads, 0, stream>>>(dItems, numItems, tiles, single);
}
}  // namespace

cudaError_t launchConvFp32Batch(const ConvItem* dItems, int numItems, long long totalGroups, cudaStream_t stream,
                                int tileProbes) {
  if (numItems <= 0 || totalGroups <= 0) return cudaSuccess;
  if (tileProbes != 16 && tileProbes != 32) return cudaErrorInvalidValue;
  k_conv_weights_batch<<<dim3(kOctTexels, numItems), 256, 0, stream>>>(dItems);
  if (tileProbes == 32) launchTiles<false, 4>(dItems, numItems, totalGroups, ConvItem{}, stream);
  else launchTiles<false, 2>(dItems, numItems, totalGroups, ConvItem{}, stream);
  return cudaGetLastError();
}

cudaError_t launchConvWeights(int n, const float4* dirs, float* wt, float* wsum, cudaStream_t stream) {
  k_conv_weights<<<kOctTexels, 256, 0, stream>>>(n, dirs, wt, wsum);
  return cudaGetLastError();
}

cudaError_t launchConvFp32(const GridGPU& g, const void* rayRad, const float* wt, const float* wsum,
                           void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags,
                           cudaStream_t stream) {
  if (layerEnd <= layerBegin) return cudaSuccess;
  ConvItem it{};
  it.g = g;
  it.rayRad = rayRad;
  it.wt = const_cast<float*>(wt);
  it.wsum = const_cast<float*>(wsum);
  it.atlas = atlas;
  it.layerBegin = layerBegin;
  it.layerEnd = layerEnd;
  it.hysteresis = hysteresis;
  it.flags = flags;
  it.groupBegin = 0;
  const int tp = convTileProbes((long long)(layerEnd - layerBegin) * g.X * g.Z);
  const long long tiles = convGroups(g, layerBegin, layerEnd, tp);
  if (tp == 32) launchTiles<true, 4>(nullptr, 1, tiles, it, stream);
  else launchTiles<true, 2>(nullptr, 1, tiles, it, stream);
  return cudaGetLastError();
}

}  // namespace ddgi
