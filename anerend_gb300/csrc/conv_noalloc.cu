// Probe convolution for callers that cannot allocate device memory.
//
// ddgi_convolve_raw needs scratch for the cosine-weight table (N x 64 floats) and the 64 weight sums, and
// takes it from the stream-ordered allocator on every call. Some callers cannot allocate at the point
// where they run the probe update:
//   - renderers that reserve all device memory before the frame loop and forbid allocation inside a frame,
//     because cudaMalloc can synchronise the device and an allocator call can fail under memory pressure
//     in the middle of a frame;
//   - processes whose device memory is fully committed to a budget (a serving loop admitting work by HBM
//     footprint), where an extra allocation at update time could fail or push another request out.
// This file gives them ddgi_convolve_raw_noalloc: the same kernels, with the scratch in a file-scope
// __device__ array of fixed size (kNoAllocMaxRays x 64 + 64 floats = 131,328 bytes). Every GPU that loads
// the library holds that array until the process exits.
//
// The first call on a device looks up the array's device address with cudaGetSymbolAddress (with that
// device current) and caches it; make that first call before capturing the stream into a graph. All calls
// share the one array and it keeps the last call's contents. Each call rewrites every weight and weight sum
// it later reads (nothing accumulates in the scratch), so no clearing is needed; but calls that overlap on
// the GPU (different streams without ordering between them) race on the array and must be serialised by
// the caller.
#include "objects.h"

#include <mutex>

namespace {

constexpr int kNoAllocMaxRays = DDGI_NOALLOC_MAX_RAYS;
constexpr size_t kScratchFloats = (size_t)kNoAllocMaxRays * ddgi::kOctTexels + ddgi::kOctTexels;

static __device__ __align__(256) float g_convScratch[kScratchFloats];

constexpr int kMaxDevices = 64;
std::mutex g_scratchMu;
float* g_scratchPtr[kMaxDevices] = {};

// Device address of g_convScratch on the current device (looked up once per device).
int scratchAddress(float** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DDGI_EDEVICE;
  std::lock_guard<std::mutex> lk(g_scratchMu);
  if (!g_scratchPtr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_convScratch) != cudaSuccess || !p) return DDGI_EDEVICE;
    g_scratchPtr[dev] = static_cast<float*>(p);
  }
  *out = g_scratchPtr[dev];
  return DDGI_OK;
}

}  // namespace

extern "C" int ddgi_convolve_raw_noalloc(const DdgiGridDesc* desc, const void* rayRadiance, const float* dirs,
                                         void* atlas, int layerBegin, int layerEnd, uint32_t flags,
                                         void* stream) {
  // the same argument checks as ddgi_convolve_raw, then the one limit of the static scratch
  if (ddgi::detail::validateGridDesc(nullptr, desc) != DDGI_OK || !rayRadiance || !dirs || !atlas) return DDGI_EINVAL;
  if (layerBegin < 0 || layerEnd > desc->dims[1] || layerBegin > layerEnd) return DDGI_EINVAL;
  if (desc->raysPerProbe > kNoAllocMaxRays) return DDGI_EINVAL;  // the scratch holds the weights of that many rays
  float* scratch = nullptr;
  int rc = scratchAddress(&scratch);
  if (rc != DDGI_OK) return rc;
  const ddgi::GridGPU g = ddgi::detail::makeGridGPU(*desc);
  float* wt = scratch;
  float* wsum = scratch + (size_t)g.N * ddgi::kOctTexels;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = ddgi::launchConvWeights(g.N, (const float4*)dirs, wt, wsum, st);
  if (e == cudaSuccess)
    e = ddgi::launchConvFp32(g, rayRadiance, wt, wsum, atlas, layerBegin, layerEnd, desc->hysteresis,
                             flags, st);
  return e == cudaSuccess ? DDGI_OK : DDGI_EDEVICE;
}
