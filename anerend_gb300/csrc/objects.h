// Internal objects of the C ABI (context, scene, grid) and the host helpers shared by api.cu and batch.cu.
#pragma once

#include "ddgi_common.cuh"
#include "kernels.h"
#include "lbvh.h"

#include <mutex>
#include <string>
#include <vector>

using namespace ddgi;

// Pinned host staging for per-launch records copied to the device with cudaMemcpyAsync: a ring of slots,
// each reused only after the copy that last read it has executed (an event per slot).
struct StagingRing {
  static constexpr int kSlots = 4;
  unsigned char* host = nullptr;
  size_t slotBytes = 0;
  cudaEvent_t done[kSlots] = {};
  int next = 0;

  cudaError_t init(size_t bytes) {
    slotBytes = (bytes + 255) & ~(size_t)255;
    cudaError_t e = cudaMallocHost(&host, slotBytes * kSlots);
    for (int i = 0; i < kSlots && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
    return e;
  }
  void release() {
    for (int i = 0; i < kSlots; ++i)
      if (done[i]) cudaEventDestroy(done[i]);
    if (host) cudaFreeHost(host);
    host = nullptr;
  }
  // A slot whose previous copy has finished (waits for it on the host).
  unsigned char* acquire(int* slot) {
    int s = next;
    next = (next + 1) % kSlots;
    cudaEventSynchronize(done[s]);
    *slot = s;
    return host + s * slotBytes;
  }
  // Copies `bytes` of slot `slot` to `dst` on `st` and marks the slot busy until the copy has run.
  cudaError_t copy(int slot, void* dst, size_t bytes, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(dst, host + slot * slotBytes, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(done[slot], st);
    return e;
  }
};


struct DdgiContext {
  int device = 0;
  int numSms = 0;
  uint32_t* dErr = nullptr;  // sticky device error word
  std::mutex mu;
  std::string err;
  ddgi::WaitCfg waits;                 // bounded device waits (ddgi_context_set_waits)
  DdgiAllocHook allocHook = nullptr;   // ddgi_context_set_alloc_hook
  void* allocUser = nullptr;
};

namespace ddgi {
namespace detail {
// The context's allocation hook: true when it refuses an allocation of `bytes` (no hook: never).
inline bool allocRefused(const DdgiContext* ctx, size_t bytes) {
  return ctx && ctx->allocHook && ctx->allocHook(ctx->allocUser, (uint64_t)bytes) != 0;
}
}  // namespace detail
}  // namespace ddgi

struct DdgiScene {
  DdgiContext* ctx = nullptr;
  DdgiPackedVertex* vertices = nullptr;
  uint32_t* indices = nullptr;
  DdgiMeshInfo* meshes = nullptr;
  InstanceGPU* instances = nullptr;
  DdgiMaterialInfo* materials = nullptr;
  LbvhResult bvh;
  float4* shade = nullptr;            // shading records of bvh's records (SceneGPU::shade)
  DdgiSceneInfo info{};
  SceneGPU view{};
  std::vector<InstanceGPU> hostInst;  // host copy (composed into the shadow BVH's transforms)
  uint64_t numIndices = 0, numVertices = 0;
  LbvhResult shadowBvh;               // built for shadowLight, rebuilt when the light direction changes
  float shadowLight[3] = {0, 0, 0};
  bool shadowValid = false;
  std::mutex mu;
};

struct DdgiGrid {
  DdgiContext* ctx = nullptr;
  DdgiGridDesc desc{};
  GridGPU g{};
  void* atlas[2] = {nullptr, nullptr};  // current atlas and the translation temp (swapped on a move)
  int cur = 0;
  void* rayRad = nullptr;   // ray images in g.rayFmt texels
  void* rayDir = nullptr;
  int* rayHit = nullptr;
  float4* lattice = nullptr;
  double* latticeUnit = nullptr;  // the unrotated unit lattice in FP64, 3 per direction, computed once
  float4* rayDirs = nullptr;      // per direction of the lattice its ray record (2 float4, packRayDir)
  int* order = nullptr;   // trace-kernel direction order (N ints), then its inverse (N ints)
  // closest-hit seeding (grids made by ddgi_grid_create; served grids trace once and keep none): the last
  // traced lattice, per direction the nearest direction of that lattice, and per (probe, direction) the
  // closest-hit record of the last trace (-1 for a miss)
  float4* latticePrev = nullptr;
  int* seedDir = nullptr;
  int* hitMemo = nullptr;
  int* occMemo = nullptr;  // per (probe, direction): the shadow ray's occluder record of a trace, -1 if unshadowed
  bool memoValid = false;  // hitMemo and occMemo hold a trace's records
  DdgiTuning tuning{};
  void* rad16 = nullptr;  // planar 16-bit radiance for the tensor-core convolution (3 x P x N)
  void* tcScratch = nullptr;
  float* wt = nullptr;    // N x 64 convolution weights (transposed)
  float* wsum = nullptr;  // 64 weight sums
  int rayH = 0;
  uint64_t atlasBytes = 0;
  uint64_t rayBytes = 0;  // one ray image
  // buffers bound by ddgi_grid_bind_external (the caller's; never freed here): the current atlas (slot 0),
  // the translation temp (slot 1), the ray images. With either atlas bound, translations copy instead of
  // swapping the two slots.
  bool extAtlas = false, extTemp = false, extRays = false, extDirs = false;
  int lastProbeIdx[2] = {0, 0};  // IrradianceProbeTranslationPass.h:17
  int currentLayer = 0;          // IrradianceProbeRayTracingPass _currentLayer
  int tracedBegin = 0, tracedEnd = 0;  // the "ProbeLayer" blackboard value, as a range
  bool latticeValid = false;
  bool rad16Written = false;  // the last trace also wrote the 16-bit radiance of its layers
  // allocation mode: served grids take their memory stream-ordered (cudaMallocAsync / cudaFreeAsync on
  // allocStream), so creating and freeing them never synchronizes the device
  bool asyncAlloc = false;
  cudaStream_t allocStream = nullptr;
  // counters and scratch of the single-grid trace (the batched trace kernels with one item, its record in
  // the kernel parameters), allocated on first use
  unsigned long long* dQueue = nullptr;  // kTraceCounters trace counters
  float4* dHits = nullptr;               // trace scratch for every ray slot of the grid (hit records,
  float4* dShadow = nullptr;             // then the shadow list)
  // asynchronous atlas download (allocated on first use): a stream-ordered device snapshot of the atlas,
  // copied to the host on dlStream after dlSnap; dlDone marks the end of the last copy to the host
  void* dlStage = nullptr;
  cudaStream_t dlStream = nullptr;
  cudaEvent_t dlSnap = nullptr, dlDone = nullptr;
  bool dlPending = false;
};

namespace ddgi {
namespace detail {

int fail(DdgiContext* ctx, int code, const char* fmt, ...);
int cudaFail(DdgiContext* ctx, cudaError_t e, const char* what);
int validateGridDesc(DdgiContext* ctx, const DdgiGridDesc* d);
GridGPU makeGridGPU(const DdgiGridDesc& d);
int applyTuning(DdgiGrid* g, const DdgiTuning& t);
int frameToGPU(DdgiContext* ctx, const DdgiFrame* f, FrameGPU& out);
int layerRange(DdgiGrid* grid, int layer, bool advance, int& b, int& e);
int ensureShadowBvh(DdgiScene* sc, const float lightDir[3], cudaStream_t st);
// translation state update of ddgi_translate without the C-ABI argument checks
int translateGrid(DdgiGrid* g, const float cameraPos[3], int* moved, cudaStream_t st);
// Grid construction / destruction; asyncAlloc: stream-ordered memory on `st`, no device synchronization.
int gridCreate(DdgiContext* ctx, const DdgiGridDesc* desc, cudaStream_t st, bool asyncAlloc, DdgiGrid** out);
void gridDestroy(DdgiGrid* g);
// Device bytes a grid of this description holds (atlas pair, ray images, lattice and weight tables and, for
// a tensor-core convolution, the 16-bit radiance and its weight scratch).
long long maxRaySlots(const GridGPU& g);
// hitSeeds: the grid keeps the closest-hit seeding buffers (grids of ddgi_grid_create; served grids do not)
uint64_t gridFootprint(const DdgiGridDesc* d, int convMode, bool hitSeeds);
// Batched launch of n (grid, scene, frame) items through a reusable launch state (records, staging, graph).
struct LaunchState;
LaunchState* launchStateCreate(DdgiContext* ctx);
void launchStateDestroy(LaunchState* s);
int launchStateReserve(LaunchState* s, int n);
int batchLaunch(DdgiContext* ctx, LaunchState* S, const DdgiBatchTuning& t, DdgiGrid* const* grids,
                DdgiScene* const* scenes, const DdgiFrame* frames, int n, cudaStream_t st, bool allowGraph,
                DdgiBatchStats* stats);
int checkBatchTuning(DdgiContext* ctx, const DdgiBatchTuning& t);
int tuneGridForBatch(DdgiGrid* g, const DdgiBatchTuning& t);
DdgiBatchTuning defaultBatchTuning();

}  // namespace detail
}  // namespace ddgi

#define CK(call, what)                                               \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return ::ddgi::detail::cudaFail(ctx, e_, what); \
  } while (0)

