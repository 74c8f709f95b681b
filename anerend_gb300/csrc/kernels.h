// Launch wrappers of the device kernels (trace.cu, conv.cu, translate.cu).
#pragma once
#include "ddgi_common.cuh"

namespace ddgi {

constexpr int kTraceThreads = 128;

struct Mat3 {
  float m[9];
};


// Everything the trace of one grid needs; an array of these drives the persistent batched trace.
struct TraceItem {
  SceneGPU s;
  GridGPU g;
  FrameGPU f;
  const float4* lattice;  // written by the batched lattice kernel
  const double* latticeUnit;  // when set: the unrotated FP64 unit lattice (3 per direction), rotated per frame
  const float4* rayDirs;      // when set: 2 float4 per direction, its ray record (packRayDir), written with the lattice
  const int* order;       // 2N ints: the trace's direction order, then its inverse (the position of each direction)
  const void* atlasPrev;
  int atlasPairs;         // atlasPrev is aligned to a texel pair (32 B RGBA32F, 16 B RGBA16F): the lookups load pairs
  void* rayRad;  // ray images in g.rayFmt texels
  void* rayDir;
  int* rayHit;
  long long warpBegin;    // first warp of this item (its ray slots start at 32 * warpBegin)
  // Closest-hit seeding. A ray first tests a candidate triangle: the closest hit of its probe's ray in the
  // nearest direction of the last traced lattice. A candidate that is hit bounds the search from the start;
  // any candidate leaves the result unchanged (the closest hit, ties to the lowest id, whatever was tested
  // first). hitMemo == nullptr: no seeding and no memo; seedOn == 0: memo written but not read (first trace).
  float4* latticePrev;    // the lattice kernel saves the previous lattice here before writing the new one
  int* seedDir;           // per direction: the nearest direction of latticePrev
  int* hitMemo;           // per (probe, direction): the closest-hit record of the last trace, -1 for a miss
  // Shadow rays likewise first test the occluder of the shadow ray in the nearest previous direction (a
  // record of the BVH the shadow rays traverse); a shadowed ray that hits it needs no traversal.
  int* occMemo;           // per (probe, direction): the last shadow ray's occluder record, -1 if unshadowed
  int seedOn;
};

cudaError_t launchLattice(int n, const float rot[9], float4* out, cudaStream_t stream);
// The unrotated unit lattice of n directions in FP64 (3 doubles each), the part of every frame's lattice that
// does not depend on the rotation.
cudaError_t launchLatticeUnit(int n, double* out, cudaStream_t stream);
// Shading records (SceneGPU::shade) of the scene BVH's records, from the scene's index, vertex, mesh and
// instance records; `out` holds 3 * bvh.numTris float4.
cudaError_t launchShadingRecords(const SceneGPU& s, uint64_t numIndices, uint64_t numVerts, float4* out,
                                 uint32_t* err, cudaStream_t stream);
// Warps of one grid's trace for frame f (32 ray slots each).
long long traceWarps(const GridGPU& g, const FrameGPU& f);
// Device counters of one trace launch: closest-hit queue, shadow-list length, shadow queue, spare.
constexpr int kTraceCounters = 4;
// Scratch of one trace launch per ray slot: the hit record (16 B) and the shadow-list entry (32 B: the shadow
// ray's origin and ray id, then the shadowed radiance and the candidate / found occluder).
constexpr size_t kTraceScratchPerRay = 48;
// Records of a batched trace whose first warps travel in the kernel parameters (ItemsGlobal, trace.cu).
constexpr int kParamItems = 64;
// Lattices of every item (rotation per item), then the wavefront trace of all items' ray slots:
// closest-hit traversal, shading, shadow traversal, shadowed-ray resolve. dHits holds 32 * totalWarps float4,
// dShadow twice that. hItems / hRot: a single record and its rotation on the host, passed to every
// kernel by value (constant-bank reads; dItems and dRots are not read), otherwise the kernels read dItems and
// dRots. The lattice kernel zeroes dCounters, so no copy or memset runs ahead of the launches. hBegins: the
// records' first warps on the host (at most kParamItems of them are passed in the parameters; a captured
// launch must be re-captured when they change).
cudaError_t launchTraceBatch(const TraceItem* dItems, const Mat3* dRots, int numItems, int maxN, long long totalWarps,
                             unsigned long long* dCounters, float4* dHits, float4* dShadow, int blocks,
                             int refillLanes, bool wide, bool lightSpace, uint32_t* err, cudaStream_t stream,
                             const TraceItem* hItems = nullptr, const Mat3* hRot = nullptr,
                             const long long* hBegins = nullptr);


// Ray queries on one BVH: DdgiRay -> DdgiHit (closest or any hit), or, with `points`, the RT shadow pass's
// visibility mask along shadowDir. counter: one device word of scratch. recordIds: DdgiHit.triangle holds the
// hit's triangle record (BVH order) instead of its global id.
// light: with `points`, run them in light's light-space shadow BVH (light->shadow, sheared by light->shear*) along
// +z instead of `bvh`; shadowDir must be the normalised direction toward the light it was built for.
cudaError_t launchTraceRays(const BvhRef& bvh, bool wide, const DdgiRay* rays, long long count, bool anyHit,
                            DdgiHit* hits, const float4* points, float3 shadowDir, float* vis,
                            unsigned long long* counter, uint32_t* err, cudaStream_t stream, bool recordIds = false,
                            const SceneGPU* light = nullptr);
// Ambient term of G-buffer points from an atlas (deferred_tiled.comp:263-299), CLAMP_TO_EDGE sampling.
cudaError_t launchQueryIrradiance(const GridGPU& g, const FrameGPU& f, const void* atlas, const DdgiSurfacePoint* pts,
                                  long long count, float4* out, cudaStream_t stream);
// Specular GI mirror pass (mirror_reflections.rgen/.rchit/.rmiss): radiance and hit distance per G-buffer
// point, sampling `atlas` as the probe update does (REPEAT). scratch: mirrorScratchBytes(count) device bytes, 16-byte
// aligned; counter: one device word.
size_t mirrorScratchBytes(long long count);
cudaError_t launchMirror(const SceneGPU& s, const GridGPU& g, const FrameGPU& f, const void* atlas,
                         const DdgiMirrorPoint* pts, long long count, float4* out, void* scratch,
                         unsigned long long* counter, uint32_t* err, cudaStream_t stream);

// probe_conv.comp: weights table (N x 64, transposed) and per-texel weight sums from the lattice.
cudaError_t launchConvWeights(int n, const float4* dirs, float* wt, float* wsum, cudaStream_t stream);
// Convolution + hysteresis (or bake accumulation) of layers [layerBegin, layerEnd) into `atlas`.
cudaError_t launchConvFp32(const GridGPU& g, const void* rayRad, const float* wt, const float* wsum,
                           void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags,
                           cudaStream_t stream);

// FP32 convolution of many grids in one launch (conv.cu).
struct ConvItem {
  GridGPU g;
  const void* rayRad;  // g.rayFmt texels
  const float4* dirs;
  float* wt;        // N x 64 weights of this item (written by the weights kernel)
  float* wsum;
  void* atlas;
  int layerBegin, layerEnd;
  float hysteresis;
  uint32_t flags;
  long long groupBegin;  // first 32-probe tile of this item
};
// Tiles of tileProbes (16 or 32) probes of one grid's layer range; convTileProbes: the tile size for a launch
// over `probes` probes (32 when they fill the GPU twice over, else 16).
long long convGroups(const GridGPU& g, int layerBegin, int layerEnd, int tileProbes = 16);
int convTileProbes(long long probes);
cudaError_t launchConvFp32Batch(const ConvItem* dItems, int numItems, long long totalGroups, cudaStream_t stream,
                                int tileProbes = 16);

// Bounded device waits of the tensor-core convolution (DdgiWaitConfig): attempts per mbarrier wait before it
// gives up (0 means the default), and the test hook that makes each CTA's first accumulator wait wait for a
// phase no arrival completes, so that the timeout path runs.
struct WaitCfg {
  uint32_t spin = 1u << 22;
  uint32_t stall = 0;
};

// Tensor-core convolution (conv_tc.cu). rad16: planar 16-bit radiance (elemFmt 0 FP16, 1 BF16), row
// c * pTotal + p; N a multiple of 64. scratch: tcScratchBytes(N) bytes (16-bit weights + two sum rows).
size_t tcScratchBytes(int n);
int tcMaxItems();
// Host image of one tensor-core item: the device record bytes and its two tensor maps.
struct TcItemHost {
  alignas(64) unsigned char mapR[128];
  alignas(64) unsigned char mapW[128];
  alignas(16) unsigned char item[128];
  int units;  // 64-probe work units of the item
};
bool tcPrepareItem(const GridGPU& g, int elemFmt, const void* rad16, int pTotal, const float4* dirs, void* scratch,
                   void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags, int unitBegin,
                   TcItemHost* out);
cudaError_t launchConvTcItems(int elemFmt, const TcItemHost* hostItems, const void* dItems, int numItems,
                              int totalUnits, uint32_t* err, cudaStream_t stream, WaitCfg waits = WaitCfg{});
cudaError_t launchConvTc(const GridGPU& g, int elemFmt, const void* rad16, int pTotal, const float4* dirs,
                         void* scratch, void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags,
                         uint32_t* err, cudaStream_t stream, WaitCfg waits = WaitCfg{});
cudaError_t launchPackRays16(const GridGPU& g, int elemFmt, const void* rayRad, void* out16, int layerBegin,
                             int layerEnd, int pTotal, cudaStream_t stream);

// Translation copy (IrradianceProbeTranslationPass.cpp:83-168): out = in shifted by (sx, sz) probes.
cudaError_t launchTranslate(const GridGPU& g, const void* in, void* out, int sx, int sz, cudaStream_t stream);
// RGBA32F <-> RGBA16F texel conversion (round to nearest even) of `texels` atlas texels.
cudaError_t launchAtlasToHalf(const float4* in, void* out, long long texels, cudaStream_t stream);
cudaError_t launchAtlasFromHalf(const void* in, float4* out, long long texels, cudaStream_t stream);
// Fill every texel of the atlas with (0,0,0,1) (clearConvTex, IrradianceProbeConvolvePass.cpp:9-47).
cudaError_t launchClearAtlas(const GridGPU& g, void* atlas, cudaStream_t stream);

}  // namespace ddgi
