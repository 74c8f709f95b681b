// Many probe grids updated together: the batched form of the three passes.
//
// batchLaunch runs, for every (grid, scene, frame) item, the translation (host decision + copy kernel,
// outside the captured part), then one persistent trace launch whose warps pull work from a single queue
// spanning all items' rays (the wavefront kernels of launchTraceBatch), then one convolution launch over
// all items (tensor cores: k_conv_tc over every item's 64-probe units; FP32: k_conv_fp32_batch). The per-item records (grid, frame, scene
// views, atlas pointers) are copied from pinned host memory into device records before the launches, so the
// launch sequence itself only depends on the batch's shape; once the same shape repeats it is captured into a
// CUDA graph and replayed. A LaunchState owns the records, their staging and the captured graph; DdgiBatch
// (a fixed item set) and the serving loop (a new item set per launch) both drive it.
#include "objects.h"

#include <algorithm>
#include <cstring>
#include <new>

using namespace ddgi::detail;

namespace ddgi {
namespace detail {

struct LaunchState {
  DdgiContext* ctx = nullptr;
  int cap = 0;
  // device records, one block: cap TraceItem | cap Mat3 | cap ConvItem | cap x 128-byte TcItem
  unsigned char* dRec = nullptr;
  size_t offRots = 0, offConv = 0, offTc = 0, recBytes = 0;
  unsigned long long* dQueue = nullptr;  // kTraceCounters trace counters
  float4* dHits = nullptr;               // trace scratch: hit records, then shadow list (rayCap each)
  float4* dShadow = nullptr;
  long long rayCap = 0;
  StagingRing ring;  // pinned host images of the record block
  std::vector<TcItemHost> tcHost;
  std::vector<long long> begins;  // the records' first warps, in launch order
  cudaStream_t captureStream = nullptr;  // the caller's stream may be the uncapturable legacy stream
  cudaGraphExec_t exec = nullptr;
  std::vector<long long> shape, lastShape;

  TraceItem* dTrace() const { return reinterpret_cast<TraceItem*>(dRec); }
  Mat3* dRots() const { return reinterpret_cast<Mat3*>(dRec + offRots); }
  ConvItem* dConv() const { return reinterpret_cast<ConvItem*>(dRec + offConv); }
  unsigned char* dTc() const { return dRec + offTc; }

  void dropGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    lastShape.clear();
  }
  void release() {
    dropGraph();
    if (captureStream) cudaStreamDestroy(captureStream);
    captureStream = nullptr;
    cudaFree(dRec);
    cudaFree(dQueue);
    cudaFree(dHits);
    dRec = nullptr;
    dQueue = nullptr;
    dHits = dShadow = nullptr;
    rayCap = 0;
    ring.release();
    cap = 0;
  }
  // Capacity for n items; growing synchronizes the device (cudaFree), so callers reserve ahead.
  int reserve(int n) {
    if (n <= cap) return DDGI_OK;
    DdgiContext* c = ctx;
    int newCap = std::max(n, std::max(64, 2 * cap));
    dropGraph();
    if (dRec) cudaFree(dRec);
    dRec = nullptr;
    ring.release();
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    offRots = align(sizeof(TraceItem) * newCap);
    offConv = offRots + align(sizeof(Mat3) * newCap);
    offTc = offConv + align(sizeof(ConvItem) * newCap);
    recBytes = offTc + 128 * (size_t)newCap;
    cudaError_t e = cudaMalloc(&dRec, recBytes);
    if (e == cudaSuccess && !dQueue) e = cudaMalloc(&dQueue, kTraceCounters * sizeof(unsigned long long));
    if (e == cudaSuccess) e = ring.init(recBytes);
    if (e == cudaSuccess && !captureStream) e = cudaStreamCreateWithFlags(&captureStream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cudaFail(c, e, "launch records");
    cap = newCap;
    return DDGI_OK;
  }
  // Trace scratch for `rays` ray slots; growing drops the captured graph (its kernels hold the pointers).
  int reserveRays(long long rays) {
    if (rays <= rayCap) return DDGI_OK;
    long long newCap = std::max(rays, rayCap + rayCap / 2);
    dropGraph();
    cudaFree(dHits);
    dHits = dShadow = nullptr;
    rayCap = 0;
    cudaError_t e = cudaMalloc(&dHits, kTraceScratchPerRay * (size_t)newCap);
    if (e != cudaSuccess) return cudaFail(ctx, e, "trace scratch");
    dShadow = dHits + newCap;
    rayCap = newCap;
    return DDGI_OK;
  }
};

LaunchState* launchStateCreate(DdgiContext* ctx) {
  LaunchState* s = new (std::nothrow) LaunchState();
  if (s) s->ctx = ctx;
  return s;
}

void launchStateDestroy(LaunchState* s) {
  if (!s) return;
  s->release();
  delete s;
}

int launchStateReserve(LaunchState* s, int n) { return s->reserve(n); }

namespace {

// Records the launch sequence on `st` (eagerly or under capture).
int issue(LaunchState* S, const DdgiBatchTuning& t, int n, int maxN, long long totalWarps, long long totalGroups,
          int totalUnits, cudaStream_t st) {
  DdgiContext* ctx = S->ctx;
  int blocks = ctx->numSms * t.blocksPerSm;
  CK(launchTraceBatch(S->dTrace(), S->dRots(), n, maxN, totalWarps, S->dQueue, S->dHits, S->dShadow, blocks,
                      t.refillLanes, t.bvhWidth != 2, t.shadowMode == 1, ctx->dErr, st, nullptr, nullptr,
                      S->begins.data()),
     "batched trace");
  if (t.convMode != 0) {
    int fmt = t.convMode == 1 ? DDGI_ELEM_F16 : DDGI_ELEM_BF16;
    CK(launchConvTcItems(fmt, S->tcHost.data(), S->dTc(), n, totalUnits, ctx->dErr, st, ctx->waits),
       "batched tensor-core convolve");
  } else {
    CK(launchConvFp32Batch(S->dConv(), n, totalGroups, st), "batched convolve");
  }
  return DDGI_OK;
}

}  // namespace

int batchLaunch(DdgiContext* ctx, LaunchState* S, const DdgiBatchTuning& t, DdgiGrid* const* grids,
                DdgiScene* const* scenes, const DdgiFrame* frames, int n, cudaStream_t st, bool allowGraph,
                DdgiBatchStats* stats) {
  if (n <= 0) return DDGI_OK;
  const bool tc = t.convMode != 0;
  if (tc && n > tcMaxItems()) return fail(ctx, DDGI_EINVAL, "tensor-core launches hold at most %d items", tcMaxItems());
  int rc = S->reserve(n);
  if (rc) return rc;
  const int fmt = t.convMode == 1 ? DDGI_ELEM_F16 : DDGI_ELEM_BF16;
  if (tc && (int)S->tcHost.size() < n) S->tcHost.resize(n);
  long long warps = 0, groups = 0, rays = 0;
  int units = 0, maxN = 0, moved = 0;
  S->begins.assign(n, 0);
  int slot = 0;
  unsigned char* rec = S->ring.acquire(&slot);
  TraceItem* hTrace = reinterpret_cast<TraceItem*>(rec);
  Mat3* hRots = reinterpret_cast<Mat3*>(rec + S->offRots);
  ConvItem* hConv = reinterpret_cast<ConvItem*>(rec + S->offConv);
  unsigned char* hTc = rec + S->offTc;
  // launch order: the items grouped by scene (stable), so the rays in flight at any time, and the hits being
  // shaded, share one scene's BVH and records in L2; each item's results do not depend on the order
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return scenes[a] < scenes[b]; });
  for (int k = 0; k < n; ++k) {
    const int i = perm[k];
    DdgiGrid* g = grids[i];
    DdgiScene* sc = scenes[i];
    const DdgiFrame& fr = frames[i];
    FrameGPU f{};
    rc = frameToGPU(ctx, &fr, f);
    if (rc) return rc;
    setFrameGrid(f, g->g);
    if (!(fr.flags & DDGI_UBO_BAKE_MODE_ON_FLAG)) {  // the translation pass (TranslationPass.cpp:59)
      int mv = 0;
      rc = translateGrid(g, fr.cameraPos, &mv, st);
      if (rc) return rc;
      moved += mv;
    }
    int lb, le;
    rc = layerRange(g, fr.layer, true, lb, le);
    if (rc) return rc;
    f.layerBegin = lb;
    f.layerEnd = le;
    SceneGPU view = sc->view;
    if (t.shadowMode == 1) {
      rc = ensureShadowBvh(sc, fr.lightDir, st);
      if (rc) return rc;
      view = sc->view;
    } else {
      view.shadow = BvhRef{};
    }
    GridGPU gg = g->g;
    if (tc) {
      gg.rad16 = g->rad16;
      gg.rad16Fmt = fmt;
      gg.pTotal = g->g.X * g->g.Y * g->g.Z;
    }
    TraceItem& ti = hTrace[k];
    ti.s = view;
    ti.g = gg;
    ti.f = f;
    ti.lattice = g->lattice;
    ti.latticeUnit = g->latticeUnit;
    // no direction records: with the records in global memory a batched refill reads the item's record for
    // them, which measured slower than computing the direction part of each ray
    ti.rayDirs = nullptr;
    ti.order = g->order;
    ti.atlasPrev = g->atlas[g->cur];
    ti.atlasPairs = ((uintptr_t)ti.atlasPrev & (g->g.atlasFmt == DDGI_FORMAT_RGBA32F ? 31 : 15)) == 0;
    ti.rayRad = g->rayRad;
    ti.rayDir = g->rayDir;
    ti.rayHit = g->rayHit;
    ti.warpBegin = warps;
    S->begins[k] = warps;
    ti.latticePrev = g->latticePrev;
    ti.seedDir = g->seedDir;
    ti.hitMemo = g->hitMemo;
    ti.occMemo = g->occMemo;
    ti.seedOn = g->memoValid ? 1 : 0;
    warps += traceWarps(gg, f);
    rays += (long long)(le - lb) * g->g.X * g->g.Z * g->g.N;
    memcpy(hRots[k].m, fr.rotation, sizeof(float) * 9);
    maxN = std::max(maxN, g->g.N);
    if (tc) {
      TcItemHost& h = S->tcHost[k];
      if (!tcPrepareItem(g->g, fmt, g->rad16, gg.pTotal, g->lattice, g->tcScratch, g->atlas[g->cur], lb, le,
                         g->desc.hysteresis, fr.flags, units, &h))
        return fail(ctx, DDGI_EINVAL, "tensor-core item %d could not be prepared", i);
      memcpy(hTc + 128 * (size_t)k, h.item, 128);
      units += h.units;
    } else {
      ConvItem& ci = hConv[k];
      ci.g = g->g;
      ci.rayRad = g->rayRad;
      ci.dirs = g->lattice;
      ci.wt = g->wt;
      ci.wsum = g->wsum;
      ci.atlas = g->atlas[g->cur];
      ci.layerBegin = lb;
      ci.layerEnd = le;
      ci.hysteresis = g->desc.hysteresis;
      ci.flags = fr.flags;
      ci.groupBegin = groups;
      groups += convGroups(g->g, lb, le);
    }
    g->tracedBegin = lb;
    g->tracedEnd = le;
    g->latticeValid = true;
    g->memoValid = g->hitMemo != nullptr;
    g->rad16Written = tc;
  }
  rc = S->reserveRays(32 * warps);
  if (rc) return rc;
  CK(S->ring.copy(slot, S->dRec, S->recBytes, st), "launch records");
  if (stats) {
    stats->rays = (uint64_t)rays;
    stats->translations = (uint32_t)moved;
  }
  // the captured sequence depends only on these (per-item values live in the device records)
  S->shape = {n, maxN, warps, groups, units, t.convMode, t.blocksPerSm, t.refillLanes, t.bvhWidth};
  S->shape.insert(S->shape.end(), S->begins.begin(), S->begins.end());  // captured in the trace's parameters
  const bool stable = allowGraph && t.useGraph && S->shape == S->lastShape;
  if (stable && !S->exec) {
    cudaGraph_t graph = nullptr;
    cudaStream_t cs = S->captureStream;
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
    rc = issue(S, t, n, maxN, warps, groups, units, cs);
    cudaError_t ce = cudaStreamEndCapture(cs, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ce != cudaSuccess) return cudaFail(ctx, ce, "end capture");
    ce = cudaGraphInstantiate(&S->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      S->exec = nullptr;
      return cudaFail(ctx, ce, "graph instantiate");
    }
  }
  if (stable && S->exec) {
    CK(cudaGraphLaunch(S->exec, st), "graph launch");
    if (stats) stats->graphLaunches++;
  } else {
    if (S->exec) S->dropGraph();
    rc = issue(S, t, n, maxN, warps, groups, units, st);
    if (rc) return rc;
    if (stats) stats->eagerLaunches++;
  }
  S->lastShape = S->shape;
  return DDGI_OK;
}

int checkBatchTuning(DdgiContext* ctx, const DdgiBatchTuning& t) {
  if (t.warpProbes < 1 || t.warpProbes > 32 || (t.warpProbes & (t.warpProbes - 1)))
    return fail(ctx, DDGI_EINVAL, "batch warpProbes %d must be a power of two in [1, 32]", t.warpProbes);
  if (t.blocksPerSm < 1 || t.blocksPerSm > 8) return fail(ctx, DDGI_EINVAL, "blocksPerSm must be in [1, 8]");
  if (t.refillLanes < 1 || t.refillLanes > 32) return fail(ctx, DDGI_EINVAL, "refillLanes must be in [1, 32]");
  if (t.convMode < 0 || t.convMode > 2) return fail(ctx, DDGI_EINVAL, "convMode %d unknown", t.convMode);
  if (t.rayOrder != 0 && t.rayOrder != 1) return fail(ctx, DDGI_EINVAL, "rayOrder %d unknown", t.rayOrder);
  if (t.shadowMode != 0 && t.shadowMode != 1) return fail(ctx, DDGI_EINVAL, "shadowMode %d unknown", t.shadowMode);
  if (t.bvhWidth != 0 && t.bvhWidth != 2 && t.bvhWidth != 8)
    return fail(ctx, DDGI_EINVAL, "bvhWidth %d must be 2 or 8 (0 = 8)", t.bvhWidth);
  return DDGI_OK;
}

// Applies a batch tuning's per-grid part to one grid.
int tuneGridForBatch(DdgiGrid* g, const DdgiBatchTuning& t) {
  DdgiTuning gt = g->tuning;
  gt.warpProbes = std::max(t.warpProbes, std::max(1, 32 / g->g.N));
  gt.rayOrder = t.rayOrder;
  gt.shadowMode = t.shadowMode;
  gt.convMode = t.convMode;
  gt.bvhWidth = t.bvhWidth;
  gt.refillLanes = t.refillLanes;
  return applyTuning(g, gt);
}

DdgiBatchTuning defaultBatchTuning() {
  DdgiBatchTuning t{};
  t.warpProbes = 2;
  t.rayOrder = 1;
  t.shadowMode = 1;
  t.convMode = 0;
  t.blocksPerSm = 8;
  t.refillLanes = 8;
  t.useGraph = 1;
  t.bvhWidth = 8;
  return t;
}

}  // namespace detail
}  // namespace ddgi

struct DdgiBatch {
  DdgiContext* ctx = nullptr;
  std::vector<DdgiGrid*> grids;
  std::vector<DdgiScene*> scenes;
  DdgiBatchTuning tuning{};
  LaunchState* state = nullptr;
  DdgiBatchStats stats{};
};

namespace {

int applyBatchTuning(DdgiBatch* b, const DdgiBatchTuning& t) {
  DdgiContext* ctx = b->ctx;
  int rc = checkBatchTuning(ctx, t);
  if (rc) return rc;
  if (t.convMode != 0 && (int)b->grids.size() > tcMaxItems())
    return fail(ctx, DDGI_EINVAL, "tensor-core batches hold at most %d items", tcMaxItems());
  for (DdgiGrid* g : b->grids) {
    rc = tuneGridForBatch(g, t);
    if (rc) return rc;
  }
  b->tuning = t;
  b->state->dropGraph();
  return DDGI_OK;
}

}  // namespace

extern "C" {

int ddgi_batch_create(DdgiContext* ctx, const DdgiBatchItem* items, int n, DdgiBatch** out) {
  if (!ctx || !items || n <= 0 || !out) return fail(ctx, DDGI_EINVAL, "bad arguments to ddgi_batch_create");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!items[i].grid || !items[i].scene) return fail(ctx, DDGI_EINVAL, "batch item %d has no grid or scene", i);
    if (items[i].grid->ctx != ctx || items[i].scene->ctx != ctx)
      return fail(ctx, DDGI_EINVAL, "batch item %d belongs to another context", i);
    for (int k = 0; k < i; ++k)
      if (items[k].grid == items[i].grid) return fail(ctx, DDGI_EINVAL, "grid of item %d appears twice", i);
  }
  CK(cudaSetDevice(ctx->device), "set device");
  DdgiBatch* b = new (std::nothrow) DdgiBatch();
  if (!b) return fail(ctx, DDGI_ENOMEM, "host allocation");
  b->ctx = ctx;
  for (int i = 0; i < n; ++i) {
    b->grids.push_back(items[i].grid);
    b->scenes.push_back(const_cast<DdgiScene*>(items[i].scene));
  }
  b->state = launchStateCreate(ctx);
  int rc = b->state ? b->state->reserve(n) : fail(ctx, DDGI_ENOMEM, "host allocation");
  if (!rc) rc = applyBatchTuning(b, defaultBatchTuning());
  if (rc) {
    launchStateDestroy(b->state);
    delete b;
    return rc;
  }
  *out = b;
  return DDGI_OK;
}

void ddgi_batch_destroy(DdgiBatch* b) {
  if (!b) return;
  launchStateDestroy(b->state);
  delete b;
}

int ddgi_batch_get_tuning(const DdgiBatch* b, DdgiBatchTuning* out) {
  if (!b || !out) return DDGI_EINVAL;
  *out = b->tuning;
  return DDGI_OK;
}

int ddgi_batch_set_tuning(DdgiBatch* b, const DdgiBatchTuning* t) {
  if (!b || !t) return fail(b ? b->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_batch_set_tuning");
  return applyBatchTuning(b, *t);
}

int ddgi_batch_stats(const DdgiBatch* b, DdgiBatchStats* out) {
  if (!b || !out) return DDGI_EINVAL;
  *out = b->stats;
  return DDGI_OK;
}

int ddgi_batch_update(DdgiBatch* b, const DdgiFrame* frames, void* stream) {
  if (!b || !frames) return fail(b ? b->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_batch_update");
  return batchLaunch(b->ctx, b->state, b->tuning, b->grids.data(), b->scenes.data(), frames, (int)b->grids.size(),
                     (cudaStream_t)stream, true, &b->stats);
}

}  // extern "C"
