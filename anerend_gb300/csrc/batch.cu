// Many probe grids updated together: the batched form of the three passes.
//
// A DdgiBatch holds a fixed set of (grid, scene) items. ddgi_batch_update runs, for every item, the
// translation (host decision + copy kernel, outside the captured part), then one persistent trace launch
// whose warps pull work from a single queue spanning all items' rays (k_trace_batch), then one convolution
// launch over all items (tensor cores: k_conv_tc over every item's tiles; FP32: k_conv_fp32_batch). The
// per-item records (grid, frame, scene views, atlas pointers) are copied from pinned host memory into device
// buffers before the launches, so the launch sequence itself only depends on the batch's shape; once the
// shape has been seen twice in a row it is captured into a CUDA graph and replayed.
#include "objects.h"

#include <algorithm>
#include <cstring>
#include <new>

using namespace ddgi::detail;

struct DdgiBatch {
  DdgiContext* ctx = nullptr;
  std::vector<DdgiBatchItem> items;
  DdgiBatchTuning tuning{};
  int sms = 0;
  // device records, one block: n TraceItem | n Mat3 | n ConvItem | n x 128-byte TcItem
  unsigned char* dRec = nullptr;
  size_t offRots = 0, offConv = 0, offTc = 0, recBytes = 0;
  TraceItem* dTrace = nullptr;
  Mat3* dRots = nullptr;
  ConvItem* dConv = nullptr;
  unsigned char* dTc = nullptr;
  unsigned long long* dQueue = nullptr;
  StagingRing ring;  // pinned host images of the record block
  std::vector<TcItemHost> tcHost;
  // captured launch sequence
  cudaGraphExec_t exec = nullptr;
  cudaStream_t captureStream = nullptr;  // the caller's stream may be the uncapturable legacy stream
  std::vector<long long> shape, lastShape;
  DdgiBatchStats stats{};
};

namespace {

void freeBatch(DdgiBatch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->captureStream) cudaStreamDestroy(b->captureStream);
  cudaFree(b->dRec);
  cudaFree(b->dQueue);
  b->ring.release();
  delete b;
}

int applyBatchTuning(DdgiBatch* b, const DdgiBatchTuning& t) {
  DdgiContext* ctx = b->ctx;
  if (t.warpProbes < 1 || t.warpProbes > 32 || (t.warpProbes & (t.warpProbes - 1)))
    return fail(ctx, DDGI_EINVAL, "batch warpProbes %d must be a power of two in [1, 32]", t.warpProbes);
  if (t.blocksPerSm < 1 || t.blocksPerSm > 8) return fail(ctx, DDGI_EINVAL, "blocksPerSm must be in [1, 8]");
  if (t.warpsPerFetch < 1 || t.warpsPerFetch > 64) return fail(ctx, DDGI_EINVAL, "warpsPerFetch must be in [1, 64]");
  if (t.convMode < 0 || t.convMode > 2) return fail(ctx, DDGI_EINVAL, "convMode %d unknown", t.convMode);
  if (t.convMode != 0 && (int)b->items.size() > tcMaxItems())
    return fail(ctx, DDGI_EINVAL, "tensor-core batches hold at most %d items", tcMaxItems());
  for (const DdgiBatchItem& it : b->items) {
    DdgiTuning gt = it.grid->tuning;
    gt.warpProbes = std::max(t.warpProbes, std::max(1, 32 / it.grid->g.N));
    gt.rayOrder = t.rayOrder;
    gt.shadowMode = t.shadowMode;
    gt.convMode = t.convMode;
    int rc = applyTuning(it.grid, gt);
    if (rc) return rc;
  }
  b->tuning = t;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  b->lastShape.clear();
  b->tcHost.clear();
  return DDGI_OK;
}

// Records the launch sequence on `st` (eagerly or under capture).
int issue(DdgiBatch* b, int n, int maxN, long long totalWarps, long long totalGroups, int totalTiles,
          cudaStream_t st) {
  DdgiContext* ctx = b->ctx;
  int blocks = b->sms * b->tuning.blocksPerSm;
  CK(launchTraceBatch(b->dTrace, b->dRots, n, maxN, totalWarps, b->dQueue, blocks, b->tuning.warpsPerFetch, ctx->dErr,
                      st),
     "batched trace");
  if (b->tuning.convMode != 0) {
    int fmt = b->tuning.convMode == 1 ? DDGI_ELEM_F16 : DDGI_ELEM_BF16;
    CK(launchConvTcItems(fmt, b->tcHost.data(), b->dTc, n, totalTiles, ctx->dErr, st), "batched tensor-core convolve");
  } else {
    CK(launchConvFp32Batch(b->dConv, n, totalGroups, st), "batched convolve");
  }
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
  b->items.assign(items, items + n);
  b->sms = ctx->numSms;
  auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
  b->offRots = align(sizeof(TraceItem) * n);
  b->offConv = b->offRots + align(sizeof(Mat3) * n);
  b->offTc = b->offConv + align(sizeof(ConvItem) * n);
  b->recBytes = b->offTc + 128 * (size_t)n;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&b->dRec, b->recBytes);
  if (e == cudaSuccess) e = cudaMalloc(&b->dQueue, sizeof(unsigned long long));
  if (e == cudaSuccess) e = b->ring.init(b->recBytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->captureStream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    b->dTrace = reinterpret_cast<TraceItem*>(b->dRec);
    b->dRots = reinterpret_cast<Mat3*>(b->dRec + b->offRots);
    b->dConv = reinterpret_cast<ConvItem*>(b->dRec + b->offConv);
    b->dTc = b->dRec + b->offTc;
  }
  if (e != cudaSuccess) {
    freeBatch(b);
    return cudaFail(ctx, e, "batch allocation");
  }
  DdgiBatchTuning t{};
  t.warpProbes = 2;
  t.rayOrder = 1;
  t.shadowMode = 1;
  t.convMode = 0;
  t.blocksPerSm = 8;
  t.warpsPerFetch = 4;
  t.useGraph = 1;
  int rc = applyBatchTuning(b, t);
  if (rc) {
    freeBatch(b);
    return rc;
  }
  *out = b;
  return DDGI_OK;
}

void ddgi_batch_destroy(DdgiBatch* b) {
  if (b) freeBatch(b);
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
  DdgiContext* ctx = b->ctx;
  cudaStream_t st = (cudaStream_t)stream;
  const int n = (int)b->items.size();
  const bool tc = b->tuning.convMode != 0;
  const int fmt = b->tuning.convMode == 1 ? DDGI_ELEM_F16 : DDGI_ELEM_BF16;
  if (tc && (int)b->tcHost.size() != n) b->tcHost.assign(n, TcItemHost{});
  long long warps = 0, groups = 0;
  int tiles = 0, maxN = 0, moved = 0;
  int slot = 0;
  unsigned char* rec = b->ring.acquire(&slot);
  TraceItem* hTrace = reinterpret_cast<TraceItem*>(rec);
  Mat3* hRots = reinterpret_cast<Mat3*>(rec + b->offRots);
  ConvItem* hConv = reinterpret_cast<ConvItem*>(rec + b->offConv);
  unsigned char* hTc = rec + b->offTc;
  b->shape.assign(1, n);
  for (int i = 0; i < n; ++i) {
    DdgiGrid* g = b->items[i].grid;
    DdgiScene* sc = const_cast<DdgiScene*>(b->items[i].scene);
    const DdgiFrame& fr = frames[i];
    FrameGPU f{};
    int rc = frameToGPU(ctx, &fr, f);
    if (rc) return rc;
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
    if (b->tuning.shadowMode == 1) {
      rc = ensureShadowBvh(sc, fr.lightDir, st);
      if (rc) return rc;
      view = sc->view;
    } else {
      view.shadowNodes = nullptr;
      view.shadowTris = nullptr;
    }
    GridGPU gg = g->g;
    if (tc) {
      gg.rad16 = g->rad16;
      gg.rad16Fmt = fmt;
      gg.pTotal = g->g.X * g->g.Y * g->g.Z;
    }
    TraceItem& ti = hTrace[i];
    ti.s = view;
    ti.g = gg;
    ti.f = f;
    ti.lattice = g->lattice;
    ti.order = g->order;
    ti.atlasPrev = g->atlas[g->cur];
    ti.rayRad = g->rayRad;
    ti.rayDir = g->rayDir;
    ti.rayHit = g->rayHit;
    ti.warpBegin = warps;
    warps += traceWarps(gg, f);
    memcpy(hRots[i].m, fr.rotation, sizeof(float) * 9);
    maxN = std::max(maxN, g->g.N);
    if (tc) {
      TcItemHost& h = b->tcHost[i];
      if (!tcPrepareItem(g->g, fmt, g->rad16, gg.pTotal, g->lattice, g->tcScratch, g->atlas[g->cur], lb, le,
                         g->desc.hysteresis, fr.flags, tiles, &h))
        return fail(ctx, DDGI_EINVAL, "tensor-core item %d could not be prepared", i);
      memcpy(hTc + 128 * (size_t)i, h.item, 128);
      tiles += h.tiles;
    } else {
      ConvItem& ci = hConv[i];
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
    g->rad16Written = tc;
  }
  // the captured sequence depends only on these (per-item values live in the device records)
  b->shape.push_back(maxN);
  b->shape.push_back(warps);
  b->shape.push_back(groups);
  b->shape.push_back(tiles);
  CK(b->ring.copy(slot, b->dRec, b->recBytes, st), "batch records");

  long long rays = 0;
  for (int i = 0; i < n; ++i) {
    const TraceItem& ti = hTrace[i];
    rays += (long long)(ti.f.layerEnd - ti.f.layerBegin) * ti.g.X * ti.g.Z * ti.g.N;
  }
  b->stats.rays = (uint64_t)rays;
  b->stats.translations = (uint32_t)moved;

  const bool stable = b->tuning.useGraph && b->shape == b->lastShape;
  if (stable && !b->exec) {
    cudaGraph_t graph = nullptr;
    cudaStream_t cs = b->captureStream;
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
    int rc = issue(b, n, maxN, warps, groups, tiles, cs);
    cudaError_t ce = cudaStreamEndCapture(cs, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ce != cudaSuccess) return cudaFail(ctx, ce, "end capture");
    ce = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      b->exec = nullptr;
      return cudaFail(ctx, ce, "graph instantiate");
    }
  }
  if (stable && b->exec) {
    CK(cudaGraphLaunch(b->exec, st), "graph launch");
    b->stats.graphLaunches++;
  } else {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    int rc = issue(b, n, maxN, warps, groups, tiles, st);
    if (rc) return rc;
    b->stats.eagerLaunches++;
  }
  b->lastShape = b->shape;
  return DDGI_OK;
}

}  // extern "C"
