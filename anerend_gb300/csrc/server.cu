// Serving loop: continuous batching of probe-update requests over resident scenes.
//
// A worker thread owns the device side. Requests are admitted, in arrival order or shortest first with aging
// (DdgiServerConfig.policy), while their grids' memory fits the budget and a launch slot is free; each admitted request gets a grid allocated stream-ordered on
// the slot's stream (no device synchronization), and the admitted set is launched as one batch (persistent
// trace over all of their rays + one convolution launch). Up to `inFlight` batches run at once on separate
// streams, so requests that arrive while others are on the GPU are admitted as slots and memory free up and
// their work overlaps the running batch. A finished batch (its event has fired) releases its grids and memory
// and stamps its requests' completion times, from which the latency percentiles are computed.
#include "objects.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <new>
#include <thread>
#include <unordered_map>

using namespace ddgi::detail;

namespace {

struct Req {
  uint64_t id = 0;
  DdgiRequest r{};
  DdgiGrid* grid = nullptr;
  uint64_t bytes = 0;
  uint64_t rays = 0;  // probes x rays per probe (all layers)
  int state = DDGI_REQUEST_QUEUED;
  int error = DDGI_OK;
  double tSubmit = 0, tAdmit = 0, tDone = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  LaunchState* state = nullptr;
  std::vector<Req*> reqs;
  bool busy = false;
};

}  // namespace

struct DdgiServer {
  DdgiContext* ctx = nullptr;
  DdgiServerConfig cfg{};
  DdgiBatchTuning tuning{};
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  std::deque<Req*> pending;
  std::unordered_map<uint64_t, Req*> all;
  uint64_t nextId = 1;
  uint64_t usedBytes = 0, peakBytes = 0;
  std::vector<Slot> slots;
  std::vector<double> latencies;
  uint64_t submitted = 0, completed = 0, rejected = 0, failed = 0, batches = 0, rays = 0;
  double busySeconds = 0;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

// The next pending request to admit (its index in s->pending), or -1. FIFO: the head. Shortest first: the
// smallest aged ray count, rays x max(0, 1 - wait / agingMs), ties to the older request. Either way the pick
// must fit the memory budget, or nothing is admitted until memory frees up (a request that cannot fit now is
// not overtaken, so it is not starved); with `capLeft` > 0 it must also fit the launch's remaining ray cap,
// else the scan takes the next fitting one (the request waits for the next launch). Called with the lock held.
long pickNext(const DdgiServer* s, uint64_t capLeft, bool capApplies, double now) {
  if (s->pending.empty()) return -1;
  if (s->cfg.policy != DDGI_SERVE_SHORTEST_FIRST) {
    const Req* r = s->pending.front();
    if (s->usedBytes + r->bytes > s->cfg.memoryBudget) return -1;
    if (capApplies && r->rays > capLeft) return -1;
    return 0;
  }
  const double aging = (s->cfg.agingMs > 0.f ? s->cfg.agingMs : 50.0f) * 1e-3;
  long best = -1;
  double bestKey = 0;
  for (size_t i = 0; i < s->pending.size(); ++i) {
    const Req* r = s->pending[i];
    const double key = (double)r->rays * std::max(0.0, 1.0 - (now - r->tSubmit) / aging);
    if (best < 0 || key < bestKey) {  // pending is in arrival order: ties keep the older request
      best = (long)i;
      bestKey = key;
    }
  }
  const Req* r = s->pending[(size_t)best];
  if (s->usedBytes + r->bytes > s->cfg.memoryBudget) return -1;
  if (capApplies && r->rays > capLeft) {
    // the top pick waits for the next launch; fill this one with the best that fits the remaining cap
    long fit = -1;
    double fitKey = 0;
    for (size_t i = 0; i < s->pending.size(); ++i) {
      const Req* q = s->pending[i];
      if (q->rays > capLeft || s->usedBytes + q->bytes > s->cfg.memoryBudget) continue;
      const double key = (double)q->rays * std::max(0.0, 1.0 - (now - q->tSubmit) / aging);
      if (fit < 0 || key < fitKey) {
        fit = (long)i;
        fitKey = key;
      }
    }
    return fit;
  }
  return best;
}

// Completes the batches whose events have fired; called with the lock held.
void reap(DdgiServer* s) {
  for (Slot& sl : s->slots) {
    if (!sl.busy) continue;
    cudaError_t q = cudaEventQuery(sl.done);
    if (q == cudaErrorNotReady) continue;
    double t = s->now();
    for (Req* r : sl.reqs) {
      r->tDone = t;
      if (q == cudaSuccess) {
        r->state = DDGI_REQUEST_DONE;
        s->completed++;
        s->latencies.push_back(t - r->tSubmit);
      } else {
        r->state = DDGI_REQUEST_FAILED;
        r->error = DDGI_EDEVICE;
        s->failed++;
      }
      gridDestroy(r->grid);  // stream-ordered frees: the work that used the grid has finished
      r->grid = nullptr;
      s->usedBytes -= r->bytes;
    }
    sl.reqs.clear();
    sl.busy = false;
  }
}

void workerLoop(DdgiServer* s) {
  cudaSetDevice(s->ctx->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    reap(s);
    bool inFlight = std::any_of(s->slots.begin(), s->slots.end(), [](const Slot& x) { return x.busy; });
    if (s->stop && s->pending.empty() && !inFlight) break;
    Slot* free = nullptr;
    for (Slot& sl : s->slots)
      if (!sl.busy) { free = &sl; break; }
    std::vector<Req*> batch;
    uint64_t batchRays = 0;
    const uint64_t rayCap = (uint64_t)s->cfg.maxBatchMRays * 1000000ull;
    if (free) {
      const double tNow = s->now();
      while (!s->pending.empty() && (int)batch.size() < s->cfg.maxBatch) {
        const bool capApplies = rayCap && !batch.empty();
        const long pick = pickNext(s, capApplies ? rayCap - std::min(rayCap, batchRays) : 0, capApplies, tNow);
        if (pick < 0) break;  // waits for memory, or for the next launch
        Req* r = s->pending[(size_t)pick];
        s->pending.erase(s->pending.begin() + pick);
        int rc = gridCreate(s->ctx, &r->r.grid, free->stream, true, &r->grid);
        if (!rc) rc = tuneGridForBatch(r->grid, s->tuning);
        if (rc) {
          if (r->grid) gridDestroy(r->grid);
          r->grid = nullptr;
          r->state = DDGI_REQUEST_FAILED;
          r->error = rc;
          r->tDone = s->now();
          s->failed++;
          continue;
        }
        s->usedBytes += r->bytes;
        batchRays += r->rays;
        s->peakBytes = std::max(s->peakBytes, s->usedBytes);
        r->state = DDGI_REQUEST_RUNNING;
        r->tAdmit = s->now();
        batch.push_back(r);
      }
    }
    if (!batch.empty()) {
      std::vector<DdgiGrid*> grids;
      std::vector<DdgiScene*> scenes;
      std::vector<DdgiFrame> frames;
      for (Req* r : batch) {
        grids.push_back(r->grid);
        scenes.push_back(const_cast<DdgiScene*>(r->r.scene));
        frames.push_back(r->r.frame);
      }
      DdgiBatchStats st{};
      int rc = batchLaunch(s->ctx, free->state, s->tuning, grids.data(), scenes.data(), frames.data(),
                           (int)batch.size(), free->stream, false, &st);
      for (Req* r : batch)
        if (!rc && r->r.atlasOut)
          if (cudaMemcpyAsync(r->r.atlasOut, r->grid->atlas[r->grid->cur], r->grid->atlasBytes,
                              cudaMemcpyDeviceToHost, free->stream) != cudaSuccess)
            rc = DDGI_EDEVICE;
      if (!rc && cudaEventRecord(free->done, free->stream) != cudaSuccess) rc = DDGI_EDEVICE;
      if (rc) {
        cudaStreamSynchronize(free->stream);
        for (Req* r : batch) {
          r->state = DDGI_REQUEST_FAILED;
          r->error = rc;
          r->tDone = s->now();
          gridDestroy(r->grid);
          r->grid = nullptr;
          s->usedBytes -= r->bytes;
          s->failed++;
        }
      } else {
        free->reqs = batch;
        free->busy = true;
        s->batches++;
        s->rays += st.rays;
      }
      continue;
    }
    // nothing launched: wait for a submission, or poll the running batches
    inFlight = std::any_of(s->slots.begin(), s->slots.end(), [](const Slot& x) { return x.busy; });
    if (inFlight) {
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    } else {
      s->cv.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

void destroyServer(DdgiServer* s) {
  for (Slot& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (Req* r : sl.reqs)
      if (r->grid) gridDestroy(r->grid);
    launchStateDestroy(sl.state);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  for (auto& kv : s->all) {
    if (kv.second->grid) gridDestroy(kv.second->grid);
    delete kv.second;
  }
  delete s;
}

}  // namespace

extern "C" {

int ddgi_server_create(DdgiContext* ctx, const DdgiServerConfig* cfg, DdgiServer** out) {
  if (!ctx || !cfg || !out) return fail(ctx, DDGI_EINVAL, "NULL argument to ddgi_server_create");
  *out = nullptr;
  if (cfg->memoryBudget == 0) return fail(ctx, DDGI_EINVAL, "memoryBudget must be > 0");
  if (cfg->maxBatch < 1 || cfg->maxBatch > 64) return fail(ctx, DDGI_EINVAL, "maxBatch must be in [1, 64]");
  if (cfg->inFlight < 1 || cfg->inFlight > 8) return fail(ctx, DDGI_EINVAL, "inFlight must be in [1, 8]");
  if (cfg->policy != DDGI_SERVE_FIFO && cfg->policy != DDGI_SERVE_SHORTEST_FIRST)
    return fail(ctx, DDGI_EINVAL, "serving policy %d unknown", cfg->policy);
  if (!(cfg->agingMs >= 0.0f)) return fail(ctx, DDGI_EINVAL, "agingMs must be >= 0");
  DdgiBatchTuning t = defaultBatchTuning();
  t.convMode = cfg->convMode;
  t.useGraph = 0;  // a new item set per launch
  int rc = checkBatchTuning(ctx, t);
  if (rc) return rc;
  CK(cudaSetDevice(ctx->device), "set device");
  DdgiServer* s = new (std::nothrow) DdgiServer();
  if (!s) return fail(ctx, DDGI_ENOMEM, "host allocation");
  s->ctx = ctx;
  s->cfg = *cfg;
  s->tuning = t;
  s->slots.resize(cfg->inFlight);
  for (Slot& sl : s->slots) {
    cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    sl.state = launchStateCreate(ctx);
    if (e == cudaSuccess && (!sl.state || launchStateReserve(sl.state, cfg->maxBatch) != DDGI_OK)) e = cudaErrorMemoryAllocation;
    if (e != cudaSuccess) {
      destroyServer(s);
      return cudaFail(ctx, e, "server streams");
    }
  }
  // keep freed request memory in the device's pool up to the budget instead of returning it to the driver
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
    uint64_t keep = cfg->memoryBudget;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  s->worker = std::thread(workerLoop, s);
  *out = s;
  return DDGI_OK;
}

int ddgi_server_submit(DdgiServer* s, const DdgiRequest* req, uint64_t* id) {
  if (!s || !req || !req->scene) return fail(s ? s->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_server_submit");
  DdgiContext* ctx = s->ctx;
  int rc = validateGridDesc(ctx, &req->grid);
  if (rc) return rc;
  if (s->tuning.convMode != 0 && req->grid.raysPerProbe % 64)
    return fail(ctx, DDGI_EINVAL, "tensor-core serving needs raysPerProbe %% 64 == 0");
  if (req->scene->ctx != ctx) return fail(ctx, DDGI_EINVAL, "scene belongs to another context");
  Req* r = new (std::nothrow) Req();
  if (!r) return fail(ctx, DDGI_ENOMEM, "host allocation");
  r->r = *req;
  r->bytes = gridFootprint(&req->grid, s->tuning.convMode, false);  // served grids keep no hit memo
  r->rays = (uint64_t)req->grid.dims[0] * req->grid.dims[1] * req->grid.dims[2] * (uint64_t)req->grid.raysPerProbe;
  std::lock_guard<std::mutex> lk(s->mu);
  r->id = s->nextId++;
  r->tSubmit = s->now();
  s->all[r->id] = r;
  s->submitted++;
  if (id) *id = r->id;
  if (r->bytes > s->cfg.memoryBudget) {
    r->state = DDGI_REQUEST_REJECTED;
    r->error = DDGI_EBUSY;
    r->tDone = r->tSubmit;
    s->rejected++;
    return fail(ctx, DDGI_EBUSY, "request needs %llu bytes, more than the %llu-byte budget",
                (unsigned long long)r->bytes, (unsigned long long)s->cfg.memoryBudget);
  }
  s->pending.push_back(r);
  s->cv.notify_one();
  return DDGI_OK;
}

int ddgi_server_status(DdgiServer* s, uint64_t id, DdgiRequestStatus* out) {
  if (!s || !out) return DDGI_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return fail(s->ctx, DDGI_EINVAL, "unknown request %llu", (unsigned long long)id);
  const Req* r = it->second;
  out->state = r->state;
  out->error = r->error;
  out->submitSeconds = r->tSubmit;
  out->admitSeconds = r->tAdmit;
  out->doneSeconds = r->tDone;
  return DDGI_OK;
}

int ddgi_server_drain(DdgiServer* s, double timeoutSeconds) {
  if (!s) return DDGI_EINVAL;
  auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeoutSeconds);
  while (true) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      bool inFlight = std::any_of(s->slots.begin(), s->slots.end(), [](const Slot& x) { return x.busy; });
      if (s->pending.empty() && !inFlight) return DDGI_OK;
    }
    if (std::chrono::steady_clock::now() > deadline)
      return fail(s->ctx, DDGI_ETIMEDOUT, "server did not drain within %.3f s", timeoutSeconds);
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
}

int ddgi_server_stats(DdgiServer* s, DdgiServerStats* out) {
  if (!s || !out) return DDGI_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = DdgiServerStats{};
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->rejected = s->rejected;
  out->failed = s->failed;
  out->batches = s->batches;
  out->rays = s->rays;
  out->peakBytes = s->peakBytes;
  out->elapsedSeconds = s->now();
  std::vector<double> v = s->latencies;
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5))]; };
    double sum = 0;
    for (double x : v) sum += x;
    out->p50LatencyMs = 1e3 * pct(0.50);
    out->p99LatencyMs = 1e3 * pct(0.99);
    out->maxLatencyMs = 1e3 * v.back();
    out->meanLatencyMs = 1e3 * sum / v.size();
  }
  return DDGI_OK;
}

void ddgi_server_destroy(DdgiServer* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (Req* r : s->pending) {
      r->state = DDGI_REQUEST_FAILED;
      r->error = DDGI_EBUSY;
    }
    s->pending.clear();
    s->cv.notify_one();
  }
  if (s->worker.joinable()) s->worker.join();
  destroyServer(s);
}

}  // extern "C"
