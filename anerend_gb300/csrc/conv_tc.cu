// Probe convolution on the tcgen05 tensor cores (probe_conv.comp:21-90 as a GEMM).
//
// All probes of a dispatch share the N ray directions, so the convolution of channel c is the product
//   D_c[probe][texel] = sum_j R_c[probe][j] * W[texel][j],   W[t][j] = max(0, d_j . omega_t) (0 if <= 1e-6)
// with R_c the 16-bit (FP16 or BF16) radiance of channel c, stored planar: row c * P + p, N rays per row.
// The probes of every item are cut into units of 64; each CTA (one per SM) takes an equal contiguous run of
// the launch's units and walks it in tiles of two units (128 probes), or one at the end of its run or of an
// item, so no SM carries more than one unit above the average. Per tile and 64-ray K-chunk a TMA producer
// warp loads the three radiance tiles (64-row boxes, one or two per channel) and the 64 x 64 weight tile
// (SWIZZLE_128B); one thread of the MMA warp issues 4 K-steps x 3 channels of tcgen05.mma (M = 128 probe
// rows, N = 64 texels, K = 16) into FP32 accumulators in TMEM (3 x 64 columns, double-buffered = 384 of 512
// columns); the rows of a one-unit tile past its 64 probes hold stale operands and are never read. Sixteen
// epilogue warps (four per TMEM lane quarter, one texel block of 16 texels each) read the accumulators with
// tcgen05.ld (thread = probe), stage them in shared memory and walk the atlas coalesced (lanes = 4 probes x 8
// texels of a row), normalising by the texel's weight sum and applying the hysteresis blend (or the bake
// accumulation) in FP32 against the old atlas texel. The epilogue is bound by the latency of its atlas
// read-modify-write, so its warps come before operand stages in the shared-memory budget: two stages.
// A single-item launch carries its record and tensor maps in the kernel parameters (TcOne); a batch reads
// its records from device memory (TcMany), so a captured launch sees per-frame values written between replays.
//
// Every mbarrier wait is bounded (WaitCfg::spin attempts): on timeout the kernel raises DDGI_DEVERR_TIMEOUT, stops
// issuing work, waits (bounded by kDrainLimit, whatever WaitCfg says) for its own TMA loads and MMAs in flight,
// frees its TMEM and returns.
#include "ddgi_common.cuh"
#include "kernels.h"

#include <cuda_bf16.h>
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

namespace ddgi {

namespace {

constexpr int kTileP = 128;                  // probe rows per tile (MMA M)
constexpr int kUnitP = 64;                   // probes per work unit (one TMA box of radiance rows)
constexpr int kChunkK = 64;                  // rays per K-chunk (128 bytes of 16-bit values)
constexpr int kStages = 2;  // 2 x 56 KB of operand staging (the epilogue's 16 staging areas take the rest)
constexpr int kATileBytes = kTileP * kChunkK * 2;   // 16 KB per channel
constexpr int kAUnitBytes = kUnitP * kChunkK * 2;   // 8 KB: one unit's rows of one channel
constexpr int kWTileBytes = kOctTexels * kChunkK * 2;  // 8 KB
constexpr int kStageBytes = 3 * kATileBytes + kWTileBytes;  // 56 KB
constexpr int kTmemCols = 512;
constexpr int kEpiWarps = 16;                // four per TMEM lane quarter, one texel block each
constexpr int kBlocksPerWarp = 16 / kEpiWarps;  // 16 (quarter, texel block) pairs per tile
constexpr int kThreadsTc = 64 + 32 * kEpiWarps;  // warp 0 TMA, warp 1 MMA, warps 2-17 epilogue
// epilogue staging: per epilogue warp, 3 channels x 32 probes x 16 texels of one texel block (row stride 17)
constexpr int kStageRow = 17;
constexpr int kStageWarpFloats = 3 * 32 * kStageRow;
constexpr size_t kSmemTc = (size_t)kStages * kStageBytes + kEpiWarps * kStageWarpFloats * sizeof(float) + 1024;
static_assert(kSmemTc <= 227 * 1024, "operand stages and epilogue staging exceed a CTA's shared memory");
static_assert(kEpiWarps % 4 == 0 && 16 % kEpiWarps == 0, "epilogue warps cover the 4 lane quarters evenly");
// attempts of a wait for the kernel's own copies and MMAs in flight before the CTA exits (after a timeout)
constexpr uint32_t kDrainLimit = 1u << 22;

DDGI_D uint32_t smemU32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

DDGI_D void mbarInit(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemU32(bar)), "r"(count) : "memory");
}
DDGI_D void mbarExpectTx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemU32(bar)), "r"(bytes) : "memory");
}
DDGI_D void mbarArrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemU32(bar)) : "memory");
}
DDGI_D bool mbarTryWait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smemU32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; false after `limit` attempts (about 64 ns apart after the first 32).
DDGI_D bool mbarWait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbarTryWait(bar, parity)) return true;
    if (i > 32) __nanosleep(64);
  }
  return false;
}

// Programmatic dependent launch: the convolution is launched while the weights kernel before it still runs
// (its prologue and its first radiance loads overlap that kernel); it waits for the weights kernel's results
// here before reading them. Without the launch attribute the wait returns at once.
DDGI_D void gridDependencyWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
DDGI_D void gridDependentsMayLaunch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

DDGI_D void tmaLoad2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smemU32(dst)),
      "l"((uint64_t)map), "r"(smemU32(bar)), "r"(x), "r"(y)
      : "memory");
}

DDGI_D void tmemAlloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemU32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
DDGI_D void tmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
DDGI_D void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
DDGI_D void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

DDGI_D void mmaF16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dTmem),
      "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
DDGI_D void mmaCommit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemU32(bar))
               : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: thread t gets lane (base lane + t), columns col .. col + 15.
DDGI_D void tmemLoad16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of a K-major, SWIZZLE_128B operand tile whose rows are 128 bytes and
// whose 8-row swizzle atoms are 1024 bytes apart (start address 1024-byte aligned, advanced by 32 bytes per
// K step of 16 elements inside the atom).
DDGI_D uint64_t smemDesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);        // start address
  d |= (uint64_t)(16 >> 4) << 16;                // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                        // descriptor version
  d |= (uint64_t)2 << 61;                        // SWIZZLE_128B
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulate, A and B both FP16 (fmt 0) or BF16 (fmt 1),
// both K-major, M = 128, N = 64.
__host__ __device__ constexpr uint32_t instrDesc(uint32_t fmt) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
}

constexpr int kMaxTcItems = 64;

// Per-grid record of a (batched) tensor-core convolution. A batch keeps the records in device memory so that
// per-frame values (atlas after a translation, layer range, flags) can change between replays of a captured
// launch; a single-item launch passes its record by value.
struct TcItem {
  int X, atlasW, atlasFmt;
  int pBegin, pEnd;       // probe range (linear over the grid, layer-major)
  int pTotal;             // rows per channel of the radiance matrix
  int numChunks;          // N / 64
  int unitBegin;          // first 64-probe unit of this item in the launch
  float hysteresis;
  uint32_t flags;
  void* atlas;
  const float4* dirs;     // lattice of the frame
  uint16_t* w16;          // 64 x N weights (written by k_tc_weights)
  float* wsum16;          // sums of the rounded weights (normalisation)
  float* wsum32;          // sums of the FP32 weights (the .w channel)
  int n;
};

DDGI_HD int tcUnits(const TcItem& it) { return (it.pEnd - it.pBegin + kUnitP - 1) / kUnitP; }

// Tensor maps of every item (radiance R with 64-row boxes, weights W); static for a batch.
struct TcMaps {
  CUtensorMap r[kMaxTcItems];
  CUtensorMap w[kMaxTcItems];
};

// Item records are kTcItemStride bytes apart in device memory (the host stages them in 128-byte slots).
constexpr int kTcItemStride = 128;
static_assert(sizeof(TcItem) <= kTcItemStride, "TcItem must fit its 128-byte record slot");

DDGI_HD const TcItem& tcItem(const unsigned char* recs, int i) {
  return *reinterpret_cast<const TcItem*>(recs + (size_t)i * kTcItemStride);
}

// Where the kernels' records and tensor maps come from (passed by value, __grid_constant__).
struct TcOne {
  CUtensorMap r, w;
  TcItem it;
  DDGI_D int numItems() const { return 1; }
  DDGI_D int itemOfUnit(int) const { return 0; }
  DDGI_D const TcItem& item(int) const { return it; }
  DDGI_D const CUtensorMap* mapR(int) const { return &r; }
  DDGI_D const CUtensorMap* mapW(int) const { return &w; }
};
struct TcMany {
  TcMaps maps;
  const unsigned char* items;
  int n;
  DDGI_D int numItems() const { return n; }
  DDGI_D int itemOfUnit(int unit) const {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (tcItem(items, mid).unitBegin <= unit) lo = mid; else hi = mid - 1;
    }
    return lo;
  }
  DDGI_D const TcItem& item(int i) const { return tcItem(items, i); }
  DDGI_D const CUtensorMap* mapR(int i) const { return &maps.r[i]; }
  DDGI_D const CUtensorMap* mapW(int i) const { return &maps.w[i]; }
};

// A CTA's run of units, walked in tiles of at most two units that do not cross an item boundary. Every warp
// role walks the same sequence.
struct TcTile {
  int item, p0, units;
};
template <class Src>
DDGI_D bool nextTile(const Src& src, int& unit, int unitEnd, TcTile& t) {
  if (unit >= unitEnd) return false;
  const int ii = src.itemOfUnit(unit);
  const TcItem& it = src.item(ii);
  const int local = unit - it.unitBegin;
  int n = tcUnits(it) - local;
  if (n > 2) n = 2;
  if (n > unitEnd - unit) n = unitEnd - unit;
  t.item = ii;
  t.p0 = it.pBegin + local * kUnitP;
  t.units = n;
  unit += n;
  return true;
}

template <int kFmt, class Src>
__global__ void __launch_bounds__(kThreadsTc, 1)
    k_conv_tc(const __grid_constant__ Src src, int totalUnits, uint32_t* __restrict__ err, WaitCfg waits) {
  extern __shared__ uint8_t smemRaw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smemRaw + 1023) & ~(uintptr_t)1023);
  // neverBar: no thread ever arrives on it; with waits.stall the epilogue's first wait is on it, so the
  // timeout path runs (the failure-detection test)
  __shared__ uint64_t fullBar[kStages], emptyBar[kStages], accFull[2], accEmpty[2], drainBar, neverBar;
  __shared__ uint32_t tmemSlot;
  __shared__ int abortFlag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's units: an equal share of the launch's, contiguous
  const int unitBegin = (int)((long long)blockIdx.x * totalUnits / gridDim.x);
  const int unitEnd = (int)((long long)(blockIdx.x + 1) * totalUnits / gridDim.x);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) { mbarInit(&fullBar[s], 1); mbarInit(&emptyBar[s], 1); }
    for (int b = 0; b < 2; ++b) { mbarInit(&accFull[b], 1); mbarInit(&accEmpty[b], 32 * kEpiWarps); }
    mbarInit(&drainBar, 1);
    mbarInit(&neverBar, 1);
    abortFlag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmemAlloc(&tmemSlot, kTmemCols);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = tmemSlot;

  auto fail = [&]() {
    atomicOr(err, DDGI_DEVERR_TIMEOUT);
    atomicExch(&abortFlag, 1);
  };
  auto aborted = [&]() { return *(volatile int*)&abortFlag != 0; };

  TcTile tile;
  int unit = unitBegin;
  if (warp == 0) {
    // ---- TMA producer ----
    if (lane == 0) {
      bool pending[kStages] = {};
      uint32_t pendingParity[kStages] = {};
      bool weightsReady = false;
      int s = 0;
      uint32_t phase = 0;
      while (!aborted() && nextTile(src, unit, unitEnd, tile)) {
        const TcItem& it = src.item(tile.item);
        const CUtensorMap* mr = src.mapR(tile.item);
        const CUtensorMap* mw = src.mapW(tile.item);
        const uint32_t bytes = (uint32_t)(3 * tile.units * kAUnitBytes + kWTileBytes);
        bool ok = true;
        for (int kc = 0; kc < it.numChunks; ++kc) {
          if (!mbarWait(&emptyBar[s], phase ^ 1, waits.spin)) { fail(); ok = false; break; }
          pending[s] = false;
          uint8_t* st = smem + (size_t)s * kStageBytes;
          mbarExpectTx(&fullBar[s], bytes);
          for (int c = 0; c < 3; ++c)
            for (int u = 0; u < tile.units; ++u)
              tmaLoad2d(st + c * kATileBytes + u * kAUnitBytes, mr, &fullBar[s], kc * kChunkK,
                        c * it.pTotal + tile.p0 + u * kUnitP);
          if (!weightsReady) {  // the weights come from the kernel launched just before this one
            gridDependencyWait();
            weightsReady = true;
          }
          tmaLoad2d(st + 3 * kATileBytes, mw, &fullBar[s], kc * kChunkK, 0);
          pending[s] = true;
          pendingParity[s] = phase;
          if (++s == kStages) { s = 0; phase ^= 1; }
        }
        if (!ok) break;
      }
      if (aborted()) {  // let loads in flight land before the CTA exits
        for (int k = 0; k < kStages; ++k)
          if (pending[k]) mbarWait(&fullBar[k], pendingParity[k], kDrainLimit);
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      const uint32_t idesc = instrDesc(kFmt);
      int s = 0;
      uint32_t phase = 0;
      int local = 0;
      bool issued = false;
      for (; !aborted() && nextTile(src, unit, unitEnd, tile); ++local) {
        const int numChunks = src.item(tile.item).numChunks;
        int b = local & 1;
        uint32_t accPhase = (local >> 1) & 1;
        if (!mbarWait(&accEmpty[b], accPhase ^ 1, waits.spin)) { fail(); break; }
        tcFenceAfter();
        const uint32_t dBase = tmem + (uint32_t)(b * 3 * kOctTexels);
        bool ok = true;
        for (int kc = 0; kc < numChunks; ++kc) {
          if (!mbarWait(&fullBar[s], phase, waits.spin)) { fail(); ok = false; break; }
          tcFenceAfter();
          uint32_t st = smemU32(smem + (size_t)s * kStageBytes);
#pragma unroll
          for (int kk = 0; kk < kChunkK / 16; ++kk) {
            uint64_t bDesc = smemDesc(st + 3 * kATileBytes + kk * 32);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              uint64_t aDesc = smemDesc(st + c * kATileBytes + kk * 32);
              mmaF16(dBase + c * kOctTexels, aDesc, bDesc, idesc, (kc > 0 || kk > 0) ? 1u : 0u);
            }
          }
          issued = true;
          mmaCommit(&emptyBar[s]);  // stage free once these MMAs have read it
          if (++s == kStages) { s = 0; phase ^= 1; }
        }
        if (!ok) break;
        mmaCommit(&accFull[b]);
      }
      if (issued) {  // drain: every MMA issued by this thread has completed
        mmaCommit(&drainBar);
        mbarWait(&drainBar, 0, kDrainLimit);
      }
    }
  } else {
    // ---- epilogue: warps 2 .. 1 + kEpiWarps ----
    // A warp may read TMEM lanes 32q..32q+31 with q = warp % 4 (its probe rows); the warps of a quarter
    // split the four blocks of 16 texels between them (kBlocksPerWarp each). Per block (two texel rows)
    // it reads its rows' accumulators (thread = probe), stages them in shared memory and then walks the
    // atlas coalesced: per step its lanes cover 4 probes x the 8 texels of one row (4 runs of 128 bytes).
    // The old texels do not depend on the MMA, so their loads are issued before the accumulator wait. A warp
    // whose rows lie past the tile's probes still waits for the accumulators before it releases them, so its
    // arrivals on accEmpty stay in the phase of their tile.
    gridDependencyWait();  // the weight sums come from the kernel launched just before this one
    const int quarter = warp & 3;  // TMEM lane quarter this warp may access
    const int blk0 = ((warp - 2) >> 2) * kBlocksPerWarp;  // its texel blocks: blk0 .. blk0 + kBlocksPerWarp - 1
    float* stage = reinterpret_cast<float*>(smem + (size_t)kStages * kStageBytes) + (warp - 2) * kStageWarpFloats;
    const int tx = lane & 7, pp = lane >> 3;
    int local = 0;
    for (; !aborted() && nextTile(src, unit, unitEnd, tile); ++local) {
      const TcItem& it = src.item(tile.item);
      const bool bake = (it.flags & DDGI_UBO_BAKE_MODE_ON_FLAG) != 0;
      const float h = it.hysteresis, a = 1.0f - h;
      const int b = local & 1;
      const uint32_t accPhase = (local >> 1) & 1;
      const int tileEnd = min(it.pEnd, tile.p0 + tile.units * kUnitP);
      // atlas offsets of the 8 probes this lane visits (probe 4g + pp of the warp's 32), texel (tx, 0)
      const int warpProbe0 = tile.p0 + quarter * 32;
      // texel indices fit 32 bits: an atlas holds at most 2^31 texels (checked when its grid is described)
      uint32_t base[8];
      uint32_t liveMask = 0;
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        const int probe = warpProbe0 + 4 * g + pp;
        const bool live = probe < tileEnd;
        const int px = live ? probe % it.X : 0, pzAll = live ? probe / it.X : 0;  // pzAll = layer * Z + z
        base[g] = (uint32_t)(kProbePix * pzAll + 1) * (uint32_t)it.atlasW + (uint32_t)(kProbePix * px + 1 + tx);
        liveMask |= (live ? 1u : 0u) << g;
      }
      const bool rowsLive = warpProbe0 < tileEnd;  // warp-uniform
      const uint32_t laneAddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * 3 * kOctTexels);
      bool ok = true;
      if (waits.stall && local == 0) {  // the test hook: a wait that no arrival ends
        if (!__all_sync(0xffffffffu, mbarWait(&neverBar, 0, waits.spin))) {
          if (lane == 0) fail();
          break;
        }
      }
      if (!rowsLive) {
        // warp-uniform outcome
        if (!__all_sync(0xffffffffu, mbarWait(&accFull[b], accPhase, waits.spin))) {
          if (lane == 0) fail();
          break;
        }
        tcFenceAfter();
      }
#pragma unroll 1
      for (int blk = blk0; rowsLive && blk < blk0 + kBlocksPerWarp; ++blk) {
        // step g of row r: probe 4g + pp, texel row ty = 2 blk + r. The first row's old texels are loaded
        // before the accumulator wait, the second row's once the first row is written (register budget).
        float4 olds[8];
#pragma unroll
        for (int g = 0; g < 8; ++g)
          olds[g] = (liveMask >> g) & 1u ? loadTexel(it.atlas, it.atlasFmt, base[g] + (uint32_t)(2 * blk) * it.atlasW)
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
        if (blk == blk0) {
          // warp-uniform outcome: the tcgen05.ld below is warp-collective
          if (!__all_sync(0xffffffffu, mbarWait(&accFull[b], accPhase, waits.spin))) {
            if (lane == 0) fail();
            ok = false;
            break;
          }
          tcFenceAfter();
        }
        // one channel at a time, so only 16 accumulator values are live next to the old texels
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float cv[16];
          tmemLoad16(laneAddr + c * kOctTexels + blk * 16, cv);
#pragma unroll
          for (int i = 0; i < 16; ++i)  // thread = probe row `lane`: conflict-free (stride 17)
            stage[c * 32 * kStageRow + lane * kStageRow + i] = cv[i];
        }
        __syncwarp();
        const int tex0 = 2 * blk * kOct + tx;  // texel (tx, 2 blk); + 8 for the second row
        const float s16a = __ldg(&it.wsum16[tex0]), s32a = __ldg(&it.wsum32[tex0]);
        const float s16b = __ldg(&it.wsum16[tex0 + kOct]), s32b = __ldg(&it.wsum32[tex0 + kOct]);
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const int g = k & 7, row2 = k >> 3, ty = 2 * blk + row2;
          if (k == 8) {  // the second row's old texels
#pragma unroll
            for (int q = 0; q < 8; ++q)
              olds[q] = (liveMask >> q) & 1u ? loadTexel(it.atlas, it.atlasFmt, base[q] + (uint32_t)ty * it.atlasW)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
          }
          if (!((liveMask >> g) & 1u)) continue;
          const int sp = (4 * g + pp) * kStageRow + row2 * kOct + tx;
          const float rr0 = stage[sp], gg0 = stage[32 * kStageRow + sp], bb0 = stage[2 * 32 * kStageRow + sp];
          const float s16 = row2 ? s16b : s16a, s32 = row2 ? s32b : s32a;
          const float4 old = olds[g];
          float4 out;
          if (bake) {
            float tw = old.w + s32;
            float rr = rr0 + old.x * old.w, gg = gg0 + old.y * old.w, bb = bb0 + old.z * old.w;
            if (tw > 1e-6f) { rr /= tw; gg /= tw; bb /= tw; }
            out = make_float4(rr, gg, bb, tw);
          } else {
            float rr = rr0, gg = gg0, bb = bb0;
            if (s16 > 1e-6f) { float inv = 1.0f / s16; rr *= inv; gg *= inv; bb *= inv; }
            out = make_float4(rr * a + old.x * h, gg * a + old.y * h, bb * a + old.z * h, s32 * a + old.w * h);
          }
          storeTexel(it.atlas, it.atlasFmt, base[g] + (uint32_t)ty * it.atlasW, out);
        }
        __syncwarp();  // the stage is rewritten by the next block
      }
      if (!ok) break;
      tcFenceBefore();
      mbarArrive(&accEmpty[b]);
    }
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 1) tmemDealloc(tmem, kTmemCols);
}

// W[t][j] in 16-bit (rows = texels, K-major), the sums of the rounded weights and of the FP32 weights;
// one block per (texel, item), threads over the rays. Records from `items` in device memory, or `one` when
// items is null.
template <int kFmt>
__global__ void __launch_bounds__(256) k_tc_weights(const unsigned char* __restrict__ items,
                                                    const __grid_constant__ TcItem one) {
  __shared__ float r16[256], r32[256];
  gridDependentsMayLaunch();
  const TcItem& it = items ? tcItem(items, blockIdx.y) : one;
  const int n = it.n;
  int t = blockIdx.x;
  float3 omega = texelDirection(t % kOct, t / kOct);
  float a16 = 0.f, a32 = 0.f;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    float w = fmaxf(0.0f, dot3(xyz(it.dirs[j]), omega));
    if (!(w > 1e-6f)) w = 0.0f;
    float r;
    uint16_t bits;
    if (kFmt == 0) {
      __half hv = __float2half_rn(w);
      bits = __half_as_ushort(hv);
      r = __half2float(hv);
    } else {
      __nv_bfloat16 bv = __float2bfloat16_rn(w);
      bits = __bfloat16_as_ushort(bv);
      r = __bfloat162float(bv);
    }
    it.w16[(size_t)t * n + j] = bits;
    a16 += r;
    a32 += w;
  }
  r16[threadIdx.x] = a16;
  r32[threadIdx.x] = a32;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      r16[threadIdx.x] += r16[threadIdx.x + o];
      r32[threadIdx.x] += r32[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    it.wsum16[t] = r16[0];
    it.wsum32[t] = r32[0];
  }
}

// Ray image (g.rayFmt texels) -> planar 16-bit radiance, row c * pTotal + p (p linear over the grid), N rays
// per row.
template <int kFmt>
__global__ void k_pack_rays16(GridGPU g, const void* __restrict__ rayRad, uint16_t* __restrict__ out, int pBegin,
                              int pEnd, int pTotal) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)(pEnd - pBegin) * g.N;
  if (i >= total) return;
  int p = pBegin + (int)(i / g.N), j = (int)(i % g.N);
  int px = p % g.X, pzAll = p / g.X;
  int rx = px * g.bw + (j % g.bw);
  int ry = pzAll * g.bh + (j / g.bw);
  const float4 v = loadTexel(rayRad, g.rayFmt, (size_t)ry * g.rayW + rx);
  float c[3] = {v.x, v.y, v.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    uint16_t bits = kFmt == 0 ? __half_as_ushort(__float2half_rn(c[k])) : __bfloat16_as_ushort(__float2bfloat16_rn(c[k]));
    out[((size_t)k * pTotal + p) * g.N + j] = bits;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encodeFn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  });
  return fn;
}

// rows x cols matrix of 16-bit values (row-major), boxes of boxRows x 64 with SWIZZLE_128B
bool makeMap(CUtensorMap* m, int fmt, const void* base, uint64_t rows, uint64_t cols, uint32_t boxRows) {
  auto fn = encodeFn();
  if (!fn) return false;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)kChunkK, boxRows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, fmt == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                  const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

cudaError_t launchPackRays16(const GridGPU& g, int elemFmt, const void* rayRad, void* out16, int layerBegin,
                             int layerEnd, int pTotal, cudaStream_t stream) {
  int pBegin = layerBegin * g.X * g.Z, pEnd = layerEnd * g.X * g.Z;
  long long total = (long long)(pEnd - pBegin) * g.N;
  if (total <= 0) return cudaSuccess;
  unsigned blocks = (unsigned)((total + 255) / 256);
  if (elemFmt == 0) k_pack_rays16<0><<<blocks, 256, 0, stream>>>(g, rayRad, (uint16_t*)out16, pBegin, pEnd, pTotal);
  else k_pack_rays16<1><<<blocks, 256, 0, stream>>>(g, rayRad, (uint16_t*)out16, pBegin, pEnd, pTotal);
  return cudaGetLastError();
}

size_t tcScratchBytes(int n) { return (size_t)kOctTexels * n * 2 + 2 * kOctTexels * sizeof(float) + 256; }

int tcMaxItems() { return kMaxTcItems; }

// Fills the item record and its two tensor maps for one grid; scratch = tcScratchBytes(N) bytes.
bool tcPrepareItem(const GridGPU& g, int elemFmt, const void* rad16, int pTotal, const float4* dirs, void* scratch,
                   void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags, int unitBegin,
                   TcItemHost* out) {
  if (g.N % kChunkK) return false;
  TcItem& it = *reinterpret_cast<TcItem*>(out->item);
  static_assert(sizeof(TcItem) <= sizeof(out->item), "TcItemHost too small");
  it.X = g.X;
  it.atlasW = g.atlasW;
  it.atlasFmt = g.atlasFmt;
  it.pBegin = layerBegin * g.X * g.Z;
  it.pEnd = layerEnd * g.X * g.Z;
  it.pTotal = pTotal;
  it.numChunks = g.N / kChunkK;
  it.unitBegin = unitBegin;
  it.hysteresis = hysteresis;
  it.flags = flags;
  it.atlas = atlas;
  it.dirs = dirs;
  it.w16 = (uint16_t*)scratch;
  it.wsum16 = (float*)((uint8_t*)scratch + (size_t)kOctTexels * g.N * 2);
  it.wsum32 = it.wsum16 + kOctTexels;
  it.n = g.N;
  out->units = tcUnits(it);
  if (!makeMap(reinterpret_cast<CUtensorMap*>(out->mapR), elemFmt, rad16, (uint64_t)3 * pTotal, (uint64_t)g.N, kUnitP))
    return false;
  if (!makeMap(reinterpret_cast<CUtensorMap*>(out->mapW), elemFmt, it.w16, kOctTexels, (uint64_t)g.N, kOctTexels))
    return false;
  return true;
}

namespace {

// Per-process, per-device launch set-up of a k_conv_tc instance (the shared-memory attribute is a property
// of the function on each device); returns the device's SM count in *sms.
template <class Kern>
cudaError_t tcLaunchSetup(Kern kern, int slot, int* sms) {
  static std::mutex mu;
  static int smCount[64] = {};
  static bool attrSet[64][4] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (!attrSet[dev][slot]) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTc);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&smCount[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    attrSet[dev][slot] = true;
  }
  *sms = smCount[dev];
  return cudaSuccess;
}

template <int kFmt, class Src>
cudaError_t launchTc(const Src& src, int slot, int totalUnits, uint32_t* err, WaitCfg waits, cudaStream_t stream) {
  int sms = 0;
  cudaError_t e = tcLaunchSetup(k_conv_tc<kFmt, Src>, slot, &sms);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(totalUnits < sms ? totalUnits : sms);
  cfg.blockDim = dim3(kThreadsTc);
  cfg.dynamicSmemBytes = kSmemTc;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (waits.spin == 0) waits.spin = WaitCfg{}.spin;
  return cudaLaunchKernelEx(&cfg, k_conv_tc<kFmt, Src>, src, totalUnits, err, waits);
}

}  // namespace

// Weights of every item, then the tensor-core convolution of all items' units in one launch.
// dItems: numItems TcItem records in device memory (copied from the TcItemHost.item bytes).
cudaError_t launchConvTcItems(int elemFmt, const TcItemHost* hostItems, const void* dItems, int numItems,
                              int totalUnits, uint32_t* err, cudaStream_t stream, WaitCfg waits) {
  if (numItems <= 0 || totalUnits <= 0) return cudaSuccess;
  if (numItems > kMaxTcItems) return cudaErrorInvalidValue;
  const unsigned char* items = (const unsigned char*)dItems;
  TcItem none;
  memset(&none, 0, sizeof none);
  dim3 wg(kOctTexels, numItems);
  if (elemFmt == 0) k_tc_weights<0><<<wg, 256, 0, stream>>>(items, none);
  else k_tc_weights<1><<<wg, 256, 0, stream>>>(items, none);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  static TcMany src;  // host staging of the kernel parameter (copied at launch)
  static std::mutex srcMu;
  std::lock_guard<std::mutex> lk(srcMu);
  for (int i = 0; i < numItems; ++i) {
    memcpy(&src.maps.r[i], hostItems[i].mapR, sizeof(CUtensorMap));
    memcpy(&src.maps.w[i], hostItems[i].mapW, sizeof(CUtensorMap));
  }
  src.items = items;
  src.n = numItems;
  return elemFmt == 0 ? launchTc<0>(src, 0, totalUnits, err, waits, stream)
                      : launchTc<1>(src, 1, totalUnits, err, waits, stream);
}

// One grid: the record and the tensor maps travel in the kernel parameters (no copy to the device).
cudaError_t launchConvTc(const GridGPU& g, int elemFmt, const void* rad16, int pTotal, const float4* dirs,
                         void* scratch, void* atlas, int layerBegin, int layerEnd, float hysteresis, uint32_t flags,
                         uint32_t* err, cudaStream_t stream, WaitCfg waits) {
  if (layerEnd <= layerBegin) return cudaSuccess;
  TcItemHost h;
  if (!tcPrepareItem(g, elemFmt, rad16, pTotal, dirs, scratch, atlas, layerBegin, layerEnd, hysteresis, flags, 0, &h))
    return cudaErrorInvalidValue;
  TcOne one;
  memcpy(&one.r, h.mapR, sizeof(CUtensorMap));
  memcpy(&one.w, h.mapW, sizeof(CUtensorMap));
  memcpy(&one.it, h.item, sizeof(TcItem));
  dim3 wg(kOctTexels, 1);
  if (elemFmt == 0) k_tc_weights<0><<<wg, 256, 0, stream>>>(nullptr, one.it);
  else k_tc_weights<1><<<wg, 256, 0, stream>>>(nullptr, one.it);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return elemFmt == 0 ? launchTc<0>(one, 2, h.units, err, waits, stream)
                      : launchTc<1>(one, 3, h.units, err, waits, stream);
}

}  // namespace ddgi
