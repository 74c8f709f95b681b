// C ABI of the DDGI probe engine (include/ddgi.h): objects, argument checks and the per-frame pass
// sequence. The exe lambdas of the three reference passes (IrradianceProbeTranslationPass.cpp:56-186,
// IrradianceProbeRayTracingPass.cpp:95-165, IrradianceProbeConvolvePass.cpp:109-143) become
// ddgi_translate / ddgi_trace / ddgi_convolve; their state (_lastProbeIdx, _currentLayer and the
// "ProbeLayer" blackboard value) lives in the grid object.
#include "objects.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

namespace ddgi {
namespace detail {

namespace {
cudaError_t gridAlloc(DdgiGrid* g, void** p, size_t bytes) {
  if (allocRefused(g->ctx, bytes)) return cudaErrorMemoryAllocation;
  if (g->asyncAlloc) return cudaMallocAsync(p, bytes, g->allocStream);
  return cudaMalloc(p, bytes);
}
void gridFree(DdgiGrid* g, void* p) {
  if (!p) return;
  if (g->asyncAlloc) cudaFreeAsync(p, g->allocStream);
  else cudaFree(p);
}
}  // namespace

int fail(DdgiContext* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->err = buf;
  }
  return code;
}

int cudaFail(DdgiContext* ctx, cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation)
    return fail(ctx, DDGI_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
  return fail(ctx, DDGI_EDEVICE, "%s: %s", what, cudaGetErrorString(e));
}


bool isPow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

int validateGridDesc(DdgiContext* ctx, const DdgiGridDesc* d) {
  if (!d) return fail(ctx, DDGI_EINVAL, "grid desc is NULL");
  for (int i = 0; i < 3; ++i)
    if (d->dims[i] <= 0 || d->dims[i] > 4096) return fail(ctx, DDGI_EINVAL, "grid dims[%d]=%d out of range", i, d->dims[i]);
  for (int i = 0; i < 3; ++i)
    if (!(d->step[i] > 0.0f) || !std::isfinite(d->step[i])) return fail(ctx, DDGI_EINVAL, "grid step[%d] must be > 0", i);
  if (!isPow2(d->raysPerProbe) || d->raysPerProbe < 16 || d->raysPerProbe > 1024)
    return fail(ctx, DDGI_EINVAL, "raysPerProbe=%d must be a power of two in [16, 1024]", d->raysPerProbe);
  if (d->atlasFormat != DDGI_FORMAT_RGBA32F && d->atlasFormat != DDGI_FORMAT_RGBA16F)
    return fail(ctx, DDGI_EINVAL, "atlasFormat=%d unknown", d->atlasFormat);
  if (!(d->hysteresis >= 0.0f && d->hysteresis <= 1.0f)) return fail(ctx, DDGI_EINVAL, "hysteresis must be in [0,1]");
  if (d->options & ~(DDGI_GRID_EDGE_CLAMP | DDGI_GRID_WRITE_DIRS | DDGI_GRID_RECORD_HITS | DDGI_GRID_RAYS_RGBA16F))
    return fail(ctx, DDGI_EINVAL, "unknown grid option bits 0x%x", d->options);
  long long aw = (long long)kProbePix * d->dims[0], ah = (long long)kProbePix * d->dims[2] * d->dims[1];
  if (aw * ah > (1ll << 31)) return fail(ctx, DDGI_EINVAL, "atlas too large");
  return DDGI_OK;
}

GridGPU makeGridGPU(const DdgiGridDesc& d) {
  GridGPU g{};
  g.X = d.dims[0];
  g.Y = d.dims[1];
  g.Z = d.dims[2];
  g.N = d.raysPerProbe;
  rayBlock(g.N, g.bw, g.bh);
  g.step = f3(d.step[0], d.step[1], d.step[2]);
  g.originY = d.originY;
  g.atlasW = kProbePix * g.X;
  g.atlasH = kProbePix * g.Z * g.Y;
  g.atlasFmt = d.atlasFormat;
  g.rayW = g.bw * g.X;
  g.rayFmt = (d.options & DDGI_GRID_RAYS_RGBA16F) ? DDGI_FORMAT_RGBA16F : DDGI_FORMAT_RGBA32F;
  g.options = d.options;
  g.magicX = divMagic((uint32_t)g.X);
  setGridWarpProbes(g, 1);
  return g;
}

// Order of the N lattice directions along a Morton curve of their octahedral coordinates, so that
// consecutive slots are neighbours on the sphere (rotations preserve neighbourhoods, so the order is
// computed once from the unrotated lattice of worldDirFromFibonacciIndex, rgen:35-46).
std::vector<int> mortonRayOrder(int n) {
  std::vector<std::pair<uint64_t, int>> keys(n);
  for (int i = 0; i < n; ++i) {
    double theta = 2.0 * kPiRgen * (double)i / kGoldenRatio;
    double phi = std::acos(1.0 - 2.0 * ((double)i + 0.5) / (double)n);
    double x = std::cos(theta) * std::sin(phi), y = std::sin(theta) * std::sin(phi), z = std::cos(phi);
    double l1 = std::fabs(x) + std::fabs(y) + std::fabs(z);
    double u = x / l1, v = y / l1;
    if (z < 0) {
      double nu = (1 - std::fabs(v)) * (u >= 0 ? 1 : -1), nv = (1 - std::fabs(u)) * (v >= 0 ? 1 : -1);
      u = nu;
      v = nv;
    }
    uint32_t qu = (uint32_t)std::min(65535.0, std::max(0.0, (u + 1) * 0.5 * 65536.0));
    uint32_t qv = (uint32_t)std::min(65535.0, std::max(0.0, (v + 1) * 0.5 * 65536.0));
    uint64_t key = 0;
    for (int b = 0; b < 16; ++b) key |= (uint64_t)((qu >> b) & 1u) << (2 * b) | (uint64_t)((qv >> b) & 1u) << (2 * b + 1);
    keys[i] = {key, i};
  }
  std::sort(keys.begin(), keys.end());
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = keys[i].second;
  return order;
}

int applyTuning(DdgiGrid* g, const DdgiTuning& t) {
  DdgiContext* ctx = g->ctx;
  int minWp = std::max(1, 32 / g->g.N);
  if (t.warpProbes < minWp || t.warpProbes > 32 || (t.warpProbes & (t.warpProbes - 1)))
    return fail(ctx, DDGI_EINVAL, "warpProbes %d must be a power of two in [%d, 32]", t.warpProbes, minWp);
  if (t.rayOrder != 0 && t.rayOrder != 1) return fail(ctx, DDGI_EINVAL, "rayOrder %d unknown", t.rayOrder);
  if (t.shadowMode != 0 && t.shadowMode != 1) return fail(ctx, DDGI_EINVAL, "shadowMode %d unknown", t.shadowMode);
  if (t.bvhWidth != 0 && t.bvhWidth != 2 && t.bvhWidth != 8)
    return fail(ctx, DDGI_EINVAL, "bvhWidth %d must be 2 or 8 (0 = 8)", t.bvhWidth);
  if (t.refillLanes < 0 || t.refillLanes > 32) return fail(ctx, DDGI_EINVAL, "refillLanes %d not in [1, 32]", t.refillLanes);
  if (t.convMode < 0 || t.convMode > 2) return fail(ctx, DDGI_EINVAL, "convMode %d unknown", t.convMode);
  if (t.convMode != 0 && g->g.N % 64)
    return fail(ctx, DDGI_EINVAL, "tensor-core convolution needs raysPerProbe %% 64 == 0 (N = %d)", g->g.N);
  if (t.convMode != 0 && !g->rad16) {
    size_t bytes = (size_t)3 * g->g.X * g->g.Y * g->g.Z * g->g.N * 2;
    CK(gridAlloc(g, &g->rad16, bytes), "16-bit radiance buffer");
    CK(gridAlloc(g, &g->tcScratch, tcScratchBytes(g->g.N)), "tensor-core weight scratch");
  }
  std::vector<int> order(g->g.N);
  if (t.rayOrder == 1) order = mortonRayOrder(g->g.N);
  else for (int i = 0; i < g->g.N; ++i) order[i] = i;
  // the inverse after it: the shading walks rays in direction order and finds each one's trace slot
  order.resize(2 * (size_t)g->g.N);
  for (int i = 0; i < g->g.N; ++i) order[g->g.N + order[i]] = i;
  if (g->asyncAlloc)  // pageable source: the call returns once the data is staged
    CK(cudaMemcpyAsync(g->order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, g->allocStream),
       "ray order upload");
  else
    CK(cudaMemcpy(g->order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice), "ray order upload");
  g->tuning = t;
  if (g->tuning.bvhWidth == 0) g->tuning.bvhWidth = 8;
  if (g->tuning.refillLanes == 0) g->tuning.refillLanes = 8;
  setGridWarpProbes(g->g, t.warpProbes);
  g->g.bvhWide = g->tuning.bvhWidth == 8 ? 1 : 0;
  return DDGI_OK;
}

int frameToGPU(DdgiContext* ctx, const DdgiFrame* f, FrameGPU& out) {
  if (!f) return fail(ctx, DDGI_EINVAL, "frame is NULL");
  out.camPos = f3(f->cameraPos[0], f->cameraPos[1], f->cameraPos[2]);
  out.lightDir = f3(f->lightDir[0], f->lightDir[1], f->lightDir[2]);
  out.skyColor = f3(f->skyColor[0], f->skyColor[1], f->skyColor[2]);
  out.sunIntensity = f->sunIntensity;
  out.skyIntensity = f->skyIntensity;
  // the miss shader's sky (rmiss:20): toLinear (bindless.glsl:240-247) of skyIntensity * skyColor
  float sky[3];
  for (int k = 0; k < 3; ++k) {
    const float c = f->skyColor[k] * f->skyIntensity;
    sky[k] = c < 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f);
  }
  out.skyLinear = f3(sky[0], sky[1], sky[2]);
  out.flags = f->flags;
  for (int i = 0; i < 3; ++i) out.bakeTile[i] = f->bakeTileInfo[i];
  if ((f->flags & DDGI_UBO_BAKE_MODE_ON_FLAG) && f->bakeTileInfo[2] <= 0)
    return fail(ctx, DDGI_EINVAL, "bake mode needs bakeTileInfo[2] (tile size) > 0");
  return DDGI_OK;
}

// Layer range of a frame: -1 all, >= 0 one layer, -2 the grid's round-robin layer.
int layerRange(DdgiGrid* grid, int layer, bool advance, int& b, int& e) {
  if (layer == -1) { b = 0; e = grid->g.Y; return DDGI_OK; }
  if (layer == -2) {
    b = grid->currentLayer;
    e = b + 1;
    if (advance) grid->currentLayer = (grid->currentLayer + 1) % grid->g.Y;
    return DDGI_OK;
  }
  if (layer < 0 || layer >= grid->g.Y) return fail(grid->ctx, DDGI_EINVAL, "layer %d out of range", layer);
  b = layer;
  e = layer + 1;
  return DDGI_OK;
}

bool invert3(const float* m12, float* out9) {
  // inverse of the 3x3 part of a row-major 3x4 matrix, in double
  double a[9] = {m12[0], m12[1], m12[2], m12[4], m12[5], m12[6], m12[8], m12[9], m12[10]};
  double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
  double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  if (!(std::fabs(det) > 1e-30) || !std::isfinite(det)) return false;
  double inv[9] = {c00, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4],
                   c01, a[0] * a[8] - a[2] * a[6], a[2] * a[3] - a[0] * a[5],
                   c02, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]};
  for (int i = 0; i < 9; ++i) out9[i] = (float)(inv[i] / det);
  return true;
}

// Woop shear of a direction: kz = dominant axis, (kx, ky) the others (swapped when d[kz] < 0),
// S = (d[kx]/d[kz], d[ky]/d[kz], 1/d[kz]). shear(v) = (v[kx] - Sx v[kz], v[ky] - Sy v[kz], Sz v[kz]) maps d
// to (0, 0, 1) and keeps distances along d.
void shearOf(const double d[3], int k[3], double S[3]) {
  double ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
  if (d[kz] < 0) std::swap(kx, ky);
  k[0] = kx; k[1] = ky; k[2] = kz;
  S[0] = d[kx] / d[kz];
  S[1] = d[ky] / d[kz];
  S[2] = 1.0 / d[kz];
}

// Builds (or reuses) the shadow BVH of `sc` for light direction lightDir: the instance transforms are
// composed with the shear of L = normalize(-lightDir) on the host (FP64) and the LBVH is built over the
// sheared triangles. Synchronizes `st` when it builds.
// The scene's instances with their transforms composed with the shear of L = normalize(-lightDir) (FP64 on
// the host): the transforms of the light-space shadow BVH. k, S: the shear's axes and factors.
bool shearedInstances(const std::vector<InstanceGPU>& src, const float lightDir[3], std::vector<InstanceGPU>& out,
                      int k[3], double S[3]) {
  double n = std::sqrt((double)lightDir[0] * lightDir[0] + (double)lightDir[1] * lightDir[1] +
                       (double)lightDir[2] * lightDir[2]);
  if (!(n > 0)) return false;
  double L[3] = {-lightDir[0] / n, -lightDir[1] / n, -lightDir[2] / n};
  shearOf(L, k, S);
  double Sm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  Sm[0][k[0]] = 1.0; Sm[0][k[2]] = -S[0];
  Sm[1][k[1]] = 1.0; Sm[1][k[2]] = -S[1];
  Sm[2][k[2]] = S[2];
  out = src;
  for (InstanceGPU& in : out) {
    double m[12];
    for (int i = 0; i < 12; ++i) m[i] = in.o2w[i];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) {
        double v = 0;
        for (int q = 0; q < 3; ++q) v += Sm[r][q] * m[4 * q + c];
        in.o2w[4 * r + c] = (float)v;
      }
  }
  return true;
}

int ensureShadowBvh(DdgiScene* sc, const float lightDir[3], cudaStream_t st) {
  DdgiContext* ctx = sc->ctx;
  std::lock_guard<std::mutex> lk(sc->mu);
  if (sc->shadowValid && sc->shadowLight[0] == lightDir[0] && sc->shadowLight[1] == lightDir[1] &&
      sc->shadowLight[2] == lightDir[2])
    return DDGI_OK;
  if (sc->view.bvh.numTris == 0) return DDGI_OK;
  int k[3];
  double S[3];
  std::vector<InstanceGPU> sh;
  if (!shearedInstances(sc->hostInst, lightDir, sh, k, S)) return fail(ctx, DDGI_EINVAL, "lightDir has zero length");
  InstanceGPU* dInst = nullptr;
  CK(cudaMalloc(&dInst, sizeof(InstanceGPU) * sh.size()), "shadow instances");
  cudaError_t e = cudaMemcpyAsync(dInst, sh.data(), sizeof(InstanceGPU) * sh.size(), cudaMemcpyHostToDevice, st);
  LbvhResult r;
  if (e == cudaSuccess)
    e = lbvhBuild(dInst, (int)sh.size(), sc->meshes, sc->indices, sc->numIndices, sc->vertices, sc->numVertices,
                  sc->view.bvh.numTris, ctx->dErr, st, &r);
  cudaFree(dInst);
  if (e != cudaSuccess) return cudaFail(ctx, e, "shadow BVH build");
  lbvhFree(&sc->shadowBvh);
  sc->shadowBvh = r;
  for (int i = 0; i < 3; ++i) {
    sc->shadowLight[i] = lightDir[i];
    sc->view.shearK[i] = k[i];
    sc->view.shearS[i] = (float)S[i];
  }
  sc->view.shadow = BvhRef{r.nodes, r.wnodes, r.tris, r.numTris, r.numNodes, r.numWNodes};
  sc->shadowValid = true;
  return DDGI_OK;
}


int translateGrid(DdgiGrid* g, const float cameraPos[3], int* moved, cudaStream_t st) {
  DdgiContext* ctx = g->ctx;
  if (moved) *moved = 0;
  // IrradianceProbeTranslationPass.cpp:61-80: int() truncation, shift by the sign of the difference
  int ix = (int)(cameraPos[0] / g->desc.step[0]);
  int iz = (int)(cameraPos[2] / g->desc.step[2]);
  int dx = ix - g->lastProbeIdx[0], dz = iz - g->lastProbeIdx[1];
  if (dx == 0 && dz == 0) return DDGI_OK;
  g->lastProbeIdx[0] = ix;
  g->lastProbeIdx[1] = iz;
  int sx = dx > 0 ? 1 : (dx < 0 ? -1 : 0), sz = dz > 0 ? 1 : (dz < 0 ? -1 : 0);
  if (g->extAtlas || g->extTemp) {
    // a caller's buffer keeps its role: copy the atlas into the temp, shift it back (the reference's two
    // copies, IrradianceProbeTranslationPass.cpp:83-168)
    CK(cudaMemcpyAsync(g->atlas[1], g->atlas[0], g->atlasBytes, cudaMemcpyDeviceToDevice, st), "translation copy");
    CK(launchTranslate(g->g, g->atlas[1], g->atlas[0], sx, sz, st), "translate");
  } else {
    CK(launchTranslate(g->g, g->atlas[g->cur], g->atlas[1 - g->cur], sx, sz, st), "translate");
    g->cur = 1 - g->cur;
  }
  if (moved) *moved = 1;
  return DDGI_OK;
}


// Ray slots of a whole-grid trace for any warpProbes: ceil(XZ / wp) * wp <= XZ + 31 probes per layer.
long long maxRaySlots(const GridGPU& g) { return ((long long)g.X * g.Z + 31) * g.Y * g.N; }

uint64_t gridFootprint(const DdgiGridDesc* d, int convMode, bool hitSeeds) {
  GridGPU g = makeGridGPU(*d);
  uint64_t texel = d->atlasFormat == DDGI_FORMAT_RGBA32F ? 16 : 8;
  uint64_t rayTexel = g.rayFmt == DDGI_FORMAT_RGBA32F ? 16 : 8;
  uint64_t rays = (uint64_t)g.rayW * g.bh * g.Z * g.Y;
  uint64_t bytes = 2 * (uint64_t)g.atlasW * g.atlasH * texel + rayTexel * rays + 16ull * g.N + 24ull * g.N + 32ull * g.N +
                   8ull * g.N + 4ull * g.N * kOctTexels + 4ull * kOctTexels;
  if (d->options & DDGI_GRID_WRITE_DIRS) bytes += rayTexel * rays;
  if (d->options & DDGI_GRID_RECORD_HITS) bytes += 4 * rays;
  if (convMode != 0) bytes += 6 * rays + tcScratchBytes(g.N);
  bytes += kTraceScratchPerRay * (uint64_t)maxRaySlots(g);  // the launch's trace scratch for this grid
  if (hitSeeds) bytes += 20ull * g.N + 8ull * g.X * g.Y * g.Z * g.N;  // previous lattice, seed map, two memos
  return bytes;
}

int gridCreate(DdgiContext* ctx, const DdgiGridDesc* desc, cudaStream_t st, bool asyncAlloc, DdgiGrid** out) {
  *out = nullptr;
  int rc = validateGridDesc(ctx, desc);
  if (rc) return rc;
  CK(cudaSetDevice(ctx->device), "set device");
  DdgiGrid* g = new (std::nothrow) DdgiGrid();
  if (!g) return fail(ctx, DDGI_ENOMEM, "host allocation");
  g->ctx = ctx;
  g->desc = *desc;
  g->g = makeGridGPU(*desc);
  g->asyncAlloc = asyncAlloc;
  g->allocStream = st;
  size_t texel = desc->atlasFormat == DDGI_FORMAT_RGBA32F ? 16 : 8;
  g->atlasBytes = (uint64_t)g->g.atlasW * g->g.atlasH * texel;
  g->rayH = g->g.bh * g->g.Z * g->g.Y;
  size_t rayTexels = (size_t)g->g.rayW * g->rayH;
  g->rayBytes = (uint64_t)rayTexels * (g->g.rayFmt == DDGI_FORMAT_RGBA32F ? 16 : 8);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = gridAlloc(g, &g->atlas[0], g->atlasBytes);
  if (e == cudaSuccess) e = gridAlloc(g, &g->atlas[1], g->atlasBytes);
  if (e == cudaSuccess) e = gridAlloc(g, &g->rayRad, g->rayBytes);
  if (e == cudaSuccess && (desc->options & DDGI_GRID_WRITE_DIRS)) e = gridAlloc(g, &g->rayDir, g->rayBytes);
  if (e == cudaSuccess && (desc->options & DDGI_GRID_RECORD_HITS)) e = gridAlloc(g, (void**)&g->rayHit, 4 * rayTexels);
  if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->lattice, 16 * (size_t)g->g.N);
  if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->latticeUnit, 3 * sizeof(double) * (size_t)g->g.N);
  if (e == cudaSuccess) e = launchLatticeUnit(g->g.N, g->latticeUnit, st);
  if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->rayDirs, 2 * sizeof(float4) * (size_t)g->g.N);
  if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->order, 2 * sizeof(int) * (size_t)g->g.N);
  if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->wt, 4 * (size_t)g->g.N * kOctTexels);
  if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->wsum, 4 * kOctTexels);
  if (!asyncAlloc) {  // closest-hit seeding for grids traced frame after frame
    if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->latticePrev, 16 * (size_t)g->g.N);
    if (e == cudaSuccess) e = gridAlloc(g, (void**)&g->seedDir, sizeof(int) * (size_t)g->g.N);
    if (e == cudaSuccess)
      e = gridAlloc(g, (void**)&g->hitMemo, sizeof(int) * (size_t)g->g.X * g->g.Y * g->g.Z * g->g.N);
    if (e == cudaSuccess)
      e = gridAlloc(g, (void**)&g->occMemo, sizeof(int) * (size_t)g->g.X * g->g.Y * g->g.Z * g->g.N);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(g->rayRad, 0, g->rayBytes, st);
  if (e == cudaSuccess) e = launchClearAtlas(g->g, g->atlas[0], st);
  if (e == cudaSuccess && !asyncAlloc) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    gridDestroy(g);
    return cudaFail(ctx, e, "grid allocation");
  }
  DdgiTuning t{};
  t.warpProbes = std::max(1, 32 / g->g.N);
  t.rayOrder = 1;
  t.shadowMode = 1;
  t.bvhWidth = 8;
  int rc2 = applyTuning(g, t);
  if (rc2 != DDGI_OK) {
    gridDestroy(g);
    return rc2;
  }
  *out = g;
  return DDGI_OK;
}

void gridDestroy(DdgiGrid* g) {
  if (!g) return;
  // buffers bound by ddgi_grid_bind_external belong to the caller
  if (!g->extAtlas) gridFree(g, g->atlas[0]);
  if (!g->extTemp) gridFree(g, g->atlas[1]);
  if (!g->extRays) gridFree(g, g->rayRad);
  if (!g->extDirs) gridFree(g, g->rayDir);
  gridFree(g, g->rayHit);
  gridFree(g, g->lattice);
  gridFree(g, g->latticeUnit);
  gridFree(g, g->rayDirs);
  gridFree(g, g->order);
  gridFree(g, g->latticePrev);
  gridFree(g, g->seedDir);
  gridFree(g, g->hitMemo);
  gridFree(g, g->occMemo);
  gridFree(g, g->rad16);
  gridFree(g, g->tcScratch);
  gridFree(g, g->wt);
  gridFree(g, g->wsum);
  cudaFree(g->dQueue);
  cudaFree(g->dHits);
  if (g->dlDone) cudaEventSynchronize(g->dlDone);  // no copy to the host still reads the staging buffer
  cudaFree(g->dlStage);
  if (g->dlSnap) cudaEventDestroy(g->dlSnap);
  if (g->dlDone) cudaEventDestroy(g->dlDone);
  if (g->dlStream) cudaStreamDestroy(g->dlStream);
  delete g;
}

// Counters and scratch of the single-grid trace (ddgi_trace), allocated on first use.
int ensureSoloRecords(DdgiGrid* g) {
  if (g->dQueue) return DDGI_OK;
  DdgiContext* ctx = g->ctx;
  const long long slots = maxRaySlots(g->g);
  if (allocRefused(ctx, kTraceScratchPerRay * (size_t)slots + kTraceCounters * sizeof(unsigned long long)))
    return fail(ctx, DDGI_ENOMEM, "trace scratch: refused by the allocation hook");
  CK(cudaMalloc(&g->dQueue, kTraceCounters * sizeof(unsigned long long)), "trace counters");
  CK(cudaMalloc(&g->dHits, kTraceScratchPerRay * (size_t)slots), "trace scratch");
  g->dShadow = g->dHits + slots;
  return DDGI_OK;
}

}  // namespace detail
}  // namespace ddgi

using namespace ddgi::detail;

extern "C" {

int ddgi_abi_version(void) { return DDGI_ABI_VERSION; }

int ddgi_context_set_waits(DdgiContext* ctx, const DdgiWaitConfig* cfg) {
  if (!ctx || !cfg) return fail(ctx, DDGI_EINVAL, "NULL argument to ddgi_context_set_waits");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->waits.spin = cfg->spinLimit ? cfg->spinLimit : WaitCfg{}.spin;
  ctx->waits.stall = cfg->stallTest ? 1u : 0u;
  return DDGI_OK;
}

int ddgi_context_set_alloc_hook(DdgiContext* ctx, DdgiAllocHook hook, void* user) {
  if (!ctx) return DDGI_EINVAL;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->allocHook = hook;
  ctx->allocUser = user;
  return DDGI_OK;
}

int ddgi_context_create(int device, DdgiContext** out) {
  if (!out) return DDGI_EINVAL;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return DDGI_EDEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return DDGI_EDEVICE;
  DdgiContext* ctx = new (std::nothrow) DdgiContext();
  if (!ctx) return DDGI_ENOMEM;
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->numSms, cudaDevAttrMultiProcessorCount, device);
  if (cudaMalloc(&ctx->dErr, sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(ctx->dErr, 0, sizeof(uint32_t)) != cudaSuccess) {
    cudaFree(ctx->dErr);
    delete ctx;
    return DDGI_ENOMEM;
  }
  *out = ctx;
  return DDGI_OK;
}

void ddgi_context_destroy(DdgiContext* ctx) {
  if (!ctx) return;
  cudaFree(ctx->dErr);
  delete ctx;
}

const char* ddgi_last_error(const DdgiContext* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int ddgi_sync(DdgiContext* ctx, void* stream) {
  if (!ctx) return DDGI_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaStreamSynchronize(s), "stream synchronize");
  uint32_t w = 0;
  CK(cudaMemcpy(&w, ctx->dErr, sizeof(w), cudaMemcpyDeviceToHost), "read device error word");
  if (w) {
    CK(cudaMemset(ctx->dErr, 0, sizeof(uint32_t)), "clear device error word");
    if (w & DDGI_DEVERR_STACK_OVERFLOW) return fail(ctx, DDGI_EOVERFLOW, "traversal stack overflow (word 0x%x)", w);
    if (w & DDGI_DEVERR_TIMEOUT) return fail(ctx, DDGI_ETIMEDOUT, "device wait timed out (word 0x%x)", w);
    return fail(ctx, DDGI_EOVERFLOW, "device bounds check failed (word 0x%x)", w);
  }
  return DDGI_OK;
}

// ---- scene ------------------------------------------------------------------------------------------
int ddgi_scene_create(DdgiContext* ctx, const DdgiSceneDesc* d, void* stream, DdgiScene** out) {
  if (!ctx || !d || !out) return fail(ctx, DDGI_EINVAL, "NULL argument to ddgi_scene_create");
  *out = nullptr;
  if (d->numMeshes && !d->meshes) return fail(ctx, DDGI_EINVAL, "meshes is NULL");
  if (d->numInstances && !d->instances) return fail(ctx, DDGI_EINVAL, "instances is NULL");
  if (d->numMaterials && !d->materials) return fail(ctx, DDGI_EINVAL, "materials is NULL");
  if (d->numVertices && !d->vertices) return fail(ctx, DDGI_EINVAL, "vertices is NULL");
  if (d->numIndices && !d->indices) return fail(ctx, DDGI_EINVAL, "indices is NULL");
  // meshes: ranges inside the arrays, every index inside its mesh's vertex range
  for (uint32_t m = 0; m < d->numMeshes; ++m) {
    const DdgiMeshInfo& mi = d->meshes[m];
    if (mi.numIndices % 3) return fail(ctx, DDGI_EINVAL, "mesh %u: numIndices %u not a multiple of 3", m, mi.numIndices);
    if ((uint64_t)mi.indexOffset + mi.numIndices > d->numIndices)
      return fail(ctx, DDGI_EINVAL, "mesh %u: index range beyond numIndices", m);
    if ((uint64_t)mi.vertexOffset + mi.numVertices > d->numVertices)
      return fail(ctx, DDGI_EINVAL, "mesh %u: vertex range beyond numVertices", m);
    for (uint32_t k = 0; k < mi.numIndices; ++k)
      if (d->indices[(uint64_t)mi.indexOffset + k] >= mi.numVertices)
        return fail(ctx, DDGI_EINVAL, "mesh %u: index %u out of its vertex range", m, k);
  }
  for (uint32_t m = 0; m < d->numMaterials; ++m)
    for (int k = 0; k < 4; ++k)
      if (d->materials[m].bindlessIndices[k] != -1)
        return fail(ctx, DDGI_EUNSUPPORTED, "material %u: textures are not supported (bindlessIndices[%d] != -1)", m, k);
  std::vector<InstanceGPU> inst(d->numInstances);
  uint64_t tris = 0;
  for (uint32_t i = 0; i < d->numInstances; ++i) {
    const DdgiInstance& s = d->instances[i];
    if (s.mesh >= d->numMeshes) return fail(ctx, DDGI_EINVAL, "instance %u: mesh %u out of range", i, s.mesh);
    if (s.material >= d->numMaterials) return fail(ctx, DDGI_EINVAL, "instance %u: material %u out of range", i, s.material);
    InstanceGPU& g = inst[i];
    memcpy(g.o2w, s.transform, sizeof(g.o2w));
    if (!invert3(s.transform, g.w2oLin)) return fail(ctx, DDGI_EINVAL, "instance %u: singular transform", i);
    g.mesh = s.mesh;
    g.material = s.material;
    g.triOffset = (uint32_t)tris;
    tris += d->meshes[s.mesh].numIndices / 3;
  }
  if (tris >= (1ull << 30)) return fail(ctx, DDGI_EINVAL, "too many triangles (%llu)", (unsigned long long)tris);
  CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t st = (cudaStream_t)stream;
  DdgiScene* sc = new (std::nothrow) DdgiScene();
  if (!sc) return fail(ctx, DDGI_ENOMEM, "host allocation");
  sc->ctx = ctx;
  auto up = [&](void** dst, const void* src, size_t bytes) -> cudaError_t {
    if (!bytes) return cudaSuccess;
    if (allocRefused(ctx, bytes)) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(dst, bytes);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = up((void**)&sc->vertices, d->vertices, sizeof(DdgiPackedVertex) * d->numVertices);
  if (e == cudaSuccess) e = up((void**)&sc->indices, d->indices, sizeof(uint32_t) * d->numIndices);
  if (e == cudaSuccess) e = up((void**)&sc->meshes, d->meshes, sizeof(DdgiMeshInfo) * d->numMeshes);
  if (e == cudaSuccess) e = up((void**)&sc->instances, inst.data(), sizeof(InstanceGPU) * inst.size());
  if (e == cudaSuccess) e = up((void**)&sc->materials, d->materials, sizeof(DdgiMaterialInfo) * d->numMaterials);
  if (e == cudaSuccess)
    e = lbvhBuild(sc->instances, (int)d->numInstances, sc->meshes, sc->indices, d->numIndices, sc->vertices,
                  d->numVertices, (int)tris, ctx->dErr, st, &sc->bvh);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    ddgi_scene_destroy(sc);
    return cudaFail(ctx, e, "scene upload / BVH build");
  }
  sc->view.bvh = BvhRef{sc->bvh.nodes, sc->bvh.wnodes, sc->bvh.tris, (int)tris, sc->bvh.numNodes, sc->bvh.numWNodes};
  sc->view.shadow = BvhRef{};
  sc->view.vertices = sc->vertices;
  sc->view.indices = sc->indices;
  sc->view.meshes = sc->meshes;
  sc->view.instances = sc->instances;
  sc->view.materials = sc->materials;
  if (tris > 0) {
    e = allocRefused(ctx, 48ull * tris) ? cudaErrorMemoryAllocation : cudaMalloc(&sc->shade, 48ull * tris);
    if (e == cudaSuccess) {
      sc->view.shade = sc->shade;
      e = launchShadingRecords(sc->view, d->numIndices, d->numVertices, sc->shade, ctx->dErr, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      ddgi_scene_destroy(sc);
      return cudaFail(ctx, e, "scene shading records");
    }
  }
  sc->info.numTriangles = tris;
  sc->info.numNodes = (uint64_t)sc->bvh.numNodes;
  sc->info.deviceBytes = sizeof(DdgiPackedVertex) * d->numVertices + 4ull * d->numIndices +
                         sizeof(DdgiMeshInfo) * d->numMeshes + sizeof(InstanceGPU) * inst.size() +
                         sizeof(DdgiMaterialInfo) * d->numMaterials + 48ull * tris + 48ull * tris +
                         64ull * (tris > 1 ? tris - 1 : 1) + 208ull * (uint64_t)sc->bvh.numWNodes;
  for (int k = 0; k < 3; ++k) {
    sc->info.boundsMin[k] = sc->bvh.centroidLo[k];
    sc->info.boundsMax[k] = sc->bvh.centroidHi[k];
  }
  sc->hostInst = inst;
  sc->numIndices = d->numIndices;
  sc->numVertices = d->numVertices;
  *out = sc;
  return DDGI_OK;
}

namespace {
// Brings the scene BVH and, if built, the light-space shadow BVH up to date with the scene's current
// instances and vertices. Synchronizes st.
int updateBvhs(DdgiScene* sc, int mode, cudaStream_t st) {
  DdgiContext* ctx = sc->ctx;
  std::lock_guard<std::mutex> lk(sc->mu);
  const int tris = sc->view.bvh.numTris;
  const int numInst = (int)sc->hostInst.size();
  if (tris == 0) return DDGI_OK;
  auto refresh = [&](LbvhResult& bvh, const InstanceGPU* dInst) -> cudaError_t {
    if (mode == DDGI_SCENE_REFIT) {
      cudaError_t e = lbvhRefit(&bvh, dInst, sc->meshes, sc->indices, sc->numIndices, sc->vertices, sc->numVertices,
                                ctx->dErr, st);
      if (e != cudaErrorNotSupported) return e;
    }
    LbvhResult r;
    cudaError_t e = lbvhBuild(dInst, numInst, sc->meshes, sc->indices, sc->numIndices, sc->vertices, sc->numVertices,
                              tris, ctx->dErr, st, &r);
    if (e != cudaSuccess) return e;
    lbvhFree(&bvh);
    bvh = r;
    return cudaSuccess;
  };
  cudaError_t e = refresh(sc->bvh, sc->instances);
  if (e != cudaSuccess) return cudaFail(ctx, e, "scene BVH update");
  sc->view.bvh = BvhRef{sc->bvh.nodes, sc->bvh.wnodes, sc->bvh.tris, tris, sc->bvh.numNodes, sc->bvh.numWNodes};
  e = launchShadingRecords(sc->view, sc->numIndices, sc->numVertices, sc->shade, ctx->dErr, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cudaFail(ctx, e, "scene shading records");
  if (sc->shadowValid) {
    int k[3];
    double S[3];
    std::vector<InstanceGPU> sh;
    shearedInstances(sc->hostInst, sc->shadowLight, sh, k, S);
    InstanceGPU* dInst = nullptr;
    CK(cudaMalloc(&dInst, sizeof(InstanceGPU) * sh.size()), "shadow instances");
    e = cudaMemcpyAsync(dInst, sh.data(), sizeof(InstanceGPU) * sh.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = refresh(sc->shadowBvh, dInst);
    cudaStreamSynchronize(st);
    cudaFree(dInst);
    if (e != cudaSuccess) {
      sc->shadowValid = false;
      return cudaFail(ctx, e, "shadow BVH update");
    }
    const LbvhResult& r = sc->shadowBvh;
    sc->view.shadow = BvhRef{r.nodes, r.wnodes, r.tris, r.numTris, r.numNodes, r.numWNodes};
  }
  return DDGI_OK;
}
}  // namespace

int ddgi_scene_update_transforms(DdgiScene* sc, const float* transforms, uint64_t numInstances, int mode,
                                 void* stream) {
  if (!sc || !transforms) return fail(sc ? sc->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_scene_update_transforms");
  DdgiContext* ctx = sc->ctx;
  if (mode != DDGI_SCENE_REFIT && mode != DDGI_SCENE_REBUILD) return fail(ctx, DDGI_EINVAL, "mode %d unknown", mode);
  if (numInstances != sc->hostInst.size())
    return fail(ctx, DDGI_EINVAL, "the scene has %zu instances, got %llu transforms", sc->hostInst.size(),
                (unsigned long long)numInstances);
  std::vector<InstanceGPU> inst = sc->hostInst;
  for (size_t i = 0; i < inst.size(); ++i) {
    memcpy(inst[i].o2w, transforms + 12 * i, sizeof(inst[i].o2w));
    if (!invert3(inst[i].o2w, inst[i].w2oLin)) return fail(ctx, DDGI_EINVAL, "instance %zu: singular transform", i);
  }
  cudaStream_t st = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(sc->instances, inst.data(), sizeof(InstanceGPU) * inst.size(), cudaMemcpyHostToDevice, st),
     "instance upload");
  sc->hostInst = inst;
  return updateBvhs(sc, mode, st);
}

int ddgi_scene_update_vertices(DdgiScene* sc, const DdgiPackedVertex* vertices, uint64_t first, uint64_t count,
                               int mode, void* stream) {
  if (!sc || (count && !vertices)) return fail(sc ? sc->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_scene_update_vertices");
  DdgiContext* ctx = sc->ctx;
  if (mode != DDGI_SCENE_REFIT && mode != DDGI_SCENE_REBUILD) return fail(ctx, DDGI_EINVAL, "mode %d unknown", mode);
  if (first > sc->numVertices || count > sc->numVertices - first)
    return fail(ctx, DDGI_EINVAL, "vertex range [%llu, +%llu) beyond the scene's %llu vertices", (unsigned long long)first,
                (unsigned long long)count, (unsigned long long)sc->numVertices);
  cudaStream_t st = (cudaStream_t)stream;
  if (count)
    CK(cudaMemcpyAsync(sc->vertices + first, vertices, sizeof(DdgiPackedVertex) * count, cudaMemcpyHostToDevice, st),
       "vertex upload");
  return updateBvhs(sc, mode, st);
}

void ddgi_scene_destroy(DdgiScene* s) {
  if (!s) return;
  cudaFree(s->vertices);
  cudaFree(s->indices);
  cudaFree(s->meshes);
  cudaFree(s->instances);
  cudaFree(s->materials);
  cudaFree(s->shade);
  lbvhFree(&s->bvh);
  lbvhFree(&s->shadowBvh);
  delete s;
}

int ddgi_scene_info(const DdgiScene* s, DdgiSceneInfo* info) {
  if (!s || !info) return DDGI_EINVAL;
  *info = s->info;
  return DDGI_OK;
}

// ---- grid -------------------------------------------------------------------------------------------
int ddgi_grid_create(DdgiContext* ctx, const DdgiGridDesc* desc, DdgiGrid** out) {
  if (!ctx || !out) return fail(ctx, DDGI_EINVAL, "NULL argument to ddgi_grid_create");
  return gridCreate(ctx, desc, nullptr, false, out);
}

void ddgi_grid_destroy(DdgiGrid* g) { gridDestroy(g); }

uint64_t ddgi_grid_footprint(const DdgiGridDesc* desc, int convMode) {
  if (validateGridDesc(nullptr, desc) != DDGI_OK) return 0;
  return gridFootprint(desc, convMode, true);
}

int ddgi_grid_buffers(const DdgiGrid* g, DdgiGridBuffers* o) {
  if (!g || !o) return DDGI_EINVAL;
  o->atlas = g->atlas[g->cur];
  o->rayRadiance = g->rayRad;
  o->rayDirection = g->rayDir;
  o->rayHit = g->rayHit;
  o->lattice = (float*)g->lattice;
  o->atlasWidth = g->g.atlasW;
  o->atlasHeight = g->g.atlasH;
  o->rayWidth = g->g.rayW;
  o->rayHeight = g->rayH;
  o->rayBlockW = g->g.bw;
  o->rayBlockH = g->g.bh;
  o->atlasBytes = g->atlasBytes;
  o->rayBytes = g->rayBytes;
  o->rayFormat = g->g.rayFmt;
  o->reserved = 0;
  return DDGI_OK;
}

int ddgi_grid_bind_external(DdgiGrid* g, const DdgiGridExternal* x, void* stream) {
  if (!g || !x) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_grid_bind_external");
  DdgiContext* ctx = g->ctx;
  auto misaligned = [](const void* p) { return ((uintptr_t)p & 15) != 0; };
  if (misaligned(x->atlas) || misaligned(x->atlasTemp) || misaligned(x->rayRadiance) || misaligned(x->rayDirection))
    return fail(ctx, DDGI_EINVAL, "external buffers must be 16-byte aligned");
  if ((x->atlas || x->atlasTemp) && x->atlasBytes != g->atlasBytes)
    return fail(ctx, DDGI_EINVAL, "external atlas must be %llu bytes, got %llu", (unsigned long long)g->atlasBytes,
                (unsigned long long)x->atlasBytes);
  if ((x->rayRadiance || x->rayDirection) && x->rayBytes != g->rayBytes)
    return fail(ctx, DDGI_EINVAL, "external ray images must be %llu bytes, got %llu", (unsigned long long)g->rayBytes,
                (unsigned long long)x->rayBytes);
  if (x->rayDirection && !(g->desc.options & DDGI_GRID_WRITE_DIRS))
    return fail(ctx, DDGI_EINVAL, "the grid writes no direction image (DDGI_GRID_WRITE_DIRS)");
  if (x->atlas && x->atlas == x->atlasTemp) return fail(ctx, DDGI_EINVAL, "atlas and atlasTemp must differ");
  if (g->asyncAlloc) return fail(ctx, DDGI_EINVAL, "served grids take no external buffers");
  // nothing in flight may still use the buffers released below
  CK(cudaSetDevice(ctx->device), "set device");
  CK(cudaStreamSynchronize((cudaStream_t)stream), "bind sync");
  if (g->dlDone) CK(cudaEventSynchronize(g->dlDone), "bind sync");
  CK(cudaDeviceSynchronize(), "bind sync");
  if (x->atlas || x->atlasTemp) {
    // roles, not slots: the current atlas and the temp (a grid that never had a binding swaps them on a move);
    // from now on the current atlas is slot 0, the temp slot 1, and translations copy instead of swapping
    void* cur = g->atlas[g->cur];
    void* tmp = g->atlas[1 - g->cur];
    bool curExt = g->extAtlas, tmpExt = g->extTemp;
    if (x->atlas) {
      if (!curExt) gridFree(g, cur);
      cur = x->atlas;
      curExt = true;
    }
    if (x->atlasTemp) {
      if (!tmpExt) gridFree(g, tmp);
      tmp = x->atlasTemp;
      tmpExt = true;
    }
    g->atlas[0] = cur;
    g->atlas[1] = tmp;
    g->cur = 0;
    g->extAtlas = curExt;
    g->extTemp = tmpExt;
  }
  if (x->rayRadiance) {
    if (!g->extRays) gridFree(g, g->rayRad);
    g->rayRad = x->rayRadiance;
    g->extRays = true;
  }
  if (x->rayDirection) {
    if (!g->extDirs) gridFree(g, g->rayDir);
    g->rayDir = x->rayDirection;
    g->extDirs = true;
  }
  return DDGI_OK;
}

int ddgi_grid_get_tuning(const DdgiGrid* g, DdgiTuning* out) {
  if (!g || !out) return DDGI_EINVAL;
  *out = g->tuning;
  return DDGI_OK;
}

int ddgi_grid_set_tuning(DdgiGrid* g, const DdgiTuning* t) {
  if (!g || !t) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_grid_set_tuning");
  return applyTuning(g, *t);
}

int ddgi_grid_reset(DdgiGrid* g, void* stream) {
  if (!g) return DDGI_EINVAL;
  DdgiContext* ctx = g->ctx;
  CK(launchClearAtlas(g->g, g->atlas[g->cur], (cudaStream_t)stream), "clear atlas");
  g->lastProbeIdx[0] = g->lastProbeIdx[1] = 0;
  g->currentLayer = 0;
  return DDGI_OK;
}

int ddgi_translate(DdgiGrid* g, const float cameraPos[3], int* moved, void* stream) {
  if (!g || !cameraPos) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_translate");
  return translateGrid(g, cameraPos, moved, (cudaStream_t)stream);
}

int ddgi_trace(DdgiGrid* g, const DdgiScene* scene, const DdgiFrame* frame, void* stream) {
  if (!g || !scene || !frame) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_trace");
  DdgiContext* ctx = g->ctx;
  if (scene->ctx != ctx) return fail(ctx, DDGI_EINVAL, "scene belongs to another context");
  FrameGPU f{};
  int rc = frameToGPU(ctx, frame, f);
  if (rc) return rc;
  setFrameGrid(f, g->g);
  int b, e;
  rc = layerRange(g, frame->layer, true, b, e);
  if (rc) return rc;
  f.layerBegin = b;
  f.layerEnd = e;
  cudaStream_t st = (cudaStream_t)stream;
  SceneGPU view = scene->view;
  if (g->tuning.shadowMode == 1) {
    rc = ensureShadowBvh(const_cast<DdgiScene*>(scene), frame->lightDir, st);
    if (rc) return rc;
    view = scene->view;
  } else {
    view.shadow = BvhRef{};
  }
  GridGPU gg = g->g;
  g->rad16Written = false;
  if (g->tuning.convMode != 0) {
    gg.rad16 = g->rad16;
    gg.rad16Fmt = g->tuning.convMode == 1 ? DDGI_ELEM_F16 : DDGI_ELEM_BF16;
    gg.pTotal = g->g.X * g->g.Y * g->g.Z;
  }
  // the persistent batched kernels with one item (the same code the batched form runs)
  rc = ensureSoloRecords(g);
  if (rc) return rc;
  // the record and rotation travel in the kernel parameters: nothing is copied ahead of the launches
  TraceItem ti{};
  ti.s = view;
  ti.g = gg;
  ti.f = f;
  ti.lattice = g->lattice;
  ti.latticeUnit = g->latticeUnit;
  ti.rayDirs = g->rayDirs;
  ti.order = g->order;
  ti.atlasPrev = g->atlas[g->cur];
  ti.atlasPairs = ((uintptr_t)ti.atlasPrev & (g->g.atlasFmt == DDGI_FORMAT_RGBA32F ? 31 : 15)) == 0;
  ti.rayRad = g->rayRad;
  ti.rayDir = g->rayDir;
  ti.rayHit = g->rayHit;
  ti.warpBegin = 0;
  ti.latticePrev = g->latticePrev;
  ti.seedDir = g->seedDir;
  ti.hitMemo = g->hitMemo;
  ti.occMemo = g->occMemo;
  ti.seedOn = g->memoValid ? 1 : 0;
  Mat3 rot;
  memcpy(rot.m, frame->rotation, sizeof(rot.m));
  CK(launchTraceBatch(nullptr, nullptr, 1, g->g.N, traceWarps(gg, f), g->dQueue, g->dHits, g->dShadow,
                      ctx->numSms * 8, g->tuning.refillLanes, g->tuning.bvhWidth != 2, g->tuning.shadowMode == 1,
                      ctx->dErr, st, &ti, &rot),
     "trace");
  g->tracedBegin = b;
  g->tracedEnd = e;
  g->latticeValid = true;
  g->memoValid = g->hitMemo != nullptr;
  g->rad16Written = gg.rad16 != nullptr;
  return DDGI_OK;
}

int ddgi_convolve(DdgiGrid* g, const DdgiFrame* frame, void* stream) {
  if (!g || !frame) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_convolve");
  DdgiContext* ctx = g->ctx;
  if (!g->latticeValid) return fail(ctx, DDGI_EINVAL, "ddgi_convolve before any ddgi_trace on this grid");
  int b, e;
  if (frame->layer == -2) {  // the layer the last trace wrote (blackboard "ProbeLayer")
    b = g->tracedBegin;
    e = g->tracedEnd;
  } else {
    int rc = layerRange(g, frame->layer, false, b, e);
    if (rc) return rc;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (g->tuning.convMode != 0) {
    int fmt = g->tuning.convMode == 1 ? DDGI_ELEM_F16 : DDGI_ELEM_BF16;
    int pTotal = g->g.X * g->g.Y * g->g.Z;
    if (!g->rad16Written || b < g->tracedBegin || e > g->tracedEnd)
      CK(launchPackRays16(g->g, fmt, g->rayRad, g->rad16, b, e, pTotal, st), "pack rays");
    CK(launchConvTc(g->g, fmt, g->rad16, pTotal, g->lattice, g->tcScratch, g->atlas[g->cur], b, e, g->desc.hysteresis,
                    frame->flags, ctx->dErr, st, ctx->waits),
       "tensor-core convolve");
    return DDGI_OK;
  }
  // the record travels in the kernel parameters (no copy to the device ahead of the launch); the weights
  // and tile kernels are those of the batched form
  CK(launchConvWeights(g->g.N, g->lattice, g->wt, g->wsum, st), "convolve weights");
  CK(launchConvFp32(g->g, g->rayRad, g->wt, g->wsum, g->atlas[g->cur], b, e, g->desc.hysteresis, frame->flags, st),
     "convolve");
  return DDGI_OK;
}

int ddgi_update(DdgiGrid* g, const DdgiScene* scene, const DdgiFrame* frame, void* stream) {
  if (!g || !scene || !frame) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_update");
  int rc = DDGI_OK;
  if (!(frame->flags & DDGI_UBO_BAKE_MODE_ON_FLAG)) {  // translation is skipped while baking (:59)
    rc = ddgi_translate(g, frame->cameraPos, nullptr, stream);
    if (rc) return rc;
  }
  rc = ddgi_trace(g, scene, frame, stream);
  if (rc) return rc;
  // layer -2 convolves the layer the trace just picked (the "ProbeLayer" blackboard value)
  return ddgi_convolve(g, frame, stream);
}

int ddgi_atlas_download(DdgiGrid* g, void* host, uint64_t bytes, void* stream) {
  if (!g || !host) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_atlas_download");
  DdgiContext* ctx = g->ctx;
  if (bytes != g->atlasBytes) return fail(ctx, DDGI_EINVAL, "atlas is %llu bytes, got %llu",
                                          (unsigned long long)g->atlasBytes, (unsigned long long)bytes);
  cudaStream_t st = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(host, g->atlas[g->cur], bytes, cudaMemcpyDeviceToHost, st), "atlas download");
  CK(cudaStreamSynchronize(st), "atlas download sync");
  return DDGI_OK;
}

int ddgi_atlas_download_async(DdgiGrid* g, void* host, uint64_t bytes, void* stream) {
  if (!g || !host) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_atlas_download_async");
  DdgiContext* ctx = g->ctx;
  if (bytes != g->atlasBytes) return fail(ctx, DDGI_EINVAL, "atlas is %llu bytes, got %llu",
                                          (unsigned long long)g->atlasBytes, (unsigned long long)bytes);
  if (!g->dlStage) {
    if (allocRefused(ctx, g->atlasBytes)) return fail(ctx, DDGI_ENOMEM, "atlas download staging: refused by the allocation hook");
    CK(cudaMalloc(&g->dlStage, g->atlasBytes), "atlas download staging");
    CK(cudaStreamCreateWithFlags(&g->dlStream, cudaStreamNonBlocking), "atlas download stream");
    CK(cudaEventCreateWithFlags(&g->dlSnap, cudaEventDisableTiming), "atlas download event");
    CK(cudaEventCreateWithFlags(&g->dlDone, cudaEventDisableTiming), "atlas download event");
  }
  cudaStream_t st = (cudaStream_t)stream;
  // the staging buffer is free once the previous copy to the host has ended
  if (g->dlPending) CK(cudaStreamWaitEvent(st, g->dlDone, 0), "atlas download order");
  CK(cudaMemcpyAsync(g->dlStage, g->atlas[g->cur], bytes, cudaMemcpyDeviceToDevice, st), "atlas snapshot");
  CK(cudaEventRecord(g->dlSnap, st), "atlas snapshot event");
  CK(cudaStreamWaitEvent(g->dlStream, g->dlSnap, 0), "atlas download order");
  CK(cudaMemcpyAsync(host, g->dlStage, bytes, cudaMemcpyDeviceToHost, g->dlStream), "atlas download");
  CK(cudaEventRecord(g->dlDone, g->dlStream), "atlas download event");
  g->dlPending = true;
  return DDGI_OK;
}

int ddgi_atlas_download_wait(DdgiGrid* g) {
  if (!g) return fail(nullptr, DDGI_EINVAL, "NULL argument to ddgi_atlas_download_wait");
  DdgiContext* ctx = g->ctx;
  if (g->dlPending) {
    CK(cudaEventSynchronize(g->dlDone), "atlas download wait");
    g->dlPending = false;
  }
  return DDGI_OK;
}

int ddgi_atlas_upload(DdgiGrid* g, const void* host, uint64_t bytes, void* stream) {
  if (!g || !host) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_atlas_upload");
  DdgiContext* ctx = g->ctx;
  if (bytes != g->atlasBytes) return fail(ctx, DDGI_EINVAL, "atlas is %llu bytes, got %llu",
                                          (unsigned long long)g->atlasBytes, (unsigned long long)bytes);
  cudaStream_t st = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(g->atlas[g->cur], host, bytes, cudaMemcpyHostToDevice, st), "atlas upload");
  CK(cudaStreamSynchronize(st), "atlas upload sync");
  return DDGI_OK;
}

int ddgi_atlas_export_rgba16f(DdgiGrid* g, void* host, uint64_t bytes, void* stream) {
  if (!g || !host) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_atlas_export_rgba16f");
  DdgiContext* ctx = g->ctx;
  const long long texels = (long long)g->g.atlasW * g->g.atlasH;
  if (bytes != 8ull * (uint64_t)texels) return fail(ctx, DDGI_EINVAL, "RGBA16F atlas is %llu bytes", 8ull * texels);
  cudaStream_t st = (cudaStream_t)stream;
  if (g->desc.atlasFormat == DDGI_FORMAT_RGBA16F) {
    CK(cudaMemcpyAsync(host, g->atlas[g->cur], bytes, cudaMemcpyDeviceToHost, st), "atlas export");
  } else {
    void* tmp = nullptr;
    CK(cudaMallocAsync(&tmp, bytes, st), "atlas export scratch");
    cudaError_t e = launchAtlasToHalf((const float4*)g->atlas[g->cur], tmp, texels, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, tmp, bytes, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(tmp, st);
    if (e != cudaSuccess) return cudaFail(ctx, e, "atlas export");
  }
  CK(cudaStreamSynchronize(st), "atlas export sync");
  return DDGI_OK;
}

int ddgi_atlas_import_rgba16f(DdgiGrid* g, const void* host, uint64_t bytes, void* stream) {
  if (!g || !host) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_atlas_import_rgba16f");
  DdgiContext* ctx = g->ctx;
  const long long texels = (long long)g->g.atlasW * g->g.atlasH;
  if (bytes != 8ull * (uint64_t)texels) return fail(ctx, DDGI_EINVAL, "RGBA16F atlas is %llu bytes", 8ull * texels);
  cudaStream_t st = (cudaStream_t)stream;
  if (g->desc.atlasFormat == DDGI_FORMAT_RGBA16F) {
    CK(cudaMemcpyAsync(g->atlas[g->cur], host, bytes, cudaMemcpyHostToDevice, st), "atlas import");
  } else {
    void* tmp = nullptr;
    CK(cudaMallocAsync(&tmp, bytes, st), "atlas import scratch");
    cudaError_t e = cudaMemcpyAsync(tmp, host, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launchAtlasFromHalf(tmp, (float4*)g->atlas[g->cur], texels, st);
    cudaFreeAsync(tmp, st);
    if (e != cudaSuccess) return cudaFail(ctx, e, "atlas import");
  }
  CK(cudaStreamSynchronize(st), "atlas import sync");
  return DDGI_OK;
}

int ddgi_rays_download(DdgiGrid* g, void* radiance, int32_t* hits, float* lattice, void* stream) {
  if (!g) return DDGI_EINVAL;
  DdgiContext* ctx = g->ctx;
  cudaStream_t st = (cudaStream_t)stream;
  size_t texels = (size_t)g->g.rayW * g->rayH;
  if (hits && !g->rayHit) return fail(ctx, DDGI_EINVAL, "grid was created without DDGI_GRID_RECORD_HITS");
  if (radiance) CK(cudaMemcpyAsync(radiance, g->rayRad, g->rayBytes, cudaMemcpyDeviceToHost, st), "ray download");
  if (hits) CK(cudaMemcpyAsync(hits, g->rayHit, 4 * texels, cudaMemcpyDeviceToHost, st), "hit download");
  if (lattice) CK(cudaMemcpyAsync(lattice, g->lattice, 16 * (size_t)g->g.N, cudaMemcpyDeviceToHost, st), "lattice download");
  CK(cudaStreamSynchronize(st), "ray download sync");
  return DDGI_OK;
}

namespace {
int traceQuery(DdgiScene* sc, const DdgiRay* rays, const float* points, uint64_t count, bool anyHit, DdgiHit* hits,
               float3 shadowDir, float* vis, cudaStream_t st) {
  DdgiContext* ctx = sc->ctx;
  if (count == 0) return DDGI_OK;
  unsigned long long* counter = nullptr;
  CK(cudaMallocAsync(&counter, sizeof(unsigned long long), st), "ray query counter");
  cudaError_t e = launchTraceRays(sc->view.bvh, sc->view.bvh.wnodes != nullptr, rays, (long long)count, anyHit, hits,
                                  (const float4*)points, shadowDir, vis, counter, ctx->dErr, st);
  cudaFreeAsync(counter, st);
  if (e != cudaSuccess) return cudaFail(ctx, e, "ray query");
  return DDGI_OK;
}
}  // namespace

int ddgi_trace_rays(DdgiScene* sc, const DdgiRay* rays, uint64_t count, uint32_t flags, DdgiHit* hits, void* stream) {
  if (!sc) return DDGI_EINVAL;
  DdgiContext* ctx = sc->ctx;
  if (count && (!rays || !hits)) return fail(ctx, DDGI_EINVAL, "NULL rays or hits");
  if (flags & ~DDGI_RAY_ANY_HIT) return fail(ctx, DDGI_EINVAL, "unknown ray flags 0x%x", flags);
  if (((uintptr_t)rays | (uintptr_t)hits) & 15) return fail(ctx, DDGI_EINVAL, "rays and hits must be 16-byte aligned");
  return traceQuery(sc, rays, nullptr, count, (flags & DDGI_RAY_ANY_HIT) != 0, hits, f3(0.f, 0.f, 0.f), nullptr,
                    (cudaStream_t)stream);
}

int ddgi_shadow_mask(DdgiScene* sc, const DdgiFrame* frame, const float* points, uint64_t count, float* visibility,
                     void* stream) {
  if (!sc || !frame) return DDGI_EINVAL;
  DdgiContext* ctx = sc->ctx;
  if (count && (!points || !visibility)) return fail(ctx, DDGI_EINVAL, "NULL points or visibility");
  if ((uintptr_t)points & 15) return fail(ctx, DDGI_EINVAL, "points must be 16-byte aligned");
  // shadow.rgen:58: direction = -ubo.lightDir.xyz, as given (not normalised)
  const float3 dir = f3(-frame->lightDir[0], -frame->lightDir[1], -frame->lightDir[2]);
  return traceQuery(sc, nullptr, points, count, true, nullptr, dir, visibility, (cudaStream_t)stream);
}

int ddgi_query_irradiance(DdgiGrid* g, const DdgiFrame* frame, const DdgiSurfacePoint* points, uint64_t count,
                          float* ambient, void* stream) {
  if (!g || !frame) return fail(g ? g->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_query_irradiance");
  DdgiContext* ctx = g->ctx;
  if (count == 0) return DDGI_OK;
  if (!points || !ambient) return fail(ctx, DDGI_EINVAL, "NULL points or output");
  if (((uintptr_t)points | (uintptr_t)ambient) & 15) return fail(ctx, DDGI_EINVAL, "points and ambient must be 16-byte aligned");
  FrameGPU f{};
  int rc = frameToGPU(ctx, frame, f);
  if (rc) return rc;
  setFrameGrid(f, g->g);
  CK(launchQueryIrradiance(g->g, f, g->atlas[g->cur], points, (long long)count, (float4*)ambient,
                           (cudaStream_t)stream),
     "irradiance query");
  return DDGI_OK;
}

int ddgi_mirror_reflections(DdgiGrid* g, DdgiScene* sc, const DdgiFrame* frame, const DdgiMirrorPoint* points,
                            uint64_t count, float* out, void* stream) {
  if (!g || !sc || !frame) return fail(g ? g->ctx : sc ? sc->ctx : nullptr, DDGI_EINVAL, "NULL argument to ddgi_mirror_reflections");
  DdgiContext* ctx = g->ctx;
  if (sc->ctx != ctx) return fail(ctx, DDGI_EINVAL, "grid and scene belong to different contexts");
  if (count == 0) return DDGI_OK;
  if (!points || !out) return fail(ctx, DDGI_EINVAL, "NULL points or output");
  if (((uintptr_t)points | (uintptr_t)out) & 15) return fail(ctx, DDGI_EINVAL, "points and out must be 16-byte aligned");
  if (count > (1ull << 40)) return fail(ctx, DDGI_EINVAL, "count %llu too large", (unsigned long long)count);
  FrameGPU f{};
  int rc = frameToGPU(ctx, frame, f);
  if (rc) return rc;
  setFrameGrid(f, g->g);
  cudaStream_t st = (cudaStream_t)stream;
  // shadow rays in the light-space BVH of this frame's light when the grid traces its shadows there
  SceneGPU view = sc->view;
  if (g->tuning.shadowMode == 1) {
    rc = ensureShadowBvh(sc, frame->lightDir, st);
    if (rc) return rc;
    view = sc->view;
  } else {
    view.shadow = BvhRef{};
  }
  // rays, hits, shadow points, shadowed radiance, visibility; released once the stream has consumed them
  void* scratch = nullptr;
  unsigned long long* counter = nullptr;
  CK(cudaMallocAsync(&scratch, mirrorScratchBytes((long long)count), st), "mirror scratch");
  cudaError_t e = cudaMallocAsync(&counter, sizeof(unsigned long long), st);
  if (e == cudaSuccess)
    e = launchMirror(view, g->g, f, g->atlas[g->cur], points, (long long)count, (float4*)out, scratch, counter,
                     ctx->dErr, st);
  cudaFreeAsync(scratch, st);
  if (counter) cudaFreeAsync(counter, st);
  if (e != cudaSuccess) return cudaFail(ctx, e, "mirror reflections");
  return DDGI_OK;
}

// ---- raw kernels --------------------------------------------------------------------------------------
int ddgi_fibonacci_lattice(int numRays, const float rot[9], float* dirs, void* stream) {
  if (numRays <= 0 || numRays > (1 << 20) || !rot || !dirs) return DDGI_EINVAL;
  return launchLattice(numRays, rot, (float4*)dirs, (cudaStream_t)stream) == cudaSuccess ? DDGI_OK : DDGI_EDEVICE;
}

int ddgi_convolve_raw(const DdgiGridDesc* desc, const void* rayRadiance, const float* dirs, void* atlas,
                      int layerBegin, int layerEnd, uint32_t flags, void* stream) {
  if (validateGridDesc(nullptr, desc) != DDGI_OK || !rayRadiance || !dirs || !atlas) return DDGI_EINVAL;
  if (layerBegin < 0 || layerEnd > desc->dims[1] || layerBegin > layerEnd) return DDGI_EINVAL;
  GridGPU g = makeGridGPU(*desc);
  float* wt = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  // weights + sums in one scratch allocation, released after the stream has consumed it
  if (cudaMallocAsync(&wt, 4 * ((size_t)g.N * kOctTexels + kOctTexels), st) != cudaSuccess) return DDGI_ENOMEM;
  float* ws = wt + (size_t)g.N * kOctTexels;
  cudaError_t e = launchConvWeights(g.N, (const float4*)dirs, wt, ws, st);
  if (e == cudaSuccess)
    e = launchConvFp32(g, rayRadiance, wt, ws, atlas, layerBegin, layerEnd, desc->hysteresis, flags, st);
  cudaFreeAsync(wt, st);
  return e == cudaSuccess ? DDGI_OK : DDGI_EDEVICE;
}

int ddgi_convolve_tc_raw(DdgiContext* ctx, const DdgiGridDesc* desc, const void* radiance16, int elemFormat,
                         const float* dirs, void* atlas, int layerBegin, int layerEnd, uint32_t flags, void* stream) {
  if (!ctx) return DDGI_EINVAL;
  int rc = validateGridDesc(ctx, desc);
  if (rc) return rc;
  if (!radiance16 || !dirs || !atlas) return fail(ctx, DDGI_EINVAL, "NULL buffer to ddgi_convolve_tc_raw");
  if (elemFormat != DDGI_ELEM_F16 && elemFormat != DDGI_ELEM_BF16) return fail(ctx, DDGI_EINVAL, "elemFormat unknown");
  if (desc->raysPerProbe % 64) return fail(ctx, DDGI_EINVAL, "raysPerProbe must be a multiple of 64");
  if (layerBegin < 0 || layerEnd > desc->dims[1] || layerBegin > layerEnd) return fail(ctx, DDGI_EINVAL, "layer range");
  if (((uintptr_t)radiance16) & 15) return fail(ctx, DDGI_EINVAL, "radiance16 must be 16-byte aligned");
  GridGPU g = makeGridGPU(*desc);
  cudaStream_t st = (cudaStream_t)stream;
  void* scratch = nullptr;
  CK(cudaMallocAsync(&scratch, tcScratchBytes(g.N), st), "tensor-core weight scratch");
  cudaError_t e = launchConvTc(g, elemFormat, radiance16, g.X * g.Y * g.Z, (const float4*)dirs, scratch, atlas,
                               layerBegin, layerEnd, desc->hysteresis, flags, ctx->dErr, st, ctx->waits);
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return cudaFail(ctx, e, "tensor-core convolve");
  return DDGI_OK;
}

int ddgi_pack_rays16(const DdgiGridDesc* desc, const void* rayRadiance, void* radiance16, int elemFormat,
                     int layerBegin, int layerEnd, void* stream) {
  if (validateGridDesc(nullptr, desc) != DDGI_OK || !rayRadiance || !radiance16) return DDGI_EINVAL;
  if (elemFormat != DDGI_ELEM_F16 && elemFormat != DDGI_ELEM_BF16) return DDGI_EINVAL;
  if (layerBegin < 0 || layerEnd > desc->dims[1] || layerBegin > layerEnd) return DDGI_EINVAL;
  GridGPU g = makeGridGPU(*desc);
  return launchPackRays16(g, elemFormat, rayRadiance, radiance16, layerBegin, layerEnd,
                          g.X * g.Y * g.Z, (cudaStream_t)stream) == cudaSuccess ? DDGI_OK : DDGI_EDEVICE;
}

int ddgi_translate_raw(const DdgiGridDesc* desc, const void* atlasIn, void* atlasOut, int dx, int dz, void* stream) {
  if (validateGridDesc(nullptr, desc) != DDGI_OK || !atlasIn || !atlasOut || atlasIn == atlasOut) return DDGI_EINVAL;
  GridGPU g = makeGridGPU(*desc);
  int sx = dx > 0 ? 1 : (dx < 0 ? -1 : 0), sz = dz > 0 ? 1 : (dz < 0 ? -1 : 0);
  return launchTranslate(g, atlasIn, atlasOut, sx, sz, (cudaStream_t)stream) == cudaSuccess ? DDGI_OK : DDGI_EDEVICE;
}

}  // extern "C"
