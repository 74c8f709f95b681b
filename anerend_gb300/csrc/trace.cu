// Probe-ray generation, BVH traversal and hit shading: the work of irradiance_probe_update.rgen (ray
// generation, :48-111), .rchit (hit shading + shadow ray, :134-221) and .rmiss (sky / unshadowed,
// :17-21) on CUDA cores. The reference traverses with RT cores through traceRayEXT; here each thread
// runs a stack-based traversal (traverse.cuh) of the 8-wide BVH collapsed from the device-built LBVH, or
// of the binary LBVH itself, with a watertight ray/triangle test.
//
// Thread mapping: a warp traces 32 / warpProbes directions, consecutive in the grid's ray order, for each
// of warpProbes neighbouring probes of one layer. One persistent launch covers every grid of a batch;
// warps take their work from a shared queue.
#include "ddgi_common.cuh"
#include "kernels.h"
#include "traverse.cuh"
#include <type_traits>

#include <climits>

namespace ddgi {

// ---------------------------------------------------------------------------------------------------
// Fibonacci direction i of n before the rotation, normalised (rgen:35-46), in FP64.
DDGI_D void unitLatticeDir(int i, int n, double v[3]) {
  double theta = 2.0 * kPiRgen * (double)i / kGoldenRatio;
  double phi = acos(1.0 - 2.0 * ((double)i + 0.5) / (double)n);
  double sp = sin(phi);
  v[0] = cos(theta) * sp;
  v[1] = sin(theta) * sp;
  v[2] = cos(phi);
  double len = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= len;
  v[1] /= len;
  v[2] /= len;
}

// Golden-angle lattice (worldDirFromFibonacciIndex, rgen:35-46) rotated by mat3(randomRot) (rgen:87-88),
// in FP64. rot is column-major: out_r = sum_c rot[3c + r] * d_c.
__global__ void k_lattice(int n, Mat3 rot, float4* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[3];
  unitLatticeDir(i, n, v);
  double r[3];
  for (int row = 0; row < 3; ++row)
    r[row] = (double)rot.m[row] * v[0] + (double)rot.m[3 + row] * v[1] + (double)rot.m[6 + row] * v[2];
  out[i] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.0f);
}

// ---------------------------------------------------------------------------------------------------
// Previous-frame probe lookup: sampleSingleProbe / weightProbe / sampleProbe (pbr_light.glsl:168-363).
// Bilinear filtering is done in texel space in FP32 (the reference's REPEAT + LINEAR sampler, so texel
// indices wrap around the atlas; DDGI_GRID_EDGE_CLAMP clamps the probe index instead). The octahedral
// position of the normal, and so the texel offsets and bilinear weights inside a probe's block, are the same
// for the eight probes of a lookup: OctTap holds them, computed once per lookup.
struct OctTap {
  int dx0, dy0;              // offset of the 2 x 2 footprint inside a probe's 10 x 10 block (from texel (1, 1))
  float w00, w10, w01, w11;  // bilinear weights
};

DDGI_D OctTap octTap(float3 n) {
  const float2 o = octEncode(normalize3(n));
  const float ox = (o.x + 1.0f) * 0.5f * (float)(kOct - 1);
  const float oy = (o.y + 1.0f) * 0.5f * (float)(kOct - 1);
  const float fx0 = floorf(ox), fy0 = floorf(oy);
  const float fx = ox - fx0, fy = oy - fy0;
  OctTap t;
  t.dx0 = (int)fx0;
  t.dy0 = (int)fy0;
  t.w00 = (1.0f - fx) * (1.0f - fy);
  t.w10 = fx * (1.0f - fy);
  t.w01 = (1.0f - fx) * fy;
  t.w11 = fx * fy;
  return t;
}

// Square root of a non-negative blend of texels (sqrt.approx.f32: within 2^-23 relative, one instruction);
// the reference's shader sqrt is not correctly rounded either.
DDGI_D float sqrtBlend(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The texels x0 and x1 of an RGBA32F atlas row (x1 = x0 + 1, or its REPEAT / CLAMP_TO_EDGE replacement). For an
// even x0 both lie in the aligned 32-byte pair at x0 (the row length is even, so x1 = x0 + 1 there): one 32-byte
// load. An odd x0 is the second texel of its pair, and x1 comes from a second load made only by such lanes.
// Half the lanes thus issue one load per row instead of two. row: the row's first texel; the atlas base is
// 32-byte aligned.
DDGI_D void loadRowPair(const float4* row, int x0, int x1, float4& t0, float4& t1) {
  float4 p0, p1;
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(p0.x), "=f"(p0.y), "=f"(p0.z), "=f"(p0.w), "=f"(p1.x), "=f"(p1.y), "=f"(p1.z), "=f"(p1.w)
      : "l"(row + (x0 & ~1)));
  const bool odd = (x0 & 1) != 0;
  float4 q = p1;
  if (odd) q = __ldg(row + x1);
  t0 = odd ? p1 : p0;
  t1 = q;
}

// The same for an RGBA16F atlas: an aligned pair of 8-byte texels is one 16-byte load. row: the row's first
// texel; the atlas base is 16-byte aligned (the row length 10 X is even, so every row starts aligned).
DDGI_D float4 halfTexel(uint32_t lo, uint32_t hi) {
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&lo));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&hi));
  return make_float4(a.x, a.y, b.x, b.y);
}
DDGI_D void loadRowPairHalf(const uint2* row, int x0, int x1, float4& t0, float4& t1) {
  const uint4 p = __ldg(reinterpret_cast<const uint4*>(row + (x0 & ~1)));
  const bool odd = (x0 & 1) != 0;
  uint2 q = make_uint2(p.z, p.w);
  if (odd) q = __ldg(row + x1);
  t0 = odd ? halfTexel(p.z, p.w) : halfTexel(p.x, p.y);
  t1 = halfTexel(q.x, q.y);
}

// kPairs: 0 loads every texel alone; 1 loads texel pairs from an RGBA32F atlas (other formats alone); 2 also
// loads them from an RGBA16F atlas. The caller passes 1 or 2 only for an atlas aligned to a texel pair.
template <int kPairs = 0>
DDGI_D float3 sampleSingleProbe(const GridGPU& g, const void* atlas, int ix, int iy, int iz, const OctTap& tap) {
  if (g.options & DDGI_GRID_EDGE_CLAMP) {
    ix = min(max(ix, 0), g.X - 1);
    iy = min(max(iy, 0), g.Y - 1);
    iz = min(max(iz, 0), g.Z - 1);
  }
  int x0 = kProbePix * ix + 1 + tap.dx0;
  int y0 = kProbePix * g.Z * iy + kProbePix * iz + 1 + tap.dy0;
  int x1 = x0 + 1, y1 = y0 + 1;
  // The indices are never negative (ix, iy, iz >= 0; the octahedral offset is >= -1 and sx, sy >= 1) and
  // stay below W + 10 and H + 10 Z + 10 <= 3 H. REPEAT: conditional subtractions equal the modulo;
  // CLAMP_TO_EDGE: the last texel row / column.
  if (g.samplerClamp) {
    x0 = min(x0, g.atlasW - 1);
    x1 = min(x1, g.atlasW - 1);
    y0 = min(y0, g.atlasH - 1);
    y1 = min(y1, g.atlasH - 1);
  } else {
    if (x0 >= g.atlasW) x0 -= g.atlasW;
    if (x1 >= g.atlasW) x1 -= g.atlasW;
    if (y0 >= g.atlasH) y0 -= g.atlasH;
    if (y0 >= g.atlasH) y0 -= g.atlasH;
    if (y1 >= g.atlasH) y1 -= g.atlasH;
    if (y1 >= g.atlasH) y1 -= g.atlasH;
  }
  float4 t00, t10, t01, t11;
  if (kPairs >= 1 && g.atlasFmt == DDGI_FORMAT_RGBA32F) {
    const float4* a = reinterpret_cast<const float4*>(atlas);
    loadRowPair(a + (size_t)y0 * g.atlasW, x0, x1, t00, t10);
    loadRowPair(a + (size_t)y1 * g.atlasW, x0, x1, t01, t11);
  } else if (kPairs == 2) {
    const uint2* a = reinterpret_cast<const uint2*>(atlas);
    loadRowPairHalf(a + (size_t)y0 * g.atlasW, x0, x1, t00, t10);
    loadRowPairHalf(a + (size_t)y1 * g.atlasW, x0, x1, t01, t11);
  } else {
    t00 = loadTexel(atlas, g.atlasFmt, (size_t)y0 * g.atlasW + x0);
    t10 = loadTexel(atlas, g.atlasFmt, (size_t)y0 * g.atlasW + x1);
    t01 = loadTexel(atlas, g.atlasFmt, (size_t)y1 * g.atlasW + x0);
    t11 = loadTexel(atlas, g.atlasFmt, (size_t)y1 * g.atlasW + x1);
  }
  return xyz(t00) * tap.w00 + xyz(t10) * tap.w10 + xyz(t01) * tap.w01 + xyz(t11) * tap.w11;
}

DDGI_D void probeFrame(const GridGPU& g, const FrameGPU& f, float3& stepv, float3& offv) {
  if (f.flags & DDGI_UBO_BAKE_MODE_ON_FLAG) {
    // bake-tile grid (rgen:61-73, pbr_light.glsl:276-293)
    float tSize = (float)f.bakeTile[2];
    stepv = f3(tSize / (float)g.X, 1.0f, tSize / (float)g.Z);
    offv = f3((float)f.bakeTile[0] * tSize, g.originY, (float)f.bakeTile[1] * tSize);
  } else {
    // camera-relative grid, int() truncation of the camera probe index (rgen:75-83, pbr_light.glsl:294-308)
    const int camX = f.camIdx[0], camZ = f.camIdx[1];
    stepv = g.step;
    offv = f3((float)camX * g.step.x - g.step.x * (float)g.X / 2.0f, g.originY,
              (float)camZ * g.step.z - g.step.z * (float)g.Z / 2.0f);
  }
}

// kUnroll: how far the 8-probe loop is unrolled. The batch's shading kernel (80 registers, its records mostly
// missing L2) runs it unrolled by 2, measured 1 % faster there; the single record's stays fully unrolled (the
// rolled loop was 0.4 % slower on the single grid). Both sum the probes in the same order.
template <int kPairs = 0, int kUnroll = 8>
DDGI_D float3 sampleProbe(const GridGPU& g, const FrameGPU& f, const void* atlas, float3 wp, float3 n) {
  float3 stepv, offv;
  probeFrame(g, f, stepv, offv);
  int px = min(max((int)floorf((wp.x - offv.x) / stepv.x), 0), g.X - 1);
  int py = min(max((int)floorf((wp.y - offv.y) / stepv.y), 0), g.Y - 1);
  int pz = min(max((int)floorf((wp.z - offv.z) / stepv.z), 0), g.Z - 1);
  float3 base = f3((float)px, (float)py, (float)pz) * stepv + offv;
  float3 alpha = clamp3((wp - base) / stepv, 0.0f, 1.0f);
  // corner order of pbr_light.glsl:318-355
  const int corners[8][3] = {{0, 0, 0}, {1, 1, 1}, {1, 1, 0}, {1, 0, 0}, {0, 1, 1}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}};
  const OctTap tap = octTap(n);
  float sumW = 0.0f;
  float3 sumI = f3(0.f, 0.f, 0.f);
  auto probeTerm = [&](int ox, int oy, int oz) {
    float3 probePos = base + f3((float)ox, (float)oy, (float)oz) * stepv;
    float3 tri = f3(ox ? alpha.x : 1.0f - alpha.x, oy ? alpha.y : 1.0f - alpha.y, oz ? alpha.z : 1.0f - alpha.z);
    float3 dirToProbe = normalize3(probePos - wp);
    float c = fmaxf(0.0001f, (dot3(dirToProbe, n) + 1.0f) * 0.5f);
    float w = c * c + 0.2f;
    w = fmaxf(0.000001f, w);
    if (w < 0.2f) w *= w * w * (1.0f / (0.2f * 0.2f));
    w *= tri.x * tri.y * tri.z;
    float3 irr = sampleSingleProbe<kPairs>(g, atlas, px + ox, py + oy, pz + oz, tap);
    irr = f3(sqrtBlend(irr.x), sqrtBlend(irr.y), sqrtBlend(irr.z));
    sumI += irr * w;
    sumW += w;
  };
  if constexpr (kUnroll == 8) {
#pragma unroll
    for (int k = 0; k < 8; ++k) probeTerm(corners[k][0], corners[k][1], corners[k][2]);
  } else {  // the same corners, as bit k of one constant per axis (no local array in a rolled loop)
#pragma unroll kUnroll
    for (int k = 0; k < 8; ++k) probeTerm((0x8E >> k) & 1, (0x36 >> k) & 1, (0xD2 >> k) & 1);
  }
  float3 net = sumI * (1.0f / sumW);
  net = net * net;
  return net * 0.5f * kPiSampleProbe;
}

// calcIndirectDiffuseLight (pbr_light.glsl:365-388)
template <int kPairs = 0, int kUnroll = 8>
DDGI_D float3 calcIndirectDiffuse(const GridGPU& g, const FrameGPU& f, const void* atlas, float3 n,
                                  float3 albedo, float metallic, float roughness, float3 wp, float3 viewPos) {
  float3 V = normalize3(viewPos - wp);
  float3 F0 = mixF0(albedo, metallic);
  float3 kS = fresnelSchlickRoughness(fmaxf(dot3(n, V), 0.0f), F0, roughness * roughness);
  float3 kD = (f3(1.f, 1.f, 1.f) - kS) * (1.0f - metallic);
  float3 irr = sampleProbe<kPairs, kUnroll>(g, f, atlas, wp, n);
  return kD * (irr * albedo);
}

// ---------------------------------------------------------------------------------------------------
// Wavefront trace of one launch (every item of a batch, or one grid): four kernels in stream order, after
// the lattice and seed-map kernels.
//   k_trace_closest   persistent closest-hit traversal, seeded with a candidate hit; writes one hit record
//                     per ray slot
//   k_shade           one thread per ray slot: hit reconstruction, shading, probe lookup, outputs, hit memo;
//                     appends a shadow ray (origin + slot id) to a list for each hit whose lit and shadowed
//                     radiance differ
//   k_trace_shadow    persistent any-hit traversal over the list, seeded with a candidate occluder; flags
//                     the records of shadowed rays
//   k_shadow_resolve  one thread per shadow record: the occluder memo and the shadowed radiance of the
//                     flagged rays
// Splitting keeps each kernel small (registers, instruction cache), lets the traversal kernels refill
// idle lanes with new rays instead of waiting for a warp's longest ray, and keeps scattered per-ray output
// writes out of the traversal loops.
//
// Ray slots: item i owns slots [32 warpBegin_i, 32 (warpBegin_i + traceWarps_i)); slot 32 w + l of an item
// is lane l of its warp w. Warp w traces D = 32 / warpProbes directions, consecutive in the grid's ray
// order, for each of warpProbes neighbouring probes of one layer; with the octahedral Morton order the D
// directions are neighbours on the sphere, so rays fetched together share traversal paths.
#ifndef DDGI_TRACE_MIN_BLOCKS
#define DDGI_TRACE_MIN_BLOCKS 8
#endif
// The light-space shadow traversal (exact +z box test) fits 48 registers: 10 resident blocks per SM, and
// its launch scales the traversal grid by 10 / 8 (measured 1 % faster per probe update than 8 blocks).
constexpr int kShadowLightBlocks = 10;

struct RaySlot {
  int px, pz, layer, j;
  bool valid;
};

DDGI_D RaySlot raySlot(const GridGPU& g, const FrameGPU& f, const int* __restrict__ order, uint32_t warp,
                       int lane) {
  RaySlot r;
  r.valid = false;
  const uint32_t lgN = (uint32_t)(__ffs(g.N) - 1), lgWP = (uint32_t)(__ffs(g.warpProbes) - 1), lgD = 5u - lgWP;
  const uint32_t lgChunks = lgN - lgD;  // N / D direction chunks per probe group
  const uint32_t rest = warp >> lgChunks;
  const int dc = (int)(warp & ((1u << lgChunks) - 1u));
  const uint32_t lq = divFast(rest, (uint32_t)g.probeGroups, g.magicPG);
  const int pg = (int)(rest - lq * (uint32_t)g.probeGroups);
  r.layer = f.layerBegin + (int)lq;
  if (r.layer >= f.layerEnd) return r;
  const int p = (pg << lgWP) + (lane >> lgD);
  if (p >= g.X * g.Z) return r;
  r.j = __ldg(&order[(dc << lgD) + (lane & ((1 << lgD) - 1))]);
  const uint32_t pz = divFast((uint32_t)p, (uint32_t)g.X, g.magicX);
  r.px = p - (int)pz * g.X;
  r.pz = (int)pz;
  r.valid = true;
  return r;
}

// A ray by its natural id: the item-local index ((layer - layerBegin) * PG * WP + q) * N + j over the layer's
// probes q (padded to whole probe groups, as the trace slots are) and the directions j. Consecutive ids are
// consecutive directions of one probe, so the per-ray outputs indexed by (probe, direction) are written
// coalesced by the shading kernels, which walk rays in this order. `slot` is the ray's item-local trace slot
// (raySlot's inverse): warp ((layer - layerBegin) * PG + q / WP) * (N / D) + pos / D, lane (q % WP) * D + pos % D,
// with pos the direction's position in the trace order (order[N + j]). N, WP and D are powers of two.
struct NaturalRay {
  RaySlot rs;
  uint32_t slot;
};

DDGI_D NaturalRay naturalRay(const GridGPU& g, const FrameGPU& f, const int* __restrict__ order, uint32_t local) {
  NaturalRay r;
  r.rs.valid = false;
  r.slot = 0;
  const uint32_t lgN = (uint32_t)(__ffs(g.N) - 1), lgWP = (uint32_t)(__ffs(g.warpProbes) - 1), lgD = 5u - lgWP;
  const uint32_t XZ = (uint32_t)(g.X * g.Z);
  const uint32_t PG = (uint32_t)g.probeGroups;
  const uint32_t perLayer = PG << (lgWP + lgN);
  const uint32_t lq = divFast(local >> (lgWP + lgN), PG, g.magicPG);
  const uint32_t rem = local - lq * perLayer;
  const uint32_t q = rem >> lgN, j = rem & ((uint32_t)g.N - 1u);
  const int layer = f.layerBegin + (int)lq;
  if (layer >= f.layerEnd || q >= XZ) return r;
  const uint32_t pos = (uint32_t)__ldg(&order[g.N + (int)j]);
  const uint32_t pg = q >> lgWP, qq = q & ((uint32_t)g.warpProbes - 1u);
  r.slot = (((lq * PG + pg) << (lgN - lgD)) + (pos >> lgD)) * 32u + (qq << lgD) + (pos & ((1u << lgD) - 1u));
  r.rs.layer = layer;
  r.rs.j = (int)j;
  const uint32_t pz = divFast(q, (uint32_t)g.X, g.magicX);
  r.rs.px = (int)(q - pz * (uint32_t)g.X);
  r.rs.pz = (int)pz;
  r.rs.valid = true;
  return r;
}

DDGI_D int findItem(const TraceItem* __restrict__ items, int numItems, long long warp) {
  int lo = 0, hi = numItems - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (items[mid].warpBegin <= warp) lo = mid; else hi = mid - 1;
  }
  return lo;
}


// Where a trace launch's records come from: the first argument of the wavefront kernels, passed by value
// (__grid_constant__). ItemsOne carries a single-item launch's record itself, so the kernels' per-ray record
// reads become constant-bank reads at fixed offsets; ItemsGlobal points at the table in global memory (a
// by-value table of many records, indexed at run time, measured no faster than the L1-resident table).
// at(warp) is the record that owns ray-slot warp `warp`.
// For a launch of at most kParamItems records the first warps of the records also travel in the parameters, so
// the per-ray search for a ray's record reads the constant bank (uniform over a warp) instead of the records'
// scattered warpBegin fields.
struct ItemsGlobal {
  const TraceItem* items;
  int n;
  int inParams;  // begins[] holds the n records' first warps
  long long begins[kParamItems];
  DDGI_D const TraceItem& at(long long warp) const {
    if (!inParams) return items[findItem(items, n, warp)];
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (begins[mid] <= warp) lo = mid; else hi = mid - 1;
    }
    return items[lo];
  }
};
struct ItemsOne {
  TraceItem it;
  DDGI_D const TraceItem& at(long long) const { return it; }
};

// ray generation (rgen:51-88)
DDGI_D float3 probeOrigin(const GridGPU& g, const FrameGPU& f, const RaySlot& rs) {
  float3 stepv, offv;
  probeFrame(g, f, stepv, offv);
  return f3((float)rs.px, (float)rs.layer, (float)rs.pz) * stepv + offv;
}

DDGI_D size_t rayIndex(const GridGPU& g, const RaySlot& rs) {
  const int lgBw = __ffs(g.bw) - 1;  // bw is a power of two
  const int rx = rs.px * g.bw + (rs.j & (g.bw - 1));
  const int ry = (rs.layer * g.Z + rs.pz) * g.bh + (rs.j >> lgBw);
  return (size_t)ry * g.rayW + rx;
}

// operand of the tensor-core convolution: planar 16-bit radiance, row c * pTotal + probe
DDGI_D void storeRad16(const GridGPU& g, const RaySlot& rs, float3 L) {
  const size_t base = ((size_t)(rs.layer * g.Z + rs.pz) * g.X + rs.px) * g.N + rs.j;
  const size_t plane = (size_t)g.pTotal * g.N;
  uint16_t* o = (uint16_t*)g.rad16;
  const float c[3] = {L.x, L.y, L.z};
#pragma unroll
  for (int k = 0; k < 3; ++k)
    o[base + k * plane] = g.rad16Fmt == 0 ? __half_as_ushort(__float2half_rn(c[k]))
                                          : __bfloat16_as_ushort(__float2bfloat16_rn(c[k]));
}

constexpr int kNoRay = -2;  // hit record of a slot without a ray (past the grid's probes or layers)

// Traversal state of one lane: the binary or the 8-wide stack machine.
template <bool kWide> struct TravOf;
template <> struct TravOf<false> { using T = BinTrav; };
template <> struct TravOf<true> { using T = WideTrav; };

template <bool kWide, bool kAnyHit>
DDGI_D bool travInit(const BvhRef& b, const WRay& r, typename TravOf<kWide>::T& s, HitInfo& hit) {
  if constexpr (kWide) return wideInit<kAnyHit>(b, r, kTMax, s, hit);
  else return binInit<kAnyHit>(b, r, kTMin, kTMax, s, hit);
}
template <bool kWide, bool kAnyHit, bool kPlusZ = false, bool kNodeScale = false>
DDGI_D bool travStep(const BvhRef& b, const WRay& r, typename TravOf<kWide>::T& s, HitInfo& hit, uint32_t* err) {
  if constexpr (kWide) return wideStep<kAnyHit, kPlusZ, kNodeScale>(b, r, kTMin, s, hit, err);
  else return binStep<kAnyHit>(b, r, kTMin, s, hit, err);
}

// Closest hits of every ray slot (rgen:90-106). Each lane owns one ray; once at least refillLanes lanes of
// a warp are idle the warp takes that many new slots from the queue (counters[0]) with one atomic.
template <bool kWide, class Src>
__global__ void __launch_bounds__(kTraceThreads, DDGI_TRACE_MIN_BLOCKS)
    k_trace_closest(const __grid_constant__ Src src, long long totalRays, unsigned long long* __restrict__ counters,
                    int refillLanes, float4* __restrict__ hits, uint32_t* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  long long id = -1;
  bool drained = false;
  // the lane's BVH: a single record's launch keeps a register copy; a launch over many records keeps a pointer
  // to the lane's record's BVH instead, whose fields the steps re-read from L1, which frees nine registers of
  // the 64-register traversal (measured 1.4 % faster on the 64-grid batch). Such a launch also forms the
  // quantized nodes' scale from the node (kNodeScale): three registers fewer per ray take away the last 24
  // bytes of spills (1.5 % faster on that batch); the single record's kernel, which does not spill, measured
  // 1.2 % slower with it and keeps the ray's scale.
  constexpr bool kManyItems = !std::is_same<Src, ItemsOne>::value;
  BvhRef bvh;
  const BvhRef* bvhp = nullptr;
  WRay ray;
  HitInfo hit;
  typename TravOf<kWide>::T st;
  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, id < 0);
    if (drained && idle == 0xffffffffu) break;
    if (!drained && __popc(idle) >= refillLanes) {
      const int need = __popc(idle);
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&counters[0], (unsigned long long)need);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((long long)base + need >= totalRays) drained = true;
      const long long cand = (long long)base + __popc(idle & below);
      if (id < 0 && cand < totalRays) {
        const long long warp = cand >> 5;
        const TraceItem& T = src.at(warp);
        const RaySlot rs = raySlot(T.g, T.f, T.order, (uint32_t)(warp - T.warpBegin), (int)(cand & 31));
        if (!rs.valid) {
          hits[cand] = make_float4(__int_as_float(kNoRay), 0.f, 0.f, 0.f);
        } else {
          if (std::is_same<Src, ItemsOne>::value && T.rayDirs) {  // a single record's direction records
            RayDirRec p;
            p.a = __ldg(&T.rayDirs[2 * rs.j]);
            p.b = __ldg(&T.rayDirs[2 * rs.j + 1]);
            ray = makeRayPacked(probeOrigin(T.g, T.f, rs), p);
          } else {
            ray = makeRay(probeOrigin(T.g, T.f, rs), xyz(__ldg(&T.lattice[rs.j])));
          }
          bvh = T.s.bvh;
          bvhp = &T.s.bvh;
          if (travInit<kWide, false>(bvh, ray, st, hit)) {
            hits[cand] = make_float4(__int_as_float(hit.leaf), hit.t, hit.b1, hit.b2);
          } else {
            id = cand;
            if (T.seedOn) {  // the seed candidate: the last trace's hit in the nearest direction
              const size_t p = ((size_t)rs.layer * T.g.Z + rs.pz) * T.g.X + rs.px;
              const int c = __ldg(&T.hitMemo[p * T.g.N + __ldg(&T.seedDir[rs.j])]);
              if ((unsigned)c < (unsigned)bvh.numTris) testTri<false>(bvh, ray, c, kTMin, hit);
            }
          }
        }
      }
    }
    if (id >= 0 && travStep<kWide, false, false, kManyItems>(kManyItems ? *bvhp : bvh, ray, st, hit, err)) {
      hits[id] = make_float4(__int_as_float(hit.leaf), hit.t, hit.b1, hit.b2);
      id = -1;
    }
  }
}

// Surface at a hit: world position, shading normal, colour and material of triangle record `leaf` at
// barycentric weights (b1, b2) of its 2nd and 3rd vertices.
struct HitSurface {
  float3 pos, normal, color, emissive;  // emissive = emissive.rgb * emissive.w
  float metallic, roughness;
};

// Hit reconstruction (irradiance_probe_update.rchit:137-187; getSurfaceDataFromMat bindless.glsl:181-237
// without textures). kMirrorNormal: the normal through mat3(ObjectToWorld) (mirror_reflections.rchit:73)
// instead of normal * WorldToObject (irradiance_probe_update.rchit:72).
template <bool kMirrorNormal>
DDGI_D HitSurface reconstructHit(const SceneGPU& s, int leaf, float b1, float b2) {
  const int inst = __float_as_int(__ldg(&s.bvh.tris[3 * leaf + 1].w));
  const int prim = __float_as_int(__ldg(&s.bvh.tris[3 * leaf + 2].w));
  // the 96-byte instance record as six 16-byte loads (its buffer is 256-byte aligned): o2w in q0..q2,
  // w2oLin in q3, q4, q5.x, then mesh and material
  const float4* iq = reinterpret_cast<const float4*>(s.instances + inst);
  const float4 q0 = __ldg(iq), q1 = __ldg(iq + 1), q2 = __ldg(iq + 2), q3 = __ldg(iq + 3), q4 = __ldg(iq + 4),
               q5 = __ldg(iq + 5);
  const float m[12] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
  const uint32_t meshId = __float_as_uint(q5.y), materialId = __float_as_uint(q5.z);
  // vertexOffset and indexOffset of the mesh record, one 8-byte load
  const uint2 offs = __ldg(reinterpret_cast<const uint2*>(&s.meshes[meshId].vertexOffset));
  const uint32_t ib = offs.y + 3u * (uint32_t)prim;
  const DdgiPackedVertex* vb = s.vertices + offs.x;
  const DdgiPackedVertex& v0 = vb[__ldg(&s.indices[ib])];
  const DdgiPackedVertex& v1 = vb[__ldg(&s.indices[ib + 1])];
  const DdgiPackedVertex& v2 = vb[__ldg(&s.indices[ib + 2])];
  const float b0 = 1.0f - b1 - b2;
  const float4 a0 = __ldg((const float4*)v0.d0), a1 = __ldg((const float4*)v1.d0), a2 = __ldg((const float4*)v2.d0);
  const float4 c0 = __ldg((const float4*)v0.d1), c1 = __ldg((const float4*)v1.d1), c2 = __ldg((const float4*)v2.d1);
  const float4 e0 = __ldg((const float4*)v0.d2), e1 = __ldg((const float4*)v1.d2), e2 = __ldg((const float4*)v2.d2);
  HitSurface h;
  const float3 posObj = xyz(a0) * b0 + xyz(a1) * b1 + xyz(a2) * b2;
  h.pos = f3(m[0] * posObj.x + m[1] * posObj.y + m[2] * posObj.z + m[3],
             m[4] * posObj.x + m[5] * posObj.y + m[6] * posObj.z + m[7],
             m[8] * posObj.x + m[9] * posObj.y + m[10] * posObj.z + m[11]);
  const DdgiMaterialInfo& mat = s.materials[materialId];
  float3 nObj = f3(c0.z, c0.w, e0.x) * b0 + f3(c1.z, c1.w, e1.x) * b1 + f3(c2.z, c2.w, e2.x) * b2;
  nObj = normalize3(nObj);
  if (kMirrorNormal) {
    h.normal = normalize3(f3(m[0] * nObj.x + m[1] * nObj.y + m[2] * nObj.z, m[4] * nObj.x + m[5] * nObj.y + m[6] * nObj.z,
                             m[8] * nObj.x + m[9] * nObj.y + m[10] * nObj.z));
  } else {
    const float wi[9] = {q3.x, q3.y, q3.z, q3.w, q4.x, q4.y, q4.z, q4.w, q5.x};  // normal * WorldToObject
    h.normal = normalize3(f3(nObj.x * wi[0] + nObj.y * wi[3] + nObj.z * wi[6], nObj.x * wi[1] + nObj.y * wi[4] + nObj.z * wi[7],
                             nObj.x * wi[2] + nObj.y * wi[5] + nObj.z * wi[8]));
  }
  // the base colour factor wins when its sum exceeds 0.1; otherwise the interpolated vertex colour in
  // linear space (rchit:183-184, bindless.glsl:199-203)
  const float4 bcf = __ldg((const float4*)mat.baseColFac);
  if (bcf.x + bcf.y + bcf.z > 0.1f) {
    h.color = xyz(bcf);
  } else {
    const float3 vcol = f3(a0.w, c0.x, c0.y) * b0 + f3(a1.w, c1.x, c1.y) * b1 + f3(a2.w, c2.x, c2.y) * b2;
    h.color = toLinear(vcol);
  }
  const float4 mr = __ldg((const float4*)mat.metRough);
  const float4 em = __ldg((const float4*)mat.emissive);
  h.metallic = mr.x;
  h.roughness = mr.y;
  h.emissive = xyz(em) * em.w;
  return h;
}

// Interpolated vertex colour in linear space at record `leaf` (rchit:183-184, bindless.glsl:199-203), through
// the index and vertex records: the shading's fallback when the material's base colour factor is dark.
DDGI_D float3 vertexColour(const SceneGPU& s, int leaf, float b0, float b1, float b2) {
  const int inst = __float_as_int(__ldg(&s.bvh.tris[3 * leaf + 1].w));
  const int prim = __float_as_int(__ldg(&s.bvh.tris[3 * leaf + 2].w));
  const DdgiMeshInfo& mesh = s.meshes[s.instances[inst].mesh];
  const uint32_t ib = mesh.indexOffset + 3u * (uint32_t)prim;
  const DdgiPackedVertex* vb = s.vertices + mesh.vertexOffset;
  const DdgiPackedVertex& v0 = vb[__ldg(&s.indices[ib])];
  const DdgiPackedVertex& v1 = vb[__ldg(&s.indices[ib + 1])];
  const DdgiPackedVertex& v2 = vb[__ldg(&s.indices[ib + 2])];
  const float3 c = f3(v0.d0[3], v0.d1[0], v0.d1[1]) * b0 + f3(v1.d0[3], v1.d1[0], v1.d1[1]) * b1 +
                   f3(v2.d0[3], v2.d1[0], v2.d1[1]) * b2;
  return toLinear(c);
}

// Surface at a hit of the probe update from the BVH record (world vertices) and its shading record
// (SceneGPU::shade): position = the interpolated world vertices, normal = normalize(interpolated
// vertex normal * WorldToObject) - the reference's ObjectToWorld * interpolated object position and
// normalize(normalize(interpolated normal) * WorldToObject) (rchit:137-187), in another order of the same
// linear operations. Three dependent loads per hit (record, shading record, material) instead of five
// levels through the instance, mesh, index and vertex records.
DDGI_D HitSurface shadeSurface(const SceneGPU& s, int leaf, float b1, float b2, float4& r0) {
  r0 = __ldg(&s.bvh.tris[3 * leaf]);
  const float4 r1 = __ldg(&s.bvh.tris[3 * leaf + 1]), r2 = __ldg(&s.bvh.tris[3 * leaf + 2]);
  const float4 m0 = __ldg(&s.shade[3 * leaf]), m1 = __ldg(&s.shade[3 * leaf + 1]), m2 = __ldg(&s.shade[3 * leaf + 2]);
  const float b0 = 1.0f - b1 - b2;
  HitSurface h;
  h.pos = xyz(r0) * b0 + xyz(r1) * b1 + xyz(r2) * b2;
  h.normal = normalize3(xyz(m0) * b0 + xyz(m1) * b1 + xyz(m2) * b2);
  const DdgiMaterialInfo& mat = s.materials[__float_as_uint(m0.w)];
  const float4 bcf = __ldg((const float4*)mat.baseColFac);
  h.color = bcf.x + bcf.y + bcf.z > 0.1f ? xyz(bcf) : vertexColour(s, leaf, b0, b1, b2);
  const float4 mr = __ldg((const float4*)mat.metRough);
  const float4 em = __ldg((const float4*)mat.emissive);
  h.metallic = mr.x;
  h.roughness = mr.y;
  h.emissive = xyz(em) * em.w;
  return h;
}

// Shading records of the scene BVH's records (SceneGPU::shade), one thread per record.
__global__ void k_shading_records(SceneGPU s, uint64_t numIndices, uint64_t numVerts, float4* __restrict__ out,
                                  uint32_t* __restrict__ err) {
  const int rec = blockIdx.x * blockDim.x + threadIdx.x;
  if (rec >= s.bvh.numTris) return;
  const int inst = __float_as_int(s.bvh.tris[3 * rec + 1].w);
  const int prim = __float_as_int(s.bvh.tris[3 * rec + 2].w);
  const InstanceGPU& in = s.instances[inst];
  const DdgiMeshInfo& mesh = s.meshes[in.mesh];
  const float* wi = in.w2oLin;
  for (int k = 0; k < 3; ++k) {
    const uint64_t ii = (uint64_t)mesh.indexOffset + 3ull * (uint64_t)prim + k;
    uint64_t vv = ii < numIndices ? (uint64_t)mesh.vertexOffset + s.indices[ii] : numVerts;
    if (vv >= numVerts) {
      atomicOr(err, DDGI_DEVERR_BOUNDS);
      out[3 * rec + k] = make_float4(0.f, 0.f, 0.f, __uint_as_float(in.material));
      continue;
    }
    const DdgiPackedVertex& v = s.vertices[vv];
    const float nx = v.d1[2], ny = v.d1[3], nz = v.d2[0];
    out[3 * rec + k] = make_float4(nx * wi[0] + ny * wi[3] + nz * wi[6], nx * wi[1] + ny * wi[4] + nz * wi[7],
                                   nx * wi[2] + ny * wi[5] + nz * wi[8], __uint_as_float(in.material));
  }
}

cudaError_t launchShadingRecords(const SceneGPU& s, uint64_t numIndices, uint64_t numVerts, float4* out,
                                 uint32_t* err, cudaStream_t stream) {
  if (s.bvh.numTris <= 0) return cudaSuccess;
  k_shading_records<<<(s.bvh.numTris + 255) / 256, 256, 0, stream>>>(s, numIndices, numVerts, out, err);
  return cudaGetLastError();
}

// Hit shading (rchit:134-221) and misses (rmiss:17-21), one thread per ray in natural order (consecutive
// threads = consecutive directions of one probe, so the ray image, the 16-bit radiance and the hit memo are
// written coalesced; each thread reads its ray's hit record from the trace slot naturalRay gives). A hit's
// radiance is computed both lit and shadowed, in the reference's order of operations; the lit value is stored
// and the shadow ray is appended to shadowList (counters[1]) as two records: its origin and natural ray id,
// then the shadowed value and the candidate occluder.
// 4 resident blocks per SM (64 registers) for a single record; 3 (up to 85 registers, half the spills) for a
// batch, whose shading waits on DRAM for records and atlases that do not stay in L2 (measured 0.35 % faster
// there, 0.7 % slower on the single grid).
template <class Src>
__global__ void __launch_bounds__(256, std::is_same<Src, ItemsOne>::value ? 4 : 3) k_shade(const __grid_constant__ Src src, long long totalRays,
                                               const float4* __restrict__ hits, float4* __restrict__ shadowList,
                                               unsigned long long* __restrict__ counters) {
  constexpr int kProbeUnroll = std::is_same<Src, ItemsOne>::value ? 8 : 2;
  // texel pairs from RGBA16F atlases too in the single record's kernel (1.2 % faster per update on an RGBA16F
  // grid); the batch's kernel keeps them to RGBA32F atlases (the RGBA16F path's registers cost it 0.25 %)
  constexpr int kPairMode = std::is_same<Src, ItemsOne>::value ? 2 : 1;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < totalRays;
       id += (long long)gridDim.x * blockDim.x) {
    bool cast = false;
    float3 so = f3(0.f, 0.f, 0.f), Ls = f3(0.f, 0.f, 0.f);
    int occ = -1;
    const long long warp = id >> 5;  // natural ids share the items' slot ranges
    const TraceItem& T = src.at(warp);
    const NaturalRay nr = naturalRay(T.g, T.f, T.order, (uint32_t)(id - 32 * T.warpBegin));
    if (nr.rs.valid) {
      const SceneGPU& s = T.s;
      const GridGPU& g = T.g;
      const FrameGPU& f = T.f;
      const RaySlot& rs = nr.rs;
      const float4 hr = hits[32 * T.warpBegin + nr.slot];
      const int leaf = __float_as_int(hr.x);
      const float3 origin = probeOrigin(g, f, rs);
      const float3 dir = xyz(__ldg(&T.lattice[rs.j]));
      const size_t pj = (((size_t)rs.layer * g.Z + rs.pz) * g.X + rs.px) * g.N;
      if (T.hitMemo)  // this trace's closest-hit record, the next trace's seed candidate
        T.hitMemo[pj + rs.j] = leaf >= 0 ? leaf : -1;
      float3 L;
      int hitCode = -1;
      if (leaf < 0) {
        L = f.skyLinear;  // rmiss:20
      } else {
        float4 r0;
        const HitSurface h = shadeSurface(s, leaf, hr.z, hr.w, r0);
        const float3 pos = h.pos;
        // shadow ray origin toward the sun (rchit:155-176): the light's sheared space when built
        if (s.shadow.tris != nullptr) {
          const float pk[3] = {pos.x, pos.y, pos.z};
          const float pz = pk[s.shearK[2]];
          so = f3(pk[s.shearK[0]] - s.shearS[0] * pz, pk[s.shearK[1]] - s.shearS[1] * pz, s.shearS[2] * pz);
        } else {
          so = pos;
        }
        // lit: L = calcLight; shadowed: L = 0; then += indirect, += emissive (rchit:195-214)
        L = calcLightDirectional(h.normal, h.color, h.metallic, h.roughness, pos, origin, f.lightDir, f.sunIntensity);
        if (f.flags & DDGI_UBO_DDGI_MULTI_FLAG) {
          const float3 ind =
              T.atlasPairs ? calcIndirectDiffuse<kPairMode, kProbeUnroll>(g, f, T.atlasPrev, h.normal, h.color, h.metallic, h.roughness, pos, origin)
                           : calcIndirectDiffuse<0, kProbeUnroll>(g, f, T.atlasPrev, h.normal, h.color, h.metallic, h.roughness, pos, origin);
          L += ind;
          Ls += ind;
        }
        L += h.emissive;
        Ls += h.emissive;
        // The shadow ray only picks between L and Ls. When they have the same bits (a surface facing away
        // from the sun, N.L <= 0, makes calcLight exactly 0) its outcome cannot change the radiance, so it
        // is cast only when the values differ or the caller records per-ray hit codes (their shadow bit).
        cast = T.rayHit != nullptr || __float_as_uint(L.x) != __float_as_uint(Ls.x) ||
               __float_as_uint(L.y) != __float_as_uint(Ls.y) || __float_as_uint(L.z) != __float_as_uint(Ls.z);
        // the shadow ray's candidate occluder: the last trace's occluder in the nearest previous direction
        if (cast && T.seedOn) occ = __ldg(&T.occMemo[pj + __ldg(&T.seedDir[rs.j])]);
        hitCode = __float_as_int(r0.w) * 2;
      }
      // stores (rgen:108-109)
      const size_t idx = rayIndex(g, rs);
      storeTexel(T.rayRad, g.rayFmt, idx, make_float4(L.x, L.y, L.z, 1.0f));
      if (T.rayDir) storeTexel(T.rayDir, g.rayFmt, idx, make_float4(dir.x, dir.y, dir.z, 1.0f));
      if (T.rayHit) T.rayHit[idx] = hitCode;
      if (g.rad16) storeRad16(g, rs, L);
    }
    // append the shadow rays of this warp's rays with one atomic
    const unsigned act = __activemask();
    const unsigned want = __ballot_sync(act, cast);
    if (want) {
      const int leader = __ffs(act) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&counters[1], (unsigned long long)__popc(want));
      base = __shfl_sync(act, base, leader);
      if (cast) {
        const unsigned long long k = base + __popc(want & below);
        shadowList[2 * k] = make_float4(so.x, so.y, so.z, __uint_as_float((uint32_t)id));
        shadowList[2 * k + 1] = make_float4(Ls.x, Ls.y, Ls.z, __int_as_float(occ));
      }
    }
  }
}

// Shadow rays (rchit:155-176): any hit in [0.1, 50] toward the sun; a shadowed ray gets the top bit of its
// shadow record's ray id set and its occluder in the second record, and k_shadow_resolve gives it the
// shadowed radiance. Keeping the output writes out of this kernel keeps its finishing lanes (a few per warp at
// a time) to two stores.
// kLightSpace: every item's shadow rays run in its light-space BVH along +z (shadowMode 1).
template <bool kWide, bool kLightSpace, class Src>
__global__ void __launch_bounds__(kTraceThreads, kLightSpace ? kShadowLightBlocks : DDGI_TRACE_MIN_BLOCKS)
    k_trace_shadow(const __grid_constant__ Src src, float4* __restrict__ shadowList,
                   unsigned long long* __restrict__ counters, int refillLanes, uint32_t* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const long long total = (long long)counters[1];
  long long id = -1;  // shadow record index of this lane's ray
  uint32_t rayId = 0;  // its natural ray id
  bool drained = total == 0;
  BvhRef bvh;
  // as in k_trace_closest: a launch over many records steps through a pointer and forms the node scale
  constexpr bool kManyItems = !std::is_same<Src, ItemsOne>::value;
  const BvhRef* bvhp = nullptr;
  WRay ray;
  HitInfo hit;
  typename TravOf<kWide>::T st;
  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, id < 0);
    if (drained && idle == 0xffffffffu) break;
    bool finished = false;
    if (!drained && __popc(idle) >= refillLanes) {
      const int need = __popc(idle);
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&counters[2], (unsigned long long)need);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((long long)base + need >= total) drained = true;
      const long long k = (long long)base + __popc(idle & below);
      if (id < 0 && k < total) {
        const float4 rec = shadowList[2 * k];
        id = k;
        rayId = __float_as_uint(rec.w);
        const TraceItem& T = src.at((long long)(rayId >> 5));
        bvh = kLightSpace ? T.s.shadow : T.s.bvh;
        bvhp = kLightSpace ? &T.s.shadow : &T.s.bvh;
        ray = makeRay(xyz(rec), kLightSpace ? f3(0.f, 0.f, 1.f) : normalize3(-T.f.lightDir));
        finished = travInit<kWide, true>(bvh, ray, st, hit);
        if (!finished) {  // the candidate occluder k_shade parked: if it is hit, the ray is shadowed
          const int c = __float_as_int(shadowList[2 * k + 1].w);
          if ((unsigned)c < (unsigned)bvh.numTris) finished = testTri<true>(bvh, ray, c, kTMin, hit);
        }
      }
    }
    if (id >= 0 && !finished)
      finished = travStep<kWide, true, kLightSpace, kManyItems>(kManyItems ? *bvhp : bvh, ray, st, hit, err);
    if (id >= 0 && finished) {
      if (hit.leaf >= 0) {
        reinterpret_cast<uint32_t*>(shadowList + 2 * id)[3] = rayId | 0x80000000u;
        reinterpret_cast<int*>(shadowList + 2 * id + 1)[3] = hit.leaf;  // the occluder, for the memo
      }
      id = -1;
    }
  }
}

// Shadowed rays' outputs, one thread per shadow record pair: the shadowed radiance k_shade parked in the
// second record replaces the lit one in the ray image (and the planar 16-bit copy), and the hit code gets its
// shadow bit.
template <class Src>
__global__ void __launch_bounds__(256) k_shadow_resolve(const __grid_constant__ Src src,
                                                        const float4* __restrict__ shadowList,
                                                        const unsigned long long* __restrict__ counters) {
  const long long total = (long long)counters[1];
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const uint32_t u = __float_as_uint(shadowList[2 * k].w);
    const uint32_t id = u & 0x7fffffffu;
    const long long warp = id >> 5;
    const TraceItem& T = src.at(warp);
    const bool shadowed = (u & 0x80000000u) != 0;
    if (!shadowed && !T.occMemo) continue;
    const RaySlot rs = naturalRay(T.g, T.f, T.order, (uint32_t)(id - 32 * T.warpBegin)).rs;
    const float4 hr = shadowList[2 * k + 1];
    if (T.occMemo)  // the occluder of this shadow ray (-1: unshadowed), the next trace's candidate
      T.occMemo[(((size_t)rs.layer * T.g.Z + rs.pz) * T.g.X + rs.px) * T.g.N + rs.j] =
          shadowed ? __float_as_int(hr.w) : -1;
    if (!shadowed) continue;
    const float3 Ls = xyz(hr);
    const size_t idx = rayIndex(T.g, rs);
    storeTexel(T.rayRad, T.g.rayFmt, idx, make_float4(Ls.x, Ls.y, Ls.z, 1.0f));
    if (T.rayHit) T.rayHit[idx] |= 1;
    if (T.g.rad16) storeRad16(T.g, rs, Ls);
  }
}

// Ray queries (DdgiRay -> DdgiHit) on the persistent refill loop of the probe traversal. kShadowMask:
// the rays are shadow.rgen's (origin = the point, direction = -lightDir, [0.1, 50], any hit) and the output
// is its visibility mask; points with w != 0 are sky pixels (visibility 1, no ray).
// kLightSpace (with kShadowMask): the points' rays run in the light-space BVH `bvh` along +z, each point
// sheared by (shK, shS) as the probe update's shadow rays are; shadowDir must then be the normalised
// direction toward the light that the BVH was sheared for.
template <bool kWide, bool kAnyHit, bool kShadowMask, bool kLightSpace = false>
__global__ void __launch_bounds__(kTraceThreads, DDGI_TRACE_MIN_BLOCKS)
    k_trace_rays(BvhRef bvh, const DdgiRay* __restrict__ rays, const float4* __restrict__ points, float3 shadowDir,
                 long long count, unsigned long long* __restrict__ counter, int refillLanes, DdgiHit* __restrict__ hits,
                 float* __restrict__ vis, bool recordIds, uint32_t* __restrict__ err, int3 shK, float3 shS) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  long long id = -1;
  bool drained = false;
  WRay ray;
  HitInfo hit;
  typename TravOf<kWide>::T st;
  float tmin = kTMin;
  auto finish = [&](long long i) {
    if (kShadowMask) {
      vis[i] = hit.leaf >= 0 ? 0.0f : 1.0f;  // shadow.rchit:14 / shadow.rmiss:12
    } else {
      int gid = -1;
      if (hit.leaf >= 0) gid = recordIds ? hit.leaf : __float_as_int(__ldg(&bvh.tris[3 * hit.leaf].w));
      hits[i] = DdgiHit{hit.leaf >= 0 ? hit.t : 0.0f, hit.leaf >= 0 ? hit.b1 : 0.0f, hit.leaf >= 0 ? hit.b2 : 0.0f, gid};
    }
  };
  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, id < 0);
    if (drained && idle == 0xffffffffu) break;
    if (!drained && __popc(idle) >= refillLanes) {
      const int need = __popc(idle);
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(counter, (unsigned long long)need);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((long long)base + need >= count) drained = true;
      const long long cand = (long long)base + __popc(idle & below);
      if (id < 0 && cand < count) {
        float3 o, d;
        float t1;
        bool sky = false;
        if (kShadowMask) {
          const float4 p = points[cand];
          o = xyz(p);
          d = shadowDir;
          if (kLightSpace) {
            const float pk[3] = {p.x, p.y, p.z};
            const float pz = pk[shK.z];
            o = f3(pk[shK.x] - shS.x * pz, pk[shK.y] - shS.y * pz, shS.z * pz);
            d = f3(0.f, 0.f, 1.f);
          }
          tmin = kTMin;
          t1 = kTMax;
          sky = p.w != 0.0f;
        } else {
          const DdgiRay r = rays[cand];
          o = f3(r.origin[0], r.origin[1], r.origin[2]);
          d = f3(r.direction[0], r.direction[1], r.direction[2]);
          tmin = r.tmin;
          t1 = r.tmax;
        }
        if (sky) {
          vis[cand] = 1.0f;  // shadow.rgen:44-47
        } else {
          ray = makeRay(o, d);
          bool done;
          if constexpr (kWide) done = wideInit<kAnyHit>(bvh, ray, t1, st, hit);
          else done = binInit<kAnyHit>(bvh, ray, tmin, t1, st, hit);
          if (done) finish(cand);
          else id = cand;
        }
      }
    }
    if (id >= 0) {
      bool done;
      if constexpr (kWide) done = wideStep<kAnyHit, kLightSpace>(bvh, ray, tmin, st, hit, err);
      else done = binStep<kAnyHit>(bvh, ray, tmin, st, hit, err);
      if (done) {
        finish(id);
        id = -1;
      }
    }
  }
}

cudaError_t launchTraceRays(const BvhRef& bvh, bool wide, const DdgiRay* rays, long long count, bool anyHit,
                            DdgiHit* hits, const float4* points, float3 shadowDir, float* vis,
                            unsigned long long* counter, uint32_t* err, cudaStream_t stream, bool recordIds,
                            const SceneGPU* light) {
  if (count <= 0) return cudaSuccess;
  const int3 shK = light ? make_int3(light->shearK[0], light->shearK[1], light->shearK[2]) : make_int3(0, 1, 2);
  const float3 shS = light ? f3(light->shearS[0], light->shearS[1], light->shearS[2]) : f3(0.f, 0.f, 1.f);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8;
  const int refill = 8;
  if (points && light) {  // shadow mask in the light-space BVH
    const BvhRef& lb = light->shadow;
    if (wide) k_trace_rays<true, true, true, true><<<blocks, kTraceThreads, 0, stream>>>(lb, nullptr, points, shadowDir, count, counter, refill, nullptr, vis, recordIds, err, shK, shS);
    else k_trace_rays<false, true, true, true><<<blocks, kTraceThreads, 0, stream>>>(lb, nullptr, points, shadowDir, count, counter, refill, nullptr, vis, recordIds, err, shK, shS);
  } else if (points) {  // shadow mask: any hit
    if (wide) k_trace_rays<true, true, true><<<blocks, kTraceThreads, 0, stream>>>(bvh, nullptr, points, shadowDir, count, counter, refill, nullptr, vis, recordIds, err, shK, shS);
    else k_trace_rays<false, true, true><<<blocks, kTraceThreads, 0, stream>>>(bvh, nullptr, points, shadowDir, count, counter, refill, nullptr, vis, recordIds, err, shK, shS);
  } else if (anyHit) {
    if (wide) k_trace_rays<true, true, false><<<blocks, kTraceThreads, 0, stream>>>(bvh, rays, nullptr, shadowDir, count, counter, refill, hits, nullptr, recordIds, err, shK, shS);
    else k_trace_rays<false, true, false><<<blocks, kTraceThreads, 0, stream>>>(bvh, rays, nullptr, shadowDir, count, counter, refill, hits, nullptr, recordIds, err, shK, shS);
  } else {
    if (wide) k_trace_rays<true, false, false><<<blocks, kTraceThreads, 0, stream>>>(bvh, rays, nullptr, shadowDir, count, counter, refill, hits, nullptr, recordIds, err, shK, shS);
    else k_trace_rays<false, false, false><<<blocks, kTraceThreads, 0, stream>>>(bvh, rays, nullptr, shadowDir, count, counter, refill, hits, nullptr, recordIds, err, shK, shS);
  }
  return cudaGetLastError();
}

// Atlas consumer (deferred_tiled.comp:263-299): the ambient term of G-buffer points, one thread per point.
__global__ void __launch_bounds__(256) k_query_irradiance(GridGPU g, FrameGPU f, const void* __restrict__ atlas,
                                                          const DdgiSurfacePoint* __restrict__ pts, long long count,
                                                          float4* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const DdgiSurfacePoint& p = pts[i];
    const float3 wp = f3(p.position[0], p.position[1], p.position[2]);
    const float3 n = normalize3(f3(p.normal[0], p.normal[1], p.normal[2]));  // :177
    const float3 albedo = f3(p.albedo[0], p.albedo[1], p.albedo[2]);
    const float shade = clampf(p.shadow, 0.3f, 1.0f);
    float3 amb = f3(0.f, 0.f, 0.f);  // :203
    if (f.flags & DDGI_UBO_DDGI_FLAG) {
      const float3 d = f.camPos - wp;
      if (sqrtf(dot3(d, d)) > (float)g.X * g.step.x / 2.0f)  // :271-273
        amb += f3(0.3f, 0.3f, 0.3f) * f.skyIntensity * albedo * shade;
      else
        amb += calcIndirectDiffuse(g, f, atlas, n, albedo, p.metallic, p.roughness, wp, f.camPos);  // :289-295
    } else {
      amb = f3(0.3f, 0.3f, 0.3f) * albedo * shade;  // :298
    }
    out[i] = make_float4(amb.x, amb.y, amb.z, 0.0f);
  }
}

cudaError_t launchQueryIrradiance(const GridGPU& g, const FrameGPU& f, const void* atlas, const DdgiSurfacePoint* pts,
                                  long long count, float4* out, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  GridGPU gc = g;
  gc.samplerClamp = 1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long blocks = (count + 255) / 256;
  if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
  k_query_irradiance<<<(unsigned)blocks, 256, 0, stream>>>(gc, f, atlas, pts, count, out);
  return cudaGetLastError();
}

// ---- specular GI mirror pass (SpecularGIRTPass.cpp:111-128; mirror_reflections.rgen/.rchit/.rmiss) ----------

// Ray of each G-buffer point (rgen:38-80): origin = the point, direction = reflect(v, n) = v - 2 dot(n, v) n
// with v = normalize(point - cameraPos), n = normalize(normal), range [0.1, 50]. A sky point (rgen:52-55) gets
// an empty range, so the trace reports a miss and the shading writes 0.
__global__ void __launch_bounds__(256) k_mirror_rays(FrameGPU f, const DdgiMirrorPoint* __restrict__ pts,
                                                     long long count, DdgiRay* __restrict__ rays) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const DdgiMirrorPoint p = pts[i];
    const float3 pos = f3(p.position[0], p.position[1], p.position[2]);
    DdgiRay r;
    r.origin[0] = pos.x; r.origin[1] = pos.y; r.origin[2] = pos.z;
    if (p.sky != 0.0f) {
      r.direction[0] = 0.0f; r.direction[1] = 0.0f; r.direction[2] = 1.0f;
      r.tmin = 1.0f;
      r.tmax = 0.0f;
    } else {
      const float3 n = normalize3(f3(p.normal[0], p.normal[1], p.normal[2]));
      const float3 v = normalize3(pos - f.camPos);
      const float3 d = v - n * (2.0f * dot3(n, v));
      r.direction[0] = d.x; r.direction[1] = d.y; r.direction[2] = d.z;
      r.tmin = kTMin;
      r.tmax = kTMax;
    }
    rays[i] = r;
  }
}

// Mirror hits (rchit:24-117) and misses (rmiss:17-21), one thread per point. A hit gets both radiance
// values, lit = calcLight + indirect + emissive and shadowed = indirect + emissive (the reference's order of
// additions), with the indirect term when DDGI_UBO_DDGI_FLAG is set (rchit:106) and the hit distance in .w
// (rchit:90); its world position becomes the point of a shadow ray (w = 0). Misses: the linear sky with
// distance 1e6; sky points: 0. Neither casts a shadow ray (w = 1).
__global__ void __launch_bounds__(256) k_mirror_shade(SceneGPU s, GridGPU g, FrameGPU f, const void* __restrict__ atlas,
                                                      const DdgiMirrorPoint* __restrict__ pts,
                                                      const DdgiHit* __restrict__ hits, long long count,
                                                      float4* __restrict__ out, float4* __restrict__ shadowed,
                                                      float4* __restrict__ spts) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const DdgiMirrorPoint& p = pts[i];
    const DdgiHit hr = hits[i];
    float4 lit = make_float4(0.f, 0.f, 0.f, 0.f), dark = lit, sp = make_float4(0.f, 0.f, 0.f, 1.f);
    if (p.sky == 0.0f) {
      if (hr.triangle < 0) {
        const float3 sky = f.skyLinear;
        lit = dark = make_float4(sky.x, sky.y, sky.z, 1e6f);
      } else {
        const float3 origin = f3(p.position[0], p.position[1], p.position[2]);
        const HitSurface h = reconstructHit<true>(s, hr.triangle, hr.b1, hr.b2);
        const float3 d = h.pos - origin;
        const float dist = sqrtf(dot3(d, d));
        float3 L = calcLightDirectional(h.normal, h.color, h.metallic, h.roughness, h.pos, origin, f.lightDir,
                                        f.sunIntensity);
        float3 Ls = f3(0.f, 0.f, 0.f);
        if (f.flags & DDGI_UBO_DDGI_FLAG) {
          const float3 ind = calcIndirectDiffuse(g, f, atlas, h.normal, h.color, h.metallic, h.roughness, h.pos, origin);
          L += ind;
          Ls += ind;
        }
        L += h.emissive;
        Ls += h.emissive;
        lit = make_float4(L.x, L.y, L.z, dist);
        dark = make_float4(Ls.x, Ls.y, Ls.z, dist);
        // no shadow ray when it cannot change the result: lit and shadowed radiance with the same bits
        // (calcLight exactly 0 on a surface facing away from the sun)
        const bool same = __float_as_uint(L.x) == __float_as_uint(Ls.x) && __float_as_uint(L.y) == __float_as_uint(Ls.y) &&
                          __float_as_uint(L.z) == __float_as_uint(Ls.z);
        sp = make_float4(h.pos.x, h.pos.y, h.pos.z, same ? 1.f : 0.f);
      }
    }
    out[i] = lit;
    shadowed[i] = dark;
    spts[i] = sp;
  }
}

// A hit whose shadow ray found geometry takes the shadowed radiance (rchit:92-104).
__global__ void __launch_bounds__(256) k_mirror_resolve(const float* __restrict__ vis, const float4* __restrict__ shadowed,
                                                        float4* __restrict__ out, long long count) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    if (vis[i] == 0.0f) out[i] = shadowed[i];
}

size_t mirrorScratchBytes(long long count) { return (size_t)count * (32 + 16 + 16 + 16 + 4); }

cudaError_t launchMirror(const SceneGPU& s, const GridGPU& g, const FrameGPU& f, const void* atlas,
                         const DdgiMirrorPoint* pts, long long count, float4* out, void* scratch,
                         unsigned long long* counter, uint32_t* err, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  char* b = static_cast<char*>(scratch);
  DdgiRay* rays = reinterpret_cast<DdgiRay*>(b);
  DdgiHit* hits = reinterpret_cast<DdgiHit*>(b + (size_t)count * 32);
  float4* spts = reinterpret_cast<float4*>(b + (size_t)count * 48);
  float4* dark = reinterpret_cast<float4*>(b + (size_t)count * 64);
  float* vis = reinterpret_cast<float*>(b + (size_t)count * 80);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long blocks = (count + 255) / 256;
  if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
  k_mirror_rays<<<(unsigned)blocks, 256, 0, stream>>>(f, pts, count, rays);
  const bool wide = s.bvh.wnodes != nullptr;
  cudaError_t e = launchTraceRays(s.bvh, wide, rays, count, false, hits, nullptr, f3(0.f, 0.f, 0.f), nullptr, counter,
                                  err, stream, true);
  if (e != cudaSuccess) return e;
  k_mirror_shade<<<(unsigned)blocks, 256, 0, stream>>>(s, g, f, atlas, pts, hits, count, out, dark, spts);
  // the shadow ray of rchit:45-66: normalize(-lightDir) over [0.1, 50], terminating on the first hit; in the
  // light-space BVH when the scene carries one for this light (the caller makes sure it matches)
  const float3 ld = f.lightDir * -1.0f;
  const float3 sdir = ld * (1.0f / sqrtf(ld.x * ld.x + ld.y * ld.y + ld.z * ld.z));
  const bool lightSpace = s.shadow.tris != nullptr;
  e = launchTraceRays(s.bvh, lightSpace ? s.shadow.wnodes != nullptr : wide, nullptr, count, true, nullptr, spts,
                      sdir, vis, counter, err, stream, false, lightSpace ? &s : nullptr);
  if (e != cudaSuccess) return e;
  k_mirror_resolve<<<(unsigned)blocks, 256, 0, stream>>>(vis, dark, out, count);
  return cudaGetLastError();
}

__global__ void k_lattice_unit(int n, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[3];
  unitLatticeDir(i, n, v);
  out[3 * i] = v[0];
  out[3 * i + 1] = v[1];
  out[3 * i + 2] = v[2];
}

// Rotated lattices of many grids: one block row per item. The unrotated unit lattice comes from the grid's
// FP64 table when it has one (the same values unitLatticeDir gives), else it is computed here.
// Records from `items` and `rots` in device memory, or `one` and `rotOne` when items is null. Block (0, 0)
// also zeroes the trace counters, which the wavefront kernels launched after this one use.
__global__ void k_lattice_batch(const TraceItem* __restrict__ items, const Mat3* __restrict__ rots,
                                const __grid_constant__ TraceItem one, const __grid_constant__ Mat3 rotOne,
                                unsigned long long* __restrict__ counters) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < kTraceCounters) counters[threadIdx.x] = 0ull;
  const TraceItem& it = items ? items[blockIdx.y] : one;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= it.g.N) return;
  double v[3];
  if (it.latticeUnit) {
    v[0] = it.latticeUnit[3 * i];
    v[1] = it.latticeUnit[3 * i + 1];
    v[2] = it.latticeUnit[3 * i + 2];
  } else {
    unitLatticeDir(i, it.g.N, v);
  }
  const float* m = items ? rots[blockIdx.y].m : rotOne.m;
  double r[3];
  for (int row = 0; row < 3; ++row)
    r[row] = (double)m[row] * v[0] + (double)m[3 + row] * v[1] + (double)m[6 + row] * v[2];
  if (it.latticePrev) it.latticePrev[i] = it.lattice[i];  // the last traced lattice, for the seed map
  const float4 d = make_float4((float)r[0], (float)r[1], (float)r[2], 0.0f);
  const_cast<float4*>(it.lattice)[i] = d;
  if (it.rayDirs) {  // the direction's ray record, which the closest-hit traversal's rays of direction i share
    const RayDirRec p = packRayDir(xyz(d));
    const_cast<float4*>(it.rayDirs)[2 * i] = p.a;
    const_cast<float4*>(it.rayDirs)[2 * i + 1] = p.b;
  }
}

// Seed map of the items that seed their closest hits: for each direction of the new lattice the nearest
// direction of the last traced one (largest dot product, the lowest index on ties). Any choice is exact; a
// near direction makes the candidate likely to be hit. kSeedLanes lanes share a direction: lane l scans the
// previous directions l, l + kSeedLanes, ..., and a shuffle reduction keeps the best (dot, index) pair, so a
// lattice of N directions runs on N * kSeedLanes threads.
constexpr int kSeedStageMax = 1024;  // raysPerProbe is at most 1024 (validated when a grid is created)
constexpr int kSeedLanes = 8;
constexpr int kSeedThreads = 128;  // kSeedThreads / kSeedLanes directions per block
__global__ void __launch_bounds__(kSeedThreads) k_seed_dirs(const TraceItem* __restrict__ items,
                                                            const __grid_constant__ TraceItem one) {
  __shared__ float4 sPrev[kSeedStageMax];
  const TraceItem& it = items ? items[blockIdx.y] : one;
  if (!it.seedOn) return;  // the same for the whole block
  // the fields in registers: `it` may be a parameter, read through a generic reference
  const int n = it.g.N;
  const float4* __restrict__ prev = it.latticePrev;
  // the last traced lattice staged once per block; the scan below reads it from shared memory
  const bool staged = n <= kSeedStageMax;
  if (staged)
    for (int i = threadIdx.x; i < n; i += blockDim.x) sPrev[i] = __ldg(&prev[i]);
  __syncthreads();
  const int sub = threadIdx.x % kSeedLanes;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) / kSeedLanes;
  const bool live = j < n;  // lanes past the lattice still take part in the shuffles
  const float4 d = live ? it.lattice[j] : make_float4(0.f, 0.f, 0.f, 0.f);
  float best = -3.0f;
  int bi = 0x7fffffff;
  if (live)
    for (int i = sub; i < n; i += kSeedLanes) {
      const float4 q = staged ? sPrev[i] : __ldg(&prev[i]);
      const float c = d.x * q.x + d.y * q.y + d.z * q.z;
      if (c > best) {  // increasing i within a lane: the first of equal values stays
        best = c;
        bi = i;
      }
    }
#pragma unroll
  for (int off = kSeedLanes / 2; off > 0; off >>= 1) {
    const float ob = __shfl_xor_sync(0xffffffffu, best, off);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  if (live && sub == 0) it.seedDir[j] = bi == 0x7fffffff ? 0 : bi;  // no comparable direction: any is exact
}

// ---------------------------------------------------------------------------------------------------
cudaError_t launchLatticeUnit(int n, double* out, cudaStream_t stream) {
  k_lattice_unit<<<(n + 31) / 32, 32, 0, stream>>>(n, out);
  return cudaGetLastError();
}

cudaError_t launchLattice(int n, const float rot[9], float4* out, cudaStream_t stream) {
  Mat3 m;
  for (int i = 0; i < 9; ++i) m.m[i] = rot[i];
  k_lattice<<<(n + 127) / 128, 128, 0, stream>>>(n, m, out);
  return cudaGetLastError();
}

long long traceWarps(const GridGPU& g, const FrameGPU& f) {
  int layers = f.layerEnd - f.layerBegin;
  if (layers <= 0) return 0;
  const int D = 32 / g.warpProbes;
  long long probeGroups = (g.X * g.Z + g.warpProbes - 1) / g.warpProbes;
  return probeGroups * layers * (g.N / D);
}

namespace {
// The wavefront kernels of one trace launch with records from `src`.
template <class Src>
void launchWavefront(const Src& src, long long rays, unsigned long long* dCounters, float4* dHits, float4* dShadow,
                     int blocks, int refill, long long shadeBlocks, bool wide, bool lightSpace, uint32_t* err,
                     cudaStream_t stream) {
  if (wide)
    k_trace_closest<true, Src><<<blocks, kTraceThreads, 0, stream>>>(src, rays, dCounters, refill, dHits, err);
  else
    k_trace_closest<false, Src><<<blocks, kTraceThreads, 0, stream>>>(src, rays, dCounters, refill, dHits, err);
  k_shade<Src><<<(unsigned)shadeBlocks, 256, 0, stream>>>(src, rays, dHits, dShadow, dCounters);
  auto shadow = wide ? (lightSpace ? k_trace_shadow<true, true, Src> : k_trace_shadow<true, false, Src>)
                     : (lightSpace ? k_trace_shadow<false, true, Src> : k_trace_shadow<false, false, Src>);
  const int shadowBlocks = lightSpace ? blocks * kShadowLightBlocks / DDGI_TRACE_MIN_BLOCKS : blocks;
  // the shadow rays' traversal refills at half the closest-hit threshold (their rays are shorter)
  shadow<<<shadowBlocks, kTraceThreads, 0, stream>>>(src, dShadow, dCounters, refill > 1 ? refill / 2 : 1, err);
  k_shadow_resolve<Src><<<(unsigned)shadeBlocks, 256, 0, stream>>>(src, dShadow, dCounters);
}

}  // namespace

cudaError_t launchTraceBatch(const TraceItem* dItems, const Mat3* dRots, int numItems, int maxN, long long totalWarps,
                             unsigned long long* dCounters, float4* dHits, float4* dShadow, int blocks,
                             int refillLanes, bool wide, bool lightSpace, uint32_t* err, cudaStream_t stream,
                             const TraceItem* hItems, const Mat3* hRot, const long long* hBegins) {
  // one item given on the host with its rotation: every kernel takes it in its parameters, and dItems /
  // dRots are not read
  const bool byValue = hItems && hRot && numItems == 1;
  const TraceItem one = byValue ? hItems[0] : TraceItem{};
  const Mat3 rotOne = byValue ? *hRot : Mat3{};
  // one warp per block: the FP64 lattice of a grid spreads over N / 32 SMs
  dim3 lg((maxN + 31) / 32, numItems);
  k_lattice_batch<<<lg, 32, 0, stream>>>(byValue ? nullptr : dItems, dRots, one, rotOne, dCounters);
  dim3 sg((maxN * kSeedLanes + kSeedThreads - 1) / kSeedThreads, numItems);
  k_seed_dirs<<<sg, kSeedThreads, 0, stream>>>(byValue ? nullptr : dItems, one);
  if (totalWarps <= 0) return cudaGetLastError();
  const long long rays = totalWarps * 32;
  if (rays > 0x7fffffffll) return cudaErrorInvalidValue;  // shadow records carry 31-bit slot ids + a flag
  const int refill = refillLanes < 1 ? 1 : (refillLanes > 32 ? 32 : refillLanes);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long shadeBlocks = (rays + 255) / 256;
  if (shadeBlocks > (long long)sms * 16) shadeBlocks = (long long)sms * 16;
  if (byValue) {
    launchWavefront(ItemsOne{hItems[0]}, rays, dCounters, dHits, dShadow, blocks, refill, shadeBlocks, wide, lightSpace,
                    err, stream);
  } else {
    ItemsGlobal src{};
    src.items = dItems;
    src.n = numItems;
    src.inParams = hBegins && numItems <= kParamItems ? 1 : 0;
    if (src.inParams)
      for (int i = 0; i < numItems; ++i) src.begins[i] = hBegins[i];
    launchWavefront(src, rays, dCounters, dHits, dShadow, blocks, refill, shadeBlocks, wide,
                    lightSpace, err, stream);
  }
  return cudaGetLastError();
}


}  // namespace ddgi
