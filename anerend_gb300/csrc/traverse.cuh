// Ray traversal shared by the device kernels and host builds of this header (CPU tests):
//   - the watertight ray/triangle test (Woop, Benthin, Wald 2013, "Watertight Ray/Triangle Intersection")
//   - the conservative slab test (Ize 2013, "Robust BVH Ray Traversal")
//   - traversal of the binary LBVH (Aila-Laine node layout) and of the 8-wide BVH collapsed from it
// Closest hit: smallest t, ties to the lowest global triangle id. Any hit: the first triangle in range.
// Both traversals visit every triangle whose box the conservative slab test accepts, so they return the
// same closest hit whatever the tree shape. Replaces the RT-core traceRayEXT calls of the reference
// (irradiance_probe_update.rgen:96-106, .rchit:55-66).
#pragma once

#include <limits.h>
#include <string.h>
#include "ddgi_common.cuh"

namespace ddgi {

#ifdef __CUDA_ARCH__
DDGI_D float mulRn(float a, float b) { return __fmul_rn(a, b); }
DDGI_D float subRn(float a, float b) { return __fsub_rn(a, b); }
DDGI_D float divRn(float a, float b) { return __fdiv_rn(a, b); }
template <class T> DDGI_D T ldRo(const T* p) { return __ldg(p); }
DDGI_D int asInt(float f) { return __float_as_int(f); }
DDGI_D uint32_t asUint(float f) { return __float_as_uint(f); }
DDGI_D int lowestBit(uint32_t m) { return __ffs(m) - 1; }
DDGI_D int popc(uint32_t m) { return __popc(m); }
DDGI_D int bitEnd(uint32_t m) { return 32 - __clz(m); }  // 1 + index of the highest set bit
DDGI_D uint32_t bytePerm(uint32_t x, uint32_t y, uint32_t sel) { return __byte_perm(x, y, sel); }
DDGI_D float asFloatHd(uint32_t u) { return __uint_as_float(u); }
DDGI_D void flagError(uint32_t* err, uint32_t bits) { atomicOr(err, bits); }
DDGI_D float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
DDGI_D float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
// Two round-to-nearest FMAs in one packed FP32 instruction: (a.x b.x + c.x, a.y b.y + c.y), each the same
// value fmaf gives.
DDGI_D float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long A, B, C, D;
  asm("mov.b64 %0, {%1, %2};" : "=l"(A) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(B) : "f"(b.x), "f"(b.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(C) : "f"(c.x), "f"(c.y));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(D) : "l"(A), "l"(B), "l"(C));
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(D));
  return d;
}
// Two round-to-nearest products / differences in one packed FP32 instruction (never contracted).
DDGI_D float2 mul2(float2 a, float2 b) {
  unsigned long long A, B, D;
  asm("mov.b64 %0, {%1, %2};" : "=l"(A) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(B) : "f"(b.x), "f"(b.y));
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(D) : "l"(A), "l"(B));
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(D));
  return d;
}
DDGI_D float2 sub2(float2 a, float2 b) {
  unsigned long long A, B, D;
  asm("mov.b64 %0, {%1, %2};" : "=l"(A) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(B) : "f"(b.x), "f"(b.y));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(D) : "l"(A), "l"(B));
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(D));
  return d;
}
#else
// host builds must compile with -ffp-contract=off so products and differences round separately
inline float mulRn(float a, float b) { return a * b; }
inline float subRn(float a, float b) { return a - b; }
inline float divRn(float a, float b) { return a / b; }
template <class T> inline T ldRo(const T* p) { return *p; }
inline int asInt(float f) { int i; memcpy(&i, &f, 4); return i; }
inline uint32_t asUint(float f) { uint32_t i; memcpy(&i, &f, 4); return i; }
inline int lowestBit(uint32_t m) { return __builtin_ctz(m); }
inline int popc(uint32_t m) { return __builtin_popcount(m); }
inline int bitEnd(uint32_t m) { return m ? 32 - __builtin_clz(m) : 0; }
inline float asFloatHd(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
inline uint32_t bytePerm(uint32_t x, uint32_t y, uint32_t sel) {
  uint64_t v = ((uint64_t)y << 32) | x;
  uint32_t r = 0;
  for (int k = 0; k < 4; ++k) r |= (uint32_t)((v >> (8 * ((sel >> (4 * k)) & 7))) & 0xff) << (8 * k);
  return r;
}
inline void flagError(uint32_t* err, uint32_t bits) { if (err) *err |= bits; }
inline float max3f(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }
inline float min3f(float a, float b, float c) { return fminf(fminf(a, b), c); }
inline float2 fma2(float2 a, float2 b, float2 c) { return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y)); }
inline float2 mul2(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
inline float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
#endif

struct WRay {
  float3 o, invd;
  // box distances as one FMA per plane: t = fma(plane, invd, add) with add = -o * invd widened by an
  // absolute margin (nAdd for near planes, fAdd for far planes), see wideStep
  float3 nAdd, fAdd;
  float3 invd15;  // invd * 2^15 and |invd| * 2^-21 (quantized wide nodes)
  float3 invdM;
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

// The direction-only part of a ray: the watertight test's axis permutation and shear constants and the box
// test's reciprocals, as two float4: (invd.xyz, Sx), (Sy, Sz, kx | ky << 2 | kz << 4 as bits, 0). Rays that
// share a direction (a probe grid's rays of one lattice direction) share it, so it is computed once per direction.
struct RayDirRec {
  float4 a, b;
};

DDGI_HD RayDirRec packRayDir(float3 d) {
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  float dz = get(d, kz);
  if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }
  const float Sx = get(d, kx) / dz, Sy = get(d, ky) / dz, Sz = 1.0f / dz;
  // box-test reciprocals; a zero component becomes a tiny same-signed value so (lo - o) * invd is finite
  float3 dd = f3(d.x != 0.f ? d.x : copysignf(1e-20f, d.x), d.y != 0.f ? d.y : copysignf(1e-20f, d.y),
                 d.z != 0.f ? d.z : copysignf(1e-20f, d.z));
  RayDirRec p;
  p.a = make_float4(1.0f / dd.x, 1.0f / dd.y, 1.0f / dd.z, Sx);
  p.b = make_float4(Sy, Sz, asFloatHd((uint32_t)(kx | (ky << 2) | (kz << 4))), 0.0f);
  return p;
}

// A ray from its origin and its direction record (packRayDir).
DDGI_HD WRay makeRayPacked(float3 o, const RayDirRec& p) {
  WRay r;
  r.o = o;
  const uint32_t k = asUint(p.b.z);
  r.kx = (int)(k & 3u);
  r.ky = (int)((k >> 2) & 3u);
  r.kz = (int)((k >> 4) & 3u);
  r.Sx = p.a.w;
  r.Sy = p.b.x;
  r.Sz = p.b.y;
  r.invd = f3(p.a.x, p.a.y, p.a.z);
  // margin 2^-21 |o * invd| (8 units of rounding) covers the rounding of o * invd and of the additions,
  // leaving one rounding of the FMA, within the conservative far-distance factor of the slab test
  const float wx = o.x * r.invd.x, wy = o.y * r.invd.y, wz = o.z * r.invd.z;
  const float ex = fabsf(wx) * 4.76837158203125e-7f, ey = fabsf(wy) * 4.76837158203125e-7f,
              ez = fabsf(wz) * 4.76837158203125e-7f;
  r.nAdd = f3(-wx - ex, -wy - ey, -wz - ez);
  r.fAdd = f3(-wx + ex, -wy + ey, -wz + ez);
  r.invd15 = r.invd * 32768.0f;
  r.invdM = f3(fabsf(r.invd.x), fabsf(r.invd.y), fabsf(r.invd.z)) * 4.76837158203125e-7f;
  return r;
}

// The same ray from its direction (packRayDir and makeRayPacked in one, the same arithmetic).
DDGI_HD WRay makeRay(float3 o, float3 d) {
  WRay r;
  r.o = o;
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  float dz = get(d, kz);
  if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.Sx = get(d, kx) / dz;
  r.Sy = get(d, ky) / dz;
  r.Sz = 1.0f / dz;
  float3 dd = f3(d.x != 0.f ? d.x : copysignf(1e-20f, d.x), d.y != 0.f ? d.y : copysignf(1e-20f, d.y),
                 d.z != 0.f ? d.z : copysignf(1e-20f, d.z));
  r.invd = f3(1.0f / dd.x, 1.0f / dd.y, 1.0f / dd.z);
  const float wx = o.x * r.invd.x, wy = o.y * r.invd.y, wz = o.z * r.invd.z;
  const float ex = fabsf(wx) * 4.76837158203125e-7f, ey = fabsf(wy) * 4.76837158203125e-7f,
              ez = fabsf(wz) * 4.76837158203125e-7f;
  r.nAdd = f3(-wx - ex, -wy - ey, -wz - ez);
  r.fAdd = f3(-wx + ex, -wy + ey, -wz + ez);
  r.invd15 = r.invd * 32768.0f;
  r.invdM = f3(fabsf(r.invd.x), fabsf(r.invd.y), fabsf(r.invd.z)) * 4.76837158203125e-7f;
  return r;
}

// Returns true for a hit with tmin <= t <= tmax; b1, b2 are the weights of v1, v2. Products and
// differences of the edge functions are not contracted into FMAs, so a shared edge evaluates to the same
// value (with opposite sign) from both of its triangles.
DDGI_HD bool intersectTri(const WRay& r, float3 v0, float3 v1, float3 v2, float tmin, float tmax, float& t,
                          float& b1, float& b2) {
  float3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
  float Akz = get(A, r.kz), Bkz = get(B, r.kz), Ckz = get(C, r.kz);
  // the sheared x and y of each vertex, and two of the three edge functions, as packed pairs: the same
  // separately rounded products and differences
  const float2 S = make_float2(r.Sx, r.Sy);
  const float2 Axy = sub2(make_float2(get(A, r.kx), get(A, r.ky)), mul2(S, make_float2(Akz, Akz)));
  const float2 Bxy = sub2(make_float2(get(B, r.kx), get(B, r.ky)), mul2(S, make_float2(Bkz, Bkz)));
  const float2 Cxy = sub2(make_float2(get(C, r.kx), get(C, r.ky)), mul2(S, make_float2(Ckz, Ckz)));
  const float Ax = Axy.x, Ay = Axy.y, Bx = Bxy.x, By = Bxy.y, Cx = Cxy.x, Cy = Cxy.y;
  const float2 UV = sub2(mul2(make_float2(Cx, Ax), make_float2(By, Cy)), mul2(make_float2(Cy, Ay), make_float2(Bx, Cx)));
  float U = UV.x, V = UV.y;
  float W = subRn(mulRn(Bx, Ay), mulRn(By, Ax));
  if (U == 0.0f || V == 0.0f || W == 0.0f) {  // exact fallback of the paper
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  float det = U + V + W;
  if (det == 0.0f) return false;
  float Az = mulRn(r.Sz, Akz), Bz = mulRn(r.Sz, Bkz), Cz = mulRn(r.Sz, Ckz);
  float T = U * Az + V * Bz + W * Cz;
  float tt = divRn(T, det);
  if (!(tt >= tmin && tt <= tmax)) return false;
  float inv = divRn(1.0f, det);
  t = tt;
  b1 = V * inv;
  b2 = W * inv;
  return true;
}

// Slab test with a conservative far distance (Ize 2013: 1 + 2*gamma(3)). Plane distances are
// fma(plane, invd, nAdd) for the near plane of each axis and fma(plane, invd, fAdd) for the far one; the
// margins in nAdd / fAdd keep the test conservative also for an axis-parallel ray whose origin lies exactly
// on a box face (where (plane - o) * invd would give a signed zero far distance).
DDGI_HD bool slab(const WRay& r, float lx, float hx, float ly, float hy, float lz, float hz, float tmin,
                  float tmax, float& tnear) {
  const bool sx = r.invd.x < 0.f, sy = r.invd.y < 0.f, sz = r.invd.z < 0.f;
  const float tnx = fmaf(sx ? hx : lx, r.invd.x, r.nAdd.x), tfx = fmaf(sx ? lx : hx, r.invd.x, r.fAdd.x);
  const float tny = fmaf(sy ? hy : ly, r.invd.y, r.nAdd.y), tfy = fmaf(sy ? ly : hy, r.invd.y, r.fAdd.y);
  const float tnz = fmaf(sz ? hz : lz, r.invd.z, r.nAdd.z), tfz = fmaf(sz ? lz : hz, r.invd.z, r.fAdd.z);
  const float tn = max3f(tnx, tny, fmaxf(tnz, tmin));
  const float tf = min3f(tfx, tfy, fminf(tfz, tmax));
  tnear = tn;
  return tn <= tf * 1.0000004f;
}

struct HitInfo {
  int leaf;  // triangle record index
  int gid;   // global triangle id
  float t, b1, b2;
};

// Test one triangle record; returns true when an any-hit query can stop.
template <bool kAnyHit>
DDGI_HD bool testTri(const BvhRef& b, const WRay& r, int rec, float tmin, HitInfo& hit) {
  float4 a = ldRo(&b.tris[3 * rec]), c1 = ldRo(&b.tris[3 * rec + 1]), c2 = ldRo(&b.tris[3 * rec + 2]);
  float t, b1, b2;
  if (intersectTri(r, xyz(a), xyz(c1), xyz(c2), tmin, hit.t, t, b1, b2)) {
    int g = asInt(a.w);
    if (kAnyHit) {
      hit.leaf = rec; hit.gid = g; hit.t = t; hit.b1 = b1; hit.b2 = b2;
      return true;
    }
    if (t < hit.t || (t == hit.t && g < hit.gid)) {
      hit.leaf = rec; hit.gid = g; hit.t = t; hit.b1 = b1; hit.b2 = b2;
    }
  }
  return false;
}

// ---- binary BVH ------------------------------------------------------------------------------------
// Resumable traversal: init, then step until it returns true. One step visits one node (its two child
// boxes, and the triangles of its leaf children). The persistent kernels interleave steps with refills
// of idle lanes; traverse() runs the steps to the end.
struct BinTrav {
  int node, sp;
  int stack[kStackSize];
};

// Returns true when there is nothing to traverse (no triangles, or a single triangle, tested here).
template <bool kAnyHit>
DDGI_HD bool binInit(const BvhRef& b, const WRay& r, float tmin, float tmax, BinTrav& s, HitInfo& hit) {
  hit.leaf = -1;
  hit.gid = INT_MAX;
  hit.t = tmax;
  s.node = 0;
  s.sp = 0;
  if (b.numTris <= 0) return true;
  if (b.numTris == 1) {
    testTri<kAnyHit>(b, r, 0, tmin, hit);
    return true;
  }
  return false;
}

template <bool kAnyHit>
DDGI_HD bool binStep(const BvhRef& b, const WRay& r, float tmin, BinTrav& s, HitInfo& hit, uint32_t* err) {
  if ((unsigned)s.node >= (unsigned)b.numNodes) {
    flagError(err, DDGI_DEVERR_BOUNDS);
    return true;
  }
  const float4* nd = b.nodes + 4 * s.node;
  float4 n0 = ldRo(nd), n1 = ldRo(nd + 1), n2 = ldRo(nd + 2), n3 = ldRo(nd + 3);
  float tn0, tn1;
  bool h0 = slab(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, tmin, hit.t, tn0);
  bool h1 = slab(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, tmin, hit.t, tn1);
  int c0 = asInt(n3.x), c1 = asInt(n3.y);
  if (h0 && c0 < 0) {
    if (testTri<kAnyHit>(b, r, ~c0, tmin, hit) && kAnyHit) return true;
    h0 = false;
  }
  if (h1 && c1 < 0) {
    if (testTri<kAnyHit>(b, r, ~c1, tmin, hit) && kAnyHit) return true;
    h1 = false;
  }
  if (h0 && h1) {
    int nearC = c0, farC = c1;
    if (tn1 < tn0) { nearC = c1; farC = c0; }
    if (s.sp >= kStackSize) {  // cannot happen for trees of depth <= 64; flag and stop this ray
      flagError(err, DDGI_DEVERR_STACK_OVERFLOW);
      return true;
    }
    s.stack[s.sp++] = farC;
    s.node = nearC;
  } else if (h0) {
    s.node = c0;
  } else if (h1) {
    s.node = c1;
  } else {
    if (s.sp == 0) return true;
    s.node = s.stack[--s.sp];
  }
  return false;
}

template <bool kAnyHit>
DDGI_HD bool traverse(const BvhRef& b, const WRay& r, float tmin, float tmax, HitInfo& hit, uint32_t* err) {
  BinTrav s;
  if (!binInit<kAnyHit>(b, r, tmin, tmax, s, hit))
    while (!binStep<kAnyHit>(b, r, tmin, s, hit, err)) {
    }
  return hit.leaf >= 0;
}

// ---- 8-wide BVH -------------------------------------------------------------------------------------
// Two node layouts, chosen at compile time by DDGI_WIDE_QUANT (default 1, the quantized one: 80 B per node
// against 208 B; the box tests read 2.6x fewer L1 lines per node for a byte-permute and an FMA per plane).
// FP32 node (DDGI_WIDE_QUANT=0) = 13 float4 (208 B):
//   [0]      uint4 header {childBase, triBase, slot masks, 0}
//   [1],[2]  lo.x of slots 0-7      [3],[4]   hi.x      [5],[6]  lo.y   [7],[8]  hi.y
//   [9],[10] lo.z                    [11],[12] hi.z
// Slot masks = internal-slot mask | leaf-slot mask << 8 (bit s: slot s); a slot in neither is empty. The
// internal slot s is wide node childBase + (internal slots below s); the leaf slot s is the single triangle
// record triBase + (leaf slots below s): a node's leaf records are laid out in slot order. Slot s holds the
// child that lies most toward the corner with sign bits s (bit a set = +axis a), so visiting keys
// s ^ octant(ray) in increasing order is roughly front to back.
#ifndef DDGI_WIDE_QUANT
#define DDGI_WIDE_QUANT 1
#endif
#if DDGI_WIDE_QUANT
// Quantized node = 5 float4 (80 B):
//   [0]  float origin p.x, p.y, p.z; uint biased exponents e_x | e_y << 8 | e_z << 16 (scale s_a = 2^(e_a-127))
//   [1]  uint4 header {childBase, triBase, slot masks, 0} as in the FP32 node
//   [2]  q lo.x of slots 0-7 (one byte each) | q lo.y   [3] q lo.z | q hi.x   [4] q hi.y | q hi.z
// Slot boxes are [p + q_lo s, p + q_hi s] in exact arithmetic and contain the child (quantizeSlots rounds
// outward). The traversal reads a byte q as v = 1 + q 2^-15 (one byte permute builds the float) and gets
// the plane distance as fma(v, 2^15 s invd, (p - 2^15 s - o) invd -/+ margin).
constexpr int kWideNodeF4 = 5;
#else
constexpr int kWideNodeF4 = 13;
#endif
constexpr int kWideLeafMax = 1;  // triangles per leaf slot: the header's leaf-slot mask locates one record each
constexpr int kWideStack = 64;

static_assert(kWideLeafMax == 1, "leaf records are located by the leaf-slot mask, one per leaf slot");

// Slot bits to key bits (key = slot ^ oct): swap bit pairs, pairs of pairs and nibbles per octant bit.
DDGI_HD uint32_t slotsToKeys(uint32_t x, uint32_t oct) {
  if (oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
  if (oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
  if (oct & 4u) x = ((x & 0x0fu) << 4) | (x >> 4);
  return x;
}

// node: the next wide node to test, -1 when the stack is exhausted. tMask: the last tested node's hit leaf
// slots still to test (bits 0-7) and that node's leaf-slot mask (bits 8-15), or 0 when none is left; the
// record of leaf slot k is tBase + (leaf slots below k). A step tests one of them. Stack entries are
// {childBase, (internal-slot mask << 8) | remaining keys}; the top entry is held in registers (`top`, {0, 0}
// when the stack is empty) and the ones below it in `stack` (sp of them), so a pop reads and updates
// registers, and the entry below is loaded when the top runs out, a step before it is needed.
struct WideTrav {
  int node, sp;
  uint32_t oct;
  uint32_t tBase, tMask;
  uint2 top;
  uint2 stack[kWideStack];
};

template <bool kAnyHit>
DDGI_HD bool wideInit(const BvhRef& b, const WRay& r, float tmax, WideTrav& s, HitInfo& hit) {
  hit.leaf = -1;
  hit.gid = INT_MAX;
  hit.t = tmax;
  s.node = 0;
  s.sp = 0;
  s.tBase = 0;
  s.tMask = 0;
  s.top = make_uint2(0u, 0u);
  s.oct = (r.invd.x < 0.f ? 1u : 0u) | (r.invd.y < 0.f ? 2u : 0u) | (r.invd.z < 0.f ? 4u : 0u);
  return b.numTris <= 0;
}

// The next node from the stack into s.node (-1 when it is empty). The top entry is empty only when the whole
// stack is: an exhausted top is replaced at once by the entry below it.
DDGI_HD void widePop(WideTrav& s) {
  uint32_t keys = s.top.y & 0xffu;
  if (keys == 0u) {
    s.node = -1;
    return;
  }
  const uint32_t tim = s.top.y >> 8;
  const int key = lowestBit(keys);
  keys &= keys - 1u;
  const uint32_t slot = (uint32_t)key ^ s.oct;
  s.node = (int)(s.top.x + (uint32_t)popc(tim & ((1u << slot) - 1u)));
  if (keys) s.top.y = (tim << 8) | keys;
  else if (s.sp > 0) s.top = s.stack[--s.sp];
  else s.top = make_uint2(0u, 0u);
}

// One step: a lane with pending triangles tests one of them; otherwise it tests the 8 child boxes of its
// current node, keeps the hit leaves' triangles as pending (the first is tested in the same step) and
// moves to the nearest hit internal child or the next node on the stack. A warp's lanes thus run the box
// test together and the rarer triangle tests one at a time instead of a loop as long as the most leaves
// any lane hit. Pending triangles are tested before the next node, so culling by the closest t is the
// same as testing them at once. Returns true when the ray is done.
//
// kPlusZ: every ray has direction exactly (0, 0, 1) (shadow rays in the light's sheared space); the box
// test is then exact: the origin's x, y inside the box's and the z range [lo.z - o.z, hi.z - o.z] meeting
// [tmin, t]. Otherwise near/far distances per axis are fma(plane, invd, nAdd / fAdd).
// kNodeScale (quantized nodes): the node test forms 2^15 s from the node's exponent byte instead of reading
// the ray's invd * 2^15 (WRay::invd15), one more multiply per axis and three registers fewer held per ray;
// the same plane distances either way.
template <bool kAnyHit, bool kPlusZ = false, bool kNodeScale = false>
DDGI_HD void wideNodeTest(const BvhRef& b, const WRay& r, float tmin, WideTrav& s, const HitInfo& hit, uint32_t* err);

template <bool kAnyHit, bool kPlusZ = false, bool kNodeScale = false>
DDGI_HD bool wideStep(const BvhRef& b, const WRay& r, float tmin, WideTrav& s, HitInfo& hit, uint32_t* err) {
  if (s.tMask == 0) wideNodeTest<kAnyHit, kPlusZ, kNodeScale>(b, r, tmin, s, hit, err);
  if (s.tMask != 0) {
    const uint32_t tm = s.tMask;
    const int k = lowestBit(tm);  // a pending slot: the low byte is not empty
    const int rec = (int)s.tBase + popc((tm >> 8) & ((1u << k) - 1u));
    const uint32_t rest = tm & (tm - 1u);
    s.tMask = (rest & 0xffu) ? rest : 0u;
    if (testTri<kAnyHit>(b, r, rec, tmin, hit) && kAnyHit) return true;
  }
  return s.tMask == 0 && s.node < 0;
}

template <bool kAnyHit, bool kPlusZ, bool kNodeScale>
DDGI_HD void wideNodeTest(const BvhRef& b, const WRay& r, float tmin, WideTrav& s, const HitInfo& hit, uint32_t* err) {
  if ((unsigned)s.node >= (unsigned)b.numWNodes) {
    flagError(err, DDGI_DEVERR_BOUNDS);
    s.node = -1;
    s.sp = 0;
    s.top = make_uint2(0u, 0u);
    return;
  }
  const uint32_t oct = s.oct;
  // near / far plane rows of each axis for this ray's direction signs
  const int nxo = (oct & 1) ? 3 : 1, fxo = 4 - nxo;
  const int nyo = (oct & 2) ? 7 : 5, fyo = 12 - nyo;
  const int nzo = (oct & 4) ? 11 : 9, fzo = 20 - nzo;
  const float4* nd = b.wnodes + kWideNodeF4 * s.node;
#if DDGI_WIDE_QUANT
  const float4 h0 = ldRo(nd);
  const uint4 hd = ldRo(reinterpret_cast<const uint4*>(nd + 1));
  const uint4 w0 = ldRo(reinterpret_cast<const uint4*>(nd + 2)), w1 = ldRo(reinterpret_cast<const uint4*>(nd + 3)),
              w2 = ldRo(reinterpret_cast<const uint4*>(nd + 4));
  // byte words: lo.x in w0.x/y, lo.y in w0.z/w, lo.z in w1.x/y, hi.x in w1.z/w, hi.y in w2.x/y, hi.z in w2.z/w
  // (first word: slots 0-3, second: slots 4-7). Near / far words of each axis picked by the ray's direction
  // signs with selects on named words: an array indexed by the octant would be placed in local memory.
  const bool sx = (oct & 1u) != 0, sy = (oct & 2u) != 0, sz = (oct & 4u) != 0;
  const uint32_t qn[6] = {sx ? w1.z : w0.x, sx ? w1.w : w0.y, sy ? w2.x : w0.z, sy ? w2.y : w0.w,
                          sz ? w2.z : w1.x, sz ? w2.w : w1.y};
  const uint32_t qf[6] = {sx ? w0.x : w1.z, sx ? w0.y : w1.w, sy ? w0.z : w2.x, sy ? w0.w : w2.y,
                          sz ? w1.x : w2.z, sz ? w1.y : w2.w};
  const uint32_t eb = asUint(h0.w);
  const float p[3] = {h0.x, h0.y, h0.z};
  const float o[3] = {r.o.x, r.o.y, r.o.z};
  const float iv[3] = {r.invd.x, r.invd.y, r.invd.z};
  const float iv15[3] = {r.invd15.x, r.invd15.y, r.invd15.z};
  const float ivm[3] = {r.invdM.x, r.invdM.y, r.invdM.z};
  float A[3], Bn[3], Bf[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const uint32_t e = (eb >> (8 * a)) & 0xffu;
    const float sc = asFloatHd(e << 23);
    float c;  // p - 2^15 s
    if (kNodeScale) {
      const float sc15 = sc * 32768.0f;
      c = p[a] - sc15;
      A[a] = sc15 * iv[a];
    } else {
      c = fmaf(-32768.0f, sc, p[a]);
      A[a] = sc * iv15[a];
    }
    const float B = (c - o[a]) * iv[a];
    const float E = (fabsf(c) + fabsf(o[a])) * ivm[a];
    Bn[a] = B - E;
    Bf[a] = B + E;
  }
  float Rv[2] = {0.f, 0.f};
  if (kPlusZ) {  // the origin in each axis' quantized units as 1 + R 2^-15, for the exact x / y containment
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const uint32_t e = (eb >> (8 * a)) & 0xffu;
      Rv[a] = fmaf(o[a] - p[a], asFloatHd((254u - e) << 23) * 3.0517578125e-05f, 1.0f);
    }
  }
  uint32_t hm = 0;  // slots whose box the ray meets
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int h = c >> 2, k = c & 3;
    const uint32_t sel = 0x7604u | ((uint32_t)k << 4);
    const float vnx = asFloatHd(bytePerm(qn[0 + h], 0x3F800000u, sel));
    const float vfx = asFloatHd(bytePerm(qf[0 + h], 0x3F800000u, sel));
    const float vny = asFloatHd(bytePerm(qn[2 + h], 0x3F800000u, sel));
    const float vfy = asFloatHd(bytePerm(qf[2 + h], 0x3F800000u, sel));
    const float vnz = asFloatHd(bytePerm(qn[4 + h], 0x3F800000u, sel));
    const float vfz = asFloatHd(bytePerm(qf[4 + h], 0x3F800000u, sel));
    bool in;
    if (kPlusZ) {  // oct == 0: near words are the lo words
      in = vnx <= Rv[0] + 4.76837158203125e-7f && vfx >= Rv[0] - 4.76837158203125e-7f &&
           vny <= Rv[1] + 4.76837158203125e-7f && vfy >= Rv[1] - 4.76837158203125e-7f &&
           fmaxf(fmaf(vnz, A[2], Bn[2]), tmin) <= fminf(fmaf(vfz, A[2], Bf[2]), hit.t) * 1.0000004f;
    } else {  // x and y planes as one packed FMA each for the near and far sides
      const float2 tnxy = fma2(make_float2(vnx, vny), make_float2(A[0], A[1]), make_float2(Bn[0], Bn[1]));
      const float2 tfxy = fma2(make_float2(vfx, vfy), make_float2(A[0], A[1]), make_float2(Bf[0], Bf[1]));
      const float tn = max3f(tnxy.x, tnxy.y, fmaxf(fmaf(vnz, A[2], Bn[2]), tmin));
      const float tf = min3f(tfxy.x, tfxy.y, fminf(fmaf(vfz, A[2], Bf[2]), hit.t));
      in = tn <= tf * 1.0000004f;
    }
    hm |= (in ? 1u : 0u) << c;
  }
#else
  const uint4 hd = ldRo(reinterpret_cast<const uint4*>(nd));
  uint32_t hm = 0;  // slots whose box the ray meets
  // two halves of four slots each: six float4 of planes per half keep the register footprint small
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float4 nx = ldRo(nd + nxo + h), fx = ldRo(nd + fxo + h);
    const float4 ny = ldRo(nd + nyo + h), fy = ldRo(nd + fyo + h);
    const float4 nz = ldRo(nd + nzo + h), fz = ldRo(nd + fzo + h);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = 4 * h + q;
      const float pnx = q == 0 ? nx.x : q == 1 ? nx.y : q == 2 ? nx.z : nx.w;
      const float pfx = q == 0 ? fx.x : q == 1 ? fx.y : q == 2 ? fx.z : fx.w;
      const float pny = q == 0 ? ny.x : q == 1 ? ny.y : q == 2 ? ny.z : ny.w;
      const float pfy = q == 0 ? fy.x : q == 1 ? fy.y : q == 2 ? fy.z : fy.w;
      const float pnz = q == 0 ? nz.x : q == 1 ? nz.y : q == 2 ? nz.z : nz.w;
      const float pfz = q == 0 ? fz.x : q == 1 ? fz.y : q == 2 ? fz.z : fz.w;
      bool in;
      if (kPlusZ) {  // oct == 0: near planes are the lo planes
        in = pnx <= r.o.x && r.o.x <= pfx && pny <= r.o.y && r.o.y <= pfy &&
             fmaxf(pnz - r.o.z, tmin) <= fminf(pfz - r.o.z, hit.t) * 1.0000004f;
      } else {
        const float tn = max3f(fmaf(pnx, r.invd.x, r.nAdd.x), fmaf(pny, r.invd.y, r.nAdd.y),
                               fmaxf(fmaf(pnz, r.invd.z, r.nAdd.z), tmin));
        const float tf = min3f(fmaf(pfx, r.invd.x, r.fAdd.x), fmaf(pfy, r.invd.y, r.fAdd.y),
                               fminf(fmaf(pfz, r.invd.z, r.fAdd.z), hit.t));
        in = tn <= tf * 1.0000004f;
      }
      hm |= (in ? 1u : 0u) << c;
    }
  }
#endif
  // internal hits in key order; hit leaf slots become the pending triangles (empty slots are in neither mask)
  const uint32_t imask = hd.z & 0xffu, lmask = (hd.z >> 8) & 0xffu;
  uint32_t ihits = slotsToKeys(hm & imask, oct);
  const uint32_t lhits = hm & lmask;
  if (lhits != 0u) {
    if (hd.y + (uint32_t)popc(lmask) > (uint32_t)b.numTris) {
      flagError(err, DDGI_DEVERR_BOUNDS);
      s.node = -1;
      s.sp = 0;
      s.top = make_uint2(0u, 0u);
      return;
    }
    s.tBase = hd.y;
    s.tMask = lhits | (lmask << 8);
  }
  if (ihits) {
    // descend into the nearest-keyed internal child, keep the rest of this node's hits on the stack
    const int key = lowestBit(ihits);
    ihits &= ihits - 1u;
    const uint32_t slot = (uint32_t)key ^ oct;
    const int next = (int)(hd.x + (uint32_t)popc(imask & ((1u << slot) - 1u)));
    if (ihits) {
      if (s.top.y & 0xffu) {  // the current top goes below the new one
        if (s.sp >= kWideStack) {
          flagError(err, DDGI_DEVERR_STACK_OVERFLOW);
          s.node = -1;
          s.sp = 0;
          s.top = make_uint2(0u, 0u);
          s.tMask = 0;
          return;
        }
        s.stack[s.sp++] = s.top;
      }
      s.top = make_uint2(hd.x, (imask << 8) | ihits);
    }
    s.node = next;
    return;
  }
  widePop(s);
}

template <bool kAnyHit, bool kPlusZ = false, bool kNodeScale = false>
DDGI_HD bool traverseWide(const BvhRef& b, const WRay& r, float tmin, float tmax, HitInfo& hit, uint32_t* err) {
  WideTrav s;
  if (!wideInit<kAnyHit>(b, r, tmax, s, hit))
    while (!wideStep<kAnyHit, kPlusZ, kNodeScale>(b, r, tmin, s, hit, err)) {
    }
  return hit.leaf >= 0;
}

}  // namespace ddgi
