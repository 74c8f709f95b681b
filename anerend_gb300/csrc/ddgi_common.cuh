// Shared device/host definitions of the DDGI probe engine: small vector math, the shader functions of
// the probe-update path restated for CUDA, and the internal launch records.
#pragma once

#include <stddef.h>

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include "../../include/ddgi.h"

#define DDGI_HD __host__ __device__ __forceinline__
#define DDGI_D __device__ __forceinline__

// ---- device error word bits (sticky, read and cleared by ddgi_sync) ---------------------------------
#define DDGI_DEVERR_STACK_OVERFLOW 1u
#define DDGI_DEVERR_BOUNDS 2u
#define DDGI_DEVERR_TIMEOUT 4u

namespace ddgi {

// Constants exactly as the shaders spell them.
constexpr float kPiPbr = 3.14159265359f;      // pbr_light.glsl:8
constexpr float kPiSampleProbe = 3.1415926f;  // pbr_light.glsl:362
constexpr double kGoldenRatio = 1.6180339887;  // irradiance_probe_update.rgen:13
constexpr double kPiRgen = 3.14159265359;      // irradiance_probe_update.rgen:14
constexpr float kTMin = 0.1f;                  // rgen:91, rchit:162
constexpr float kTMax = 50.0f;                 // rgen:92, rchit:163
constexpr int kOct = 8;                        // PROBE_CONV_PIX_SIZE, probe_helpers.glsl:7
constexpr int kOctTexels = kOct * kOct;
constexpr int kProbePix = kOct + 2;            // 1-texel border, IrradianceProbeConvolvePass.cpp:62-64
constexpr int kStackSize = 64;                 // traversal stack entries

// ---- float3 helpers -------------------------------------------------------------------------------
DDGI_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
DDGI_HD float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
DDGI_HD float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
DDGI_HD float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
DDGI_HD float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
DDGI_HD float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
DDGI_HD float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
DDGI_HD float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
DDGI_HD float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
DDGI_HD float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
DDGI_HD float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DDGI_HD float3 fmax3(float3 a, float s) { return f3(fmaxf(a.x, s), fmaxf(a.y, s), fmaxf(a.z, s)); }
DDGI_HD float3 fmax3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
DDGI_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
DDGI_HD float3 clamp3(float3 a, float lo, float hi) {
  return f3(clampf(a.x, lo, hi), clampf(a.y, lo, hi), clampf(a.z, lo, hi));
}
DDGI_D float3 normalize3(float3 v) {
#ifdef __CUDA_ARCH__
  float inv = rsqrtf(dot3(v, v));
#else
  float inv = 1.0f / sqrtf(dot3(v, v));  // host builds of the shared headers (CPU tests)
#endif
  return v * inv;
}
DDGI_HD float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }
DDGI_HD float get(float3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// ---- octahedral mapping (octahedron_helpers.glsl:1-34) and pixelToUv (helpers.glsl:1-4) -------------
DDGI_HD float signNotZero(float k) { return k >= 0.0f ? 1.0f : -1.0f; }

// octEncode: swap y/z, project to the L1 sphere, fold the lower half.
DDGI_HD float2 octEncode(float3 v) {
  float vx = v.x, vy = v.z, vz = v.y;
  float l1 = fabsf(vx) + fabsf(vy) + fabsf(vz);
  float rx = vx * (1.0f / l1), ry = vy * (1.0f / l1);
  if (vz < 0.0f) {
    float nx = (1.0f - fabsf(ry)) * signNotZero(rx);
    float ny = (1.0f - fabsf(rx)) * signNotZero(ry);
    rx = nx;
    ry = ny;
  }
  return make_float2(rx, ry);
}

DDGI_D float3 octDecode(float2 o) {
  float vx = o.x, vy = o.y, vz = 1.0f - fabsf(o.x) - fabsf(o.y);
  if (vz < 0.0f) {
    float nx = (1.0f - fabsf(vy)) * signNotZero(vx);
    float ny = (1.0f - fabsf(vx)) * signNotZero(vy);
    vx = nx;
    vy = ny;
  }
  return normalize3(f3(vx, vz, vy));
}

// Direction of octahedral texel (tx, ty) of an 8x8 probe (probe_conv.comp:283-286).
DDGI_D float3 texelDirection(int tx, int ty) {
  float u = (2.0f * tx + 1.0f) / (2.0f * kOct);
  float v = (2.0f * ty + 1.0f) / (2.0f * kOct);
  return octDecode(make_float2(u * 2.0f - 1.0f, v * 2.0f - 1.0f));
}

// ---- colour (bindless.glsl:240-247) ----------------------------------------------------------------
DDGI_D float toLinear1(float c) {
  return c < 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
}
DDGI_D float3 toLinear(float3 c) { return f3(toLinear1(c.x), toLinear1(c.y), toLinear1(c.z)); }

// ---- Cook-Torrance pieces (pbr_light.glsl:10-43, 88-96) ---------------------------------------------
DDGI_D float distributionGGX(float3 N, float3 H, float roughness) {
  float a = roughness * roughness;
  float a2 = a * a;
  float NdotH = fmaxf(dot3(N, H), 0.0f);
  float NdotH2 = NdotH * NdotH;
  float num = a2 + 0.001f;
  float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
  denom = kPiPbr * denom * denom;
  return num / denom;
}
DDGI_D float geometrySchlickGGX(float NdotV, float roughness) {
  float r = roughness + 1.0f;
  float k = (r * r) / 8.0f;
  return NdotV / (NdotV * (1.0f - k) + k);
}
DDGI_D float geometrySmith(float3 N, float3 V, float3 L, float roughness) {
  float NdotV = fmaxf(dot3(N, V), 0.0f);
  float NdotL = fmaxf(dot3(N, L), 0.0f);
  return geometrySchlickGGX(NdotL, roughness) * geometrySchlickGGX(NdotV, roughness);
}
DDGI_D float pow5(float x) { float x2 = x * x; return x2 * x2 * x; }
DDGI_D float3 fresnelSchlick(float cosTheta, float3 F0) {
  float p = pow5(clampf(1.0f - cosTheta, 0.0f, 1.0f));
  return F0 + (f3(1.0f, 1.0f, 1.0f) - F0) * p;
}
DDGI_D float3 fresnelSchlickRoughness(float cosTheta, float3 F0, float roughness) {
  float p = pow5(clampf(1.0f - cosTheta, 0.0f, 1.0f));
  return F0 + (fmax3(f3(1.0f - roughness, 1.0f - roughness, 1.0f - roughness), F0) - F0) * p;
}
DDGI_D float3 mixF0(float3 albedo, float metallic) {
  // mix(vec3(0.04), albedo, metallic)
  return f3(0.04f, 0.04f, 0.04f) * (1.0f - metallic) + albedo * metallic;
}

// calcLight for the directional sun with specular on (pbr_light.glsl:98-166, called from rchit:195-204).
DDGI_D float3 calcLightDirectional(float3 N, float3 albedo, float metallic, float roughness, float3 worldPos,
                                   float3 viewPos, float3 lightDir, float sunIntensity) {
  float3 V = normalize3(viewPos - worldPos);
  float3 F0 = mixF0(albedo, metallic);
  float3 L = normalize3(-lightDir);
  float3 H = normalize3(V + L);
  float3 radiance = f3(sunIntensity, sunIntensity, sunIntensity);
  float NDF = distributionGGX(N, H, roughness);
  float G = geometrySmith(N, V, L, roughness);
  float3 F = fresnelSchlick(fmaxf(dot3(H, V), 0.0f), F0);
  float3 kD = (f3(1.0f, 1.0f, 1.0f) - F) * (1.0f - metallic);
  float NdotL = fmaxf(dot3(N, L), 0.0f);
  float NdotV = fmaxf(dot3(N, V), 0.0f);
  float3 numerator = F * (NDF * G);
  float denominator = 4.0f * NdotV * NdotL + 0.0001f;
  float3 specular = clamp3(numerator / denominator, 0.0f, 1.0f);
  return (kD * albedo / kPiPbr + specular) * radiance * NdotL;
}

// ---- ray layout ---------------------------------------------------------------------------------
// Ray block of N rays: bw = 2^ceil(log2(N)/2) columns, bh = N / bw rows (16 x 16 for the reference's 256).
DDGI_HD void rayBlock(int n, int& bw, int& bh) {
  int lg = 0;
  while ((1 << lg) < n) ++lg;
  bw = 1 << ((lg + 1) / 2);
  bh = n / bw;
}

// ---- atlas and ray-image texel access -----------------------------------------------------------------
DDGI_D float4 loadTexel(const void* atlas, int fmt, size_t idx) {
  if (fmt == DDGI_FORMAT_RGBA32F) return reinterpret_cast<const float4*>(atlas)[idx];
  uint2 raw = reinterpret_cast<const uint2*>(atlas)[idx];
  __half2 a = *reinterpret_cast<__half2*>(&raw.x);
  __half2 b = *reinterpret_cast<__half2*>(&raw.y);
  float2 fa = __half22float2(a), fb = __half22float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
}
DDGI_D void storeTexel(void* atlas, int fmt, size_t idx, float4 v) {
  if (fmt == DDGI_FORMAT_RGBA32F) {
    reinterpret_cast<float4*>(atlas)[idx] = v;
    return;
  }
  __half2 a = __floats2half2_rn(v.x, v.y);
  __half2 b = __floats2half2_rn(v.z, v.w);
  uint2 raw;
  raw.x = *reinterpret_cast<uint32_t*>(&a);
  raw.y = *reinterpret_cast<uint32_t*>(&b);
  reinterpret_cast<uint2*>(atlas)[idx] = raw;
}

// ---- internal records -------------------------------------------------------------------------------
// Per-instance record on the device: object-to-world (3x4 row-major), the inverse of its 3x3 part
// (row-major), mesh, material and the first global triangle id of the instance.
struct InstanceGPU {
  float o2w[12];
  float w2oLin[9];
  uint32_t mesh, material, triOffset;
};
// hit shading reads an instance record as six float4 (o2w, w2oLin, then mesh and material in the last one)
static_assert(sizeof(InstanceGPU) == 96 && offsetof(InstanceGPU, w2oLin) == 48 && offsetof(InstanceGPU, mesh) == 84 &&
                  offsetof(InstanceGPU, material) == 88,
              "instance record layout read by reconstructHit");
static_assert(offsetof(DdgiMeshInfo, indexOffset) == offsetof(DdgiMeshInfo, vertexOffset) + 4 &&
                  offsetof(DdgiMeshInfo, vertexOffset) % 8 == 0 && sizeof(DdgiMeshInfo) % 8 == 0,
              "vertexOffset and indexOffset of a mesh record are read as one 8-byte load");

// BVH2 node in the Aila-Laine layout: child bounds packed so one node is four float4 loads.
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (child0, child1, -, -) as ints; child >= 0 internal node, child < 0 leaf ~leafIndex
// One BVH as the traversals see it (traverse.cuh). Triangles: 3 float4 per record, world v0|globalId,
// v1|instance, v2|primitive. Binary nodes: 4 float4 per internal node (Aila-Laine: both child boxes, then
// the child ids; a child id c < 0 is triangle record ~c). Wide nodes: kWideNodeF4 float4 each.
struct BvhRef {
  const float4* nodes;
  const float4* wnodes;
  const float4* tris;
  int numTris;
  int numNodes;
  int numWNodes;
};

struct SceneGPU {
  BvhRef bvh;                 // world-space triangles of every instance
  const DdgiPackedVertex* vertices;
  const uint32_t* indices;
  const DdgiMeshInfo* meshes;
  const InstanceGPU* instances;
  const DdgiMaterialInfo* materials;
  // Shading records, 3 float4 per record of `bvh` (its order): vertex k's normal times the instance's
  // WorldToObject (normal * WorldToObject, rchit:72, applied per vertex: the product is linear, so
  // interpolating afterwards gives the same direction) in .xyz, and the instance's material in .w of the
  // first. The probe-update shading reads these instead of the index / vertex / instance records.
  const float4* shade;
  // Shadow BVH in the sheared ray space of the light direction (Woop et al.'s per-ray shear, fixed for
  // every shadow ray of a frame): a shadow ray from p is the line through shear(p) along +z, so the same
  // watertight test and traversal run on it with direction (0, 0, 1). shadow.tris is null when not built.
  BvhRef shadow;
  int shearK[3];      // kx, ky, kz
  float shearS[3];    // Sx, Sy, Sz
};

struct GridGPU {
  int X, Y, Z, N, bw, bh;
  float3 step;
  float originY;
  int atlasW, atlasH, atlasFmt;
  int rayW;
  int rayFmt;      // texel format of the ray images (DDGI_FORMAT_RGBA32F or DDGI_FORMAT_RGBA16F)
  uint32_t options;
  int bvhWide;     // 1: traverse the 8-wide BVH, 0: the binary one
  int warpProbes;  // probes per warp (power of two, 32 / warpProbes <= N)
  int probeGroups;   // ceil(X Z / warpProbes): probe groups (of warpProbes probes) per layer
  uint32_t magicX, magicPG;  // divMagic(X), divMagic(probeGroups): divisions of the ray-slot mapping
  void* rad16;     // when set, the trace also writes planar 16-bit radiance (row c * pTotal + p, N per row)
  int rad16Fmt;    // 0 FP16, 1 BF16
  int pTotal;      // probes of the grid (rows per channel of rad16)
  int samplerClamp;  // atlas sampler addressing: 0 REPEAT (the trace pass), 1 CLAMP_TO_EDGE (the deferred pass)
};

// Division by an invariant d >= 1 for dividends below 2^31: with m = divMagic(d) = floor((2^32 - 1) / d),
// q = the high word of a m is floor(a / d) or one less (a m / 2^32 > a / d - a / (d 2^32) - a / 2^32 >
// a / d - 1), so one correction gives the exact quotient. Replaces the integer division of the per-ray
// slot mapping (about twenty instructions each) by four.
DDGI_HD uint32_t divMagic(uint32_t d) { return 0xFFFFFFFFu / d; }
DDGI_HD uint32_t divFast(uint32_t a, uint32_t d, uint32_t m) {
#ifdef __CUDA_ARCH__
  uint32_t q = __umulhi(a, m);
#else
  uint32_t q = (uint32_t)(((uint64_t)a * m) >> 32);
#endif
  if (a - q * d >= d) ++q;
  return q;
}

inline void setGridWarpProbes(GridGPU& g, int warpProbes) {
  g.warpProbes = warpProbes;
  g.probeGroups = (g.X * g.Z + warpProbes - 1) / warpProbes;
  g.magicPG = divMagic((uint32_t)g.probeGroups);
}

struct FrameGPU {
  float3 camPos, lightDir, skyColor;
  float3 skyLinear;  // toLinear(skyIntensity * skyColor) (rmiss:20), computed once per frame on the host
  float sunIntensity, skyIntensity;
  uint32_t flags;
  int layerBegin, layerEnd;
  int bakeTile[3];
  int camIdx[2];  // (int)(camPos.x / step.x), (int)(camPos.z / step.z) of the frame's grid (setFrameGrid)
};

// The camera's probe indices of a grid (rgen:75-83: int() of the FP32 quotient), once per frame on the host:
// IEEE division there gives the quotient the shaders' division gives.
inline void setFrameGrid(FrameGPU& f, const GridGPU& g) {
  f.camIdx[0] = (int)(f.camPos.x / g.step.x);
  f.camIdx[1] = (int)(f.camPos.z / g.step.z);
}

}  // namespace ddgi
