// Probe-ray generation, BVH traversal and hit shading: the work of irradiance_probe_update.rgen (ray
// generation, :48-111), .rchit (hit shading + shadow ray, :134-221) and .rmiss (sky / unshadowed,
// :17-21) on CUDA cores. The reference traverses with RT cores through traceRayEXT; here a stack-based
// traversal of the device-built LBVH with a watertight ray/triangle test (Woop, Benthin, Wald 2013,
// "Watertight Ray/Triangle Intersection", JCGT 2(1)) runs per thread.
//
// Thread mapping: a warp holds the same ray index j for 32 neighbouring probes of one layer. All probes
// share one direction set, so the 32 rays of a warp are parallel and start close to each other, which keeps
// traversal coherent.
#include "ddgi_common.cuh"
#include "kernels.h"

#include <climits>

namespace ddgi {

// ---------------------------------------------------------------------------------------------------
// Golden-angle lattice (worldDirFromFibonacciIndex, rgen:35-46) rotated by mat3(randomRot) (rgen:87-88),
// in FP64. rot is column-major: out_r = sum_c rot[3c + r] * d_c.
__global__ void k_lattice(int n, Mat3 rot, float4* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double theta = 2.0 * kPiRgen * (double)i / kGoldenRatio;
  double phi = acos(1.0 - 2.0 * ((double)i + 0.5) / (double)n);
  double sp = sin(phi);
  double v[3] = {cos(theta) * sp, sin(theta) * sp, cos(phi)};
  double len = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= len; v[1] /= len; v[2] /= len;
  double r[3];
  for (int row = 0; row < 3; ++row)
    r[row] = (double)rot.m[row] * v[0] + (double)rot.m[3 + row] * v[1] + (double)rot.m[6 + row] * v[2];
  out[i] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.0f);
}

// ---------------------------------------------------------------------------------------------------
// Watertight ray/triangle test.
struct WRay {
  float3 o, d, invd;
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

DDGI_D WRay makeRay(float3 o, float3 d) {
  WRay r;
  r.o = o;
  r.d = d;
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
  // box-test reciprocals; a zero component becomes a tiny same-signed value so (lo - o) * invd is finite
  float3 dd = f3(d.x != 0.f ? d.x : copysignf(1e-20f, d.x), d.y != 0.f ? d.y : copysignf(1e-20f, d.y),
                 d.z != 0.f ? d.z : copysignf(1e-20f, d.z));
  r.invd = f3(1.0f / dd.x, 1.0f / dd.y, 1.0f / dd.z);
  return r;
}

// Returns true for a hit with tmin <= t <= tmax; b1, b2 are the weights of v1, v2. Products and
// differences of the edge functions are not contracted into FMAs, so a shared edge evaluates to the same
// value (with opposite sign) from both of its triangles.
DDGI_D bool intersectTri(const WRay& r, float3 v0, float3 v1, float3 v2, float tmin, float tmax, float& t,
                         float& b1, float& b2) {
  float3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
  float Akz = get(A, r.kz), Bkz = get(B, r.kz), Ckz = get(C, r.kz);
  float Ax = __fsub_rn(get(A, r.kx), __fmul_rn(r.Sx, Akz));
  float Ay = __fsub_rn(get(A, r.ky), __fmul_rn(r.Sy, Akz));
  float Bx = __fsub_rn(get(B, r.kx), __fmul_rn(r.Sx, Bkz));
  float By = __fsub_rn(get(B, r.ky), __fmul_rn(r.Sy, Bkz));
  float Cx = __fsub_rn(get(C, r.kx), __fmul_rn(r.Sx, Ckz));
  float Cy = __fsub_rn(get(C, r.ky), __fmul_rn(r.Sy, Ckz));
  float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (U == 0.0f || V == 0.0f || W == 0.0f) {  // exact fallback of the paper
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  float det = U + V + W;
  if (det == 0.0f) return false;
  float Az = __fmul_rn(r.Sz, Akz), Bz = __fmul_rn(r.Sz, Bkz), Cz = __fmul_rn(r.Sz, Ckz);
  float T = U * Az + V * Bz + W * Cz;
  float tt = __fdiv_rn(T, det);
  if (!(tt >= tmin && tt <= tmax)) return false;
  float inv = __fdiv_rn(1.0f, det);
  t = tt;
  b1 = V * inv;
  b2 = W * inv;
  return true;
}

// Slab test with a conservative far distance (Ize 2013, "Robust BVH Ray Traversal", 1 + 2*gamma(3)).
DDGI_D bool slab(const WRay& r, float lx, float hx, float ly, float hy, float lz, float hz, float tmin,
                 float tmax, float& tnear) {
  float t0x = (lx - r.o.x) * r.invd.x, t1x = (hx - r.o.x) * r.invd.x;
  float t0y = (ly - r.o.y) * r.invd.y, t1y = (hy - r.o.y) * r.invd.y;
  float t0z = (lz - r.o.z) * r.invd.z, t1z = (hz - r.o.z) * r.invd.z;
  float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
  float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
  tnear = tn;
  return tn <= tf * 1.0000004f;
}

struct HitInfo {
  int leaf;
  int gid;
  float t, b1, b2;
};

// Closest hit (kAnyHit = false): smallest t, ties to the lowest global triangle id.
// Any hit (kAnyHit = true): returns at the first triangle with t in range.
template <bool kAnyHit>
DDGI_D bool traverse(const SceneGPU& s, const WRay& r, float tmin, float tmax, HitInfo& hit,
                     uint32_t* __restrict__ err) {
  hit.leaf = -1;
  hit.gid = INT_MAX;
  hit.t = tmax;
  if (s.numTris <= 0) return false;
  auto testLeaf = [&](int leaf) -> bool {
    float4 a = __ldg(&s.tris[3 * leaf]), b = __ldg(&s.tris[3 * leaf + 1]), c = __ldg(&s.tris[3 * leaf + 2]);
    float t, b1, b2;
    if (intersectTri(r, xyz(a), xyz(b), xyz(c), tmin, hit.t, t, b1, b2)) {
      int g = __float_as_int(a.w);
      if (kAnyHit) {
        hit.leaf = leaf; hit.gid = g; hit.t = t; hit.b1 = b1; hit.b2 = b2;
        return true;
      }
      if (t < hit.t || (t == hit.t && g < hit.gid)) {
        hit.leaf = leaf; hit.gid = g; hit.t = t; hit.b1 = b1; hit.b2 = b2;
      }
    }
    return false;
  };
  if (s.numTris == 1) {
    testLeaf(0);
    return hit.leaf >= 0;
  }
  int stack[kStackSize];
  int sp = 0;
  int node = 0;
  while (true) {
    const float4* nd = s.nodes + 4 * node;
    float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
    float tn0, tn1;
    bool h0 = slab(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, tmin, hit.t, tn0);
    bool h1 = slab(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, tmin, hit.t, tn1);
    int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
    if (h0 && c0 < 0) {
      if (testLeaf(~c0) && kAnyHit) return true;
      h0 = false;
    }
    if (h1 && c1 < 0) {
      if (testLeaf(~c1) && kAnyHit) return true;
      h1 = false;
    }
    if (h0 && h1) {
      int nearC = c0, farC = c1;
      if (tn1 < tn0) { nearC = c1; farC = c0; }
      if (sp >= kStackSize) {  // cannot happen for trees of depth <= 64; flag and stop this ray
        atomicOr(err, DDGI_DEVERR_STACK_OVERFLOW);
        break;
      }
      stack[sp++] = farC;
      node = nearC;
    } else if (h0) {
      node = c0;
    } else if (h1) {
      node = c1;
    } else {
      if (sp == 0) break;
      node = stack[--sp];
    }
  }
  return hit.leaf >= 0;
}

// ---------------------------------------------------------------------------------------------------
// Previous-frame probe lookup: sampleSingleProbe / weightProbe / sampleProbe (pbr_light.glsl:168-363).
// Bilinear filtering is done in texel space in FP32 (the reference's REPEAT + LINEAR sampler, so texel
// indices wrap around the atlas; DDGI_GRID_EDGE_CLAMP clamps the probe index instead).
DDGI_D float3 sampleSingleProbe(const GridGPU& g, const void* atlas, int ix, int iy, int iz, float3 n) {
  if (g.options & DDGI_GRID_EDGE_CLAMP) {
    ix = min(max(ix, 0), g.X - 1);
    iy = min(max(iy, 0), g.Y - 1);
    iz = min(max(iz, 0), g.Z - 1);
  }
  int sx = kProbePix * ix + 1;
  int sy = kProbePix * g.Z * iy + kProbePix * iz + 1;
  float2 o = octEncode(normalize3(n));
  float ox = (o.x + 1.0f) * 0.5f * (float)(kOct - 1);
  float oy = (o.y + 1.0f) * 0.5f * (float)(kOct - 1);
  float fx0 = floorf(ox), fy0 = floorf(oy);
  float fx = ox - fx0, fy = oy - fy0;
  int x0 = sx + (int)fx0, y0 = sy + (int)fy0;
  int x1 = x0 + 1, y1 = y0 + 1;
  x0 = ((x0 % g.atlasW) + g.atlasW) % g.atlasW;
  x1 = ((x1 % g.atlasW) + g.atlasW) % g.atlasW;
  y0 = ((y0 % g.atlasH) + g.atlasH) % g.atlasH;
  y1 = ((y1 % g.atlasH) + g.atlasH) % g.atlasH;
  float4 t00 = loadTexel(atlas, g.atlasFmt, (size_t)y0 * g.atlasW + x0);
  float4 t10 = loadTexel(atlas, g.atlasFmt, (size_t)y0 * g.atlasW + x1);
  float4 t01 = loadTexel(atlas, g.atlasFmt, (size_t)y1 * g.atlasW + x0);
  float4 t11 = loadTexel(atlas, g.atlasFmt, (size_t)y1 * g.atlasW + x1);
  float w00 = (1.0f - fx) * (1.0f - fy), w10 = fx * (1.0f - fy), w01 = (1.0f - fx) * fy, w11 = fx * fy;
  return xyz(t00) * w00 + xyz(t10) * w10 + xyz(t01) * w01 + xyz(t11) * w11;
}

DDGI_D void probeFrame(const GridGPU& g, const FrameGPU& f, float3& stepv, float3& offv) {
  if (f.flags & DDGI_UBO_BAKE_MODE_ON_FLAG) {
    // bake-tile grid (rgen:61-73, pbr_light.glsl:276-293)
    float tSize = (float)f.bakeTile[2];
    stepv = f3(tSize / (float)g.X, 1.0f, tSize / (float)g.Z);
    offv = f3((float)f.bakeTile[0] * tSize, g.originY, (float)f.bakeTile[1] * tSize);
  } else {
    // camera-relative grid, int() truncation of the camera probe index (rgen:75-83, pbr_light.glsl:294-308)
    int camX = (int)(f.camPos.x / g.step.x);
    int camZ = (int)(f.camPos.z / g.step.z);
    stepv = g.step;
    offv = f3((float)camX * g.step.x - g.step.x * (float)g.X / 2.0f, g.originY,
              (float)camZ * g.step.z - g.step.z * (float)g.Z / 2.0f);
  }
}

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
  float sumW = 0.0f;
  float3 sumI = f3(0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    int ox = corners[k][0], oy = corners[k][1], oz = corners[k][2];
    float3 probePos = base + f3((float)ox, (float)oy, (float)oz) * stepv;
    float3 tri = f3(ox ? alpha.x : 1.0f - alpha.x, oy ? alpha.y : 1.0f - alpha.y, oz ? alpha.z : 1.0f - alpha.z);
    float3 dirToProbe = normalize3(probePos - wp);
    float c = fmaxf(0.0001f, (dot3(dirToProbe, n) + 1.0f) * 0.5f);
    float w = c * c + 0.2f;
    w = fmaxf(0.000001f, w);
    if (w < 0.2f) w *= w * w * (1.0f / (0.2f * 0.2f));
    w *= tri.x * tri.y * tri.z;
    float3 irr = sampleSingleProbe(g, atlas, px + ox, py + oy, pz + oz, n);
    irr = f3(sqrtf(irr.x), sqrtf(irr.y), sqrtf(irr.z));
    sumI += irr * w;
    sumW += w;
  }
  float3 net = sumI / sumW;
  net = net * net;
  return net * 0.5f * kPiSampleProbe;
}

// calcIndirectDiffuseLight (pbr_light.glsl:365-388)
DDGI_D float3 calcIndirectDiffuse(const GridGPU& g, const FrameGPU& f, const void* atlas, float3 n,
                                  float3 albedo, float metallic, float roughness, float3 wp, float3 viewPos) {
  float3 V = normalize3(viewPos - wp);
  float3 F0 = mixF0(albedo, metallic);
  float3 kS = fresnelSchlickRoughness(fmaxf(dot3(n, V), 0.0f), F0, roughness * roughness);
  float3 kD = (f3(1.f, 1.f, 1.f) - kS) * (1.0f - metallic);
  float3 irr = sampleProbe(g, f, atlas, wp, n);
  return kD * (irr * albedo);
}

// ---------------------------------------------------------------------------------------------------
// Warp shape: a warp traces D = 32 / warpProbes directions for each of warpProbes consecutive probes of a
// layer; consecutive direction slots k map to lattice rays j = order[k]. With the octahedral Morton order
// the D directions of a warp are neighbours on the sphere, so the warp's rays share traversal paths near
// their common origin.
#ifndef DDGI_TRACE_MIN_BLOCKS
#define DDGI_TRACE_MIN_BLOCKS 8
#endif
// One warp of probe rays (warp index `warp` of the grid's trace, lanes past the grid's rays idle).
DDGI_D void traceWarp(const SceneGPU& s, const GridGPU& g, const FrameGPU& f, const float4* __restrict__ lattice,
                      const int* __restrict__ order, const void* __restrict__ atlasPrev,
                      float4* __restrict__ rayRad, float4* __restrict__ rayDir, int* __restrict__ rayHit,
                      uint32_t* __restrict__ err, long long warp, int lane) {
  const int D = 32 / g.warpProbes;                // directions per warp
  const int dirChunks = g.N / D;
  const int probeGroups = (g.X * g.Z + g.warpProbes - 1) / g.warpProbes;
  int dc = (int)(warp % dirChunks);
  long long rest = warp / dirChunks;
  int pg = (int)(rest % probeGroups);
  int layer = f.layerBegin + (int)(rest / probeGroups);
  if (layer >= f.layerEnd) return;
  int p = pg * g.warpProbes + lane / D;
  if (p >= g.X * g.Z) return;
  int j = __ldg(&order[dc * D + lane % D]);
  int px = p % g.X, pz = p / g.X;

  // ray generation (rgen:51-88)
  float3 stepv, offv;
  probeFrame(g, f, stepv, offv);
  float3 origin = f3((float)px, (float)layer, (float)pz) * stepv + offv;
  float4 d4 = __ldg(&lattice[j]);
  float3 dir = xyz(d4);

  WRay ray = makeRay(origin, dir);
  HitInfo hit;
  float3 L;
  int hitCode = -1;
  if (!traverse<false>(s, ray, kTMin, kTMax, hit, err)) {
    L = toLinear(f.skyColor * f.skyIntensity);  // rmiss:20
  } else {
    // hit reconstruction (rchit:137-152)
    int inst = __float_as_int(__ldg(&s.tris[3 * hit.leaf + 1].w));
    int prim = __float_as_int(__ldg(&s.tris[3 * hit.leaf + 2].w));
    const InstanceGPU& in = s.instances[inst];
    const DdgiMeshInfo& mesh = s.meshes[in.mesh];
    uint32_t ib = mesh.indexOffset + 3u * (uint32_t)prim;
    const DdgiPackedVertex* vb = s.vertices + mesh.vertexOffset;
    const DdgiPackedVertex& v0 = vb[__ldg(&s.indices[ib])];
    const DdgiPackedVertex& v1 = vb[__ldg(&s.indices[ib + 1])];
    const DdgiPackedVertex& v2 = vb[__ldg(&s.indices[ib + 2])];
    float b1 = hit.b1, b2 = hit.b2, b0 = 1.0f - b1 - b2;
    float4 a0 = __ldg((const float4*)v0.d0), a1 = __ldg((const float4*)v1.d0), a2 = __ldg((const float4*)v2.d0);
    float4 c0 = __ldg((const float4*)v0.d1), c1 = __ldg((const float4*)v1.d1), c2 = __ldg((const float4*)v2.d1);
    float4 e0 = __ldg((const float4*)v0.d2), e1 = __ldg((const float4*)v1.d2), e2 = __ldg((const float4*)v2.d2);
    float3 posObj = xyz(a0) * b0 + xyz(a1) * b1 + xyz(a2) * b2;
    const float* m = in.o2w;
    float3 pos = f3(m[0] * posObj.x + m[1] * posObj.y + m[2] * posObj.z + m[3],
                    m[4] * posObj.x + m[5] * posObj.y + m[6] * posObj.z + m[7],
                    m[8] * posObj.x + m[9] * posObj.y + m[10] * posObj.z + m[11]);

    // shadow ray toward the sun (rchit:155-176), any hit in [0.1, 50]
    bool shadowed;
    HitInfo shit;
    if (s.shadowNodes) {
      // the light's sheared space: the ray is the +z line through shear(pos)
      float pk[3] = {pos.x, pos.y, pos.z};
      float pz = pk[s.shearK[2]];
      float3 o = f3(pk[s.shearK[0]] - s.shearS[0] * pz, pk[s.shearK[1]] - s.shearS[1] * pz, s.shearS[2] * pz);
      SceneGPU ls = s;
      ls.nodes = s.shadowNodes;
      ls.tris = s.shadowTris;
      shadowed = traverse<true>(ls, makeRay(o, f3(0.f, 0.f, 1.f)), kTMin, kTMax, shit, err);
    } else {
      float3 shadowDir = normalize3(-f.lightDir);
      shadowed = traverse<true>(s, makeRay(pos, shadowDir), kTMin, kTMax, shit, err);
    }

    // surface (rchit:179-187, getSurfaceDataFromMat bindless.glsl:181-237 without textures)
    const DdgiMaterialInfo& mat = s.materials[in.material];
    float3 nObj = f3(c0.z, c0.w, e0.x) * b0 + f3(c1.z, c1.w, e1.x) * b1 + f3(c2.z, c2.w, e2.x) * b2;
    nObj = normalize3(nObj);
    const float* wi = in.w2oLin;  // normal * WorldToObject (row vector times the inverse 3x3)
    float3 normal = normalize3(f3(nObj.x * wi[0] + nObj.y * wi[3] + nObj.z * wi[6],
                                  nObj.x * wi[1] + nObj.y * wi[4] + nObj.z * wi[7],
                                  nObj.x * wi[2] + nObj.y * wi[5] + nObj.z * wi[8]));
    float3 vcol = f3(a0.w, c0.x, c0.y) * b0 + f3(a1.w, c1.x, c1.y) * b1 + f3(a2.w, c2.x, c2.y) * b2;
    float3 color = toLinear(vcol);
    float4 bcf = __ldg((const float4*)mat.baseColFac);
    if (bcf.x + bcf.y + bcf.z > 0.1f) color = xyz(bcf);
    float4 mr = __ldg((const float4*)mat.metRough);
    float4 em = __ldg((const float4*)mat.emissive);
    float metallic = mr.x, roughness = mr.y;

    L = f3(0.f, 0.f, 0.f);
    if (!shadowed)
      L = calcLightDirectional(normal, color, metallic, roughness, pos, origin, f.lightDir, f.sunIntensity);
    if (f.flags & DDGI_UBO_DDGI_MULTI_FLAG)
      L += calcIndirectDiffuse(g, f, atlasPrev, normal, color, metallic, roughness, pos, origin);
    L += xyz(em) * em.w;
    hitCode = hit.gid * 2 + (shadowed ? 1 : 0);
  }

  // stores (rgen:108-109)
  int rx = px * g.bw + (j % g.bw);
  int ry = (layer * g.Z + pz) * g.bh + (j / g.bw);
  size_t idx = (size_t)ry * g.rayW + rx;
  rayRad[idx] = make_float4(L.x, L.y, L.z, 1.0f);
  if (rayDir) rayDir[idx] = make_float4(dir.x, dir.y, dir.z, 1.0f);
  if (rayHit) rayHit[idx] = hitCode;
  if (g.rad16) {  // operand of the tensor-core convolution
    size_t base = ((size_t)(layer * g.Z + pz) * g.X + px) * g.N + j;
    size_t plane = (size_t)g.pTotal * g.N;
    uint16_t* o = (uint16_t*)g.rad16;
    float c[3] = {L.x, L.y, L.z};
#pragma unroll
    for (int k = 0; k < 3; ++k)
      o[base + k * plane] = g.rad16Fmt == 0 ? __half_as_ushort(__float2half_rn(c[k]))
                                            : __bfloat16_as_ushort(__float2bfloat16_rn(c[k]));
  }
}

// Persistent trace over many grids: warps take `warpsPerFetch` warps of work at a time from one queue that
// spans every item's rays (item i owns warps [warpBegin_i, warpBegin_i + numWarps_i)).
__global__ void __launch_bounds__(kTraceThreads, DDGI_TRACE_MIN_BLOCKS)
    k_trace_batch(const TraceItem* __restrict__ items, int numItems, long long totalWarps,
                  unsigned long long* __restrict__ queue, int warpsPerFetch, uint32_t* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  while (true) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(queue, (unsigned long long)warpsPerFetch);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((long long)base >= totalWarps) break;
    for (int k = 0; k < warpsPerFetch; ++k) {
      long long w = (long long)base + k;
      if (w >= totalWarps) break;
      int lo = 0, hi = numItems - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (items[mid].warpBegin <= w) lo = mid; else hi = mid - 1;
      }
      const TraceItem& it = items[lo];
      traceWarp(it.s, it.g, it.f, it.lattice, it.order, it.atlasPrev, it.rayRad, it.rayDir, it.rayHit, err,
                w - it.warpBegin, lane);
      __syncwarp();
    }
  }
}

// Rotated lattices of many grids: one block row per item.
__global__ void k_lattice_batch(const TraceItem* __restrict__ items, const Mat3* __restrict__ rots) {
  const TraceItem& it = items[blockIdx.y];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= it.g.N) return;
  double theta = 2.0 * kPiRgen * (double)i / kGoldenRatio;
  double phi = acos(1.0 - 2.0 * ((double)i + 0.5) / (double)it.g.N);
  double sp = sin(phi);
  double v[3] = {cos(theta) * sp, sin(theta) * sp, cos(phi)};
  double len = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= len; v[1] /= len; v[2] /= len;
  const float* m = rots[blockIdx.y].m;
  double r[3];
  for (int row = 0; row < 3; ++row)
    r[row] = (double)m[row] * v[0] + (double)m[3 + row] * v[1] + (double)m[6 + row] * v[2];
  const_cast<float4*>(it.lattice)[i] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.0f);
}

// ---------------------------------------------------------------------------------------------------
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

cudaError_t launchTraceBatch(const TraceItem* dItems, const Mat3* dRots, int numItems, int maxN, long long totalWarps,
                             unsigned long long* dQueue, int blocks, int warpsPerFetch, uint32_t* err,
                             cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(dQueue, 0, sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  dim3 lg((maxN + 127) / 128, numItems);
  k_lattice_batch<<<lg, 128, 0, stream>>>(dItems, dRots);
  if (totalWarps > 0)
    k_trace_batch<<<blocks, kTraceThreads, 0, stream>>>(dItems, numItems, totalWarps, dQueue, warpsPerFetch, err);
  return cudaGetLastError();
}

}  // namespace ddgi
