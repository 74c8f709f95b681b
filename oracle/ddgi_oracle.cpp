// ORACLE — test infrastructure only, never part of the product path.
//
// FP64 CPU restatement of AneRend's DDGI probe update, the parity reference of the tests and the
// benchmark's timed CPU baseline. Each function names the reference lines it follows:
//   ray generation      assets/shaders/irradiance_probe_update.rgen:35-111
//   hit shading         assets/shaders/irradiance_probe_update.rchit:134-221, .rmiss:17-21
//   lighting / lookup   assets/shaders/pbr_light.glsl:10-43, 88-166, 168-388
//   surface / colour    assets/shaders/bindless.glsl:98-109, 181-247
//   octahedral mapping  assets/shaders/octahedron_helpers.glsl:1-34, helpers.glsl:1-4
//   convolution         assets/shaders/probe_conv.comp:21-90
//   translation         src/anerend/render/passes/IrradianceProbeTranslationPass.cpp:56-186
// The reference traverses with the Vulkan driver's closed BVH and RT hardware; here a ray hits the closest
// triangle by an exact FP64 watertight test (Woop, Benthin, Wald 2013), ties to the lowest global
// triangle id, and every ray carries an "uncertain" flag when an FP32 implementation could legitimately
// decide differently (hit within an edge epsilon, near-tie in t, t near the range ends, shadow occluder
// near an edge). The hardware sampler's fixed-point bilinear weights are replaced by exact weights.
//
// Pinning: the reference publishes no tests or golden data, and its GLSL cannot run here (Vulkan, no graphics
// stack). The restatement is pinned against the reference shader sources compiled as FP64 C++ (oracle/ref_shader)
// on the reference's own grid constants, and by known-answer tests.
#include "../include/ddgi.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct d3 {
  double x, y, z;
};
inline d3 D3(double x, double y, double z) { return d3{x, y, z}; }
inline d3 operator+(d3 a, d3 b) { return D3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline d3 operator-(d3 a, d3 b) { return D3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline d3 operator*(d3 a, d3 b) { return D3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline d3 operator/(d3 a, d3 b) { return D3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline d3 operator*(d3 a, double s) { return D3(a.x * s, a.y * s, a.z * s); }
inline d3 operator/(d3 a, double s) { return D3(a.x / s, a.y / s, a.z / s); }
inline d3 operator-(d3 a) { return D3(-a.x, -a.y, -a.z); }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline d3 normalize(d3 v) { return v / std::sqrt(dot(v, v)); }
inline double comp(d3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
inline double clampd(double x, double lo, double hi) { return std::min(std::max(x, lo), hi); }
inline d3 clamp3(d3 v, double lo, double hi) { return D3(clampd(v.x, lo, hi), clampd(v.y, lo, hi), clampd(v.z, lo, hi)); }
inline d3 max3(d3 a, d3 b) { return D3(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)); }

constexpr double kPi = 3.14159265359;          // pbr_light.glsl:8, rgen:14
constexpr double kPiSample = 3.1415926;        // pbr_light.glsl:362
constexpr double kGolden = 1.6180339887;       // rgen:13
constexpr double kTMin = 0.1, kTMax = 50.0;    // rgen:91-92, rchit:162-163
constexpr int kOct = 8, kPix = 10;

// uncertainty margins (FP32 implementations stay well inside these)
constexpr double kEpsBary = 1e-4;   // barycentric distance to an edge
constexpr double kEpsT = 1e-4;      // absolute t margin at the range ends and for near-ties
constexpr double kEpsTRel = 2e-5;   // relative t margin for near-ties

// ---- octahedral helpers (octahedron_helpers.glsl) ---------------------------------------------------
inline double signNotZero(double k) { return k >= 0.0 ? 1.0 : -1.0; }
void octEncode(d3 v, double& ox, double& oy) {  // :10-20
  double vx = v.x, vy = v.z, vz = v.y;
  double l1 = std::fabs(vx) + std::fabs(vy) + std::fabs(vz);
  double rx = vx / l1, ry = vy / l1;
  if (vz < 0.0) {
    double nx = (1.0 - std::fabs(ry)) * signNotZero(rx);
    double ny = (1.0 - std::fabs(rx)) * signNotZero(ry);
    rx = nx;
    ry = ny;
  }
  ox = rx;
  oy = ry;
}
d3 octDecode(double ox, double oy) {  // :25-34
  double vx = ox, vy = oy, vz = 1.0 - std::fabs(ox) - std::fabs(oy);
  if (vz < 0.0) {
    double nx = (1.0 - std::fabs(vy)) * signNotZero(vx);
    double ny = (1.0 - std::fabs(vx)) * signNotZero(vy);
    vx = nx;
    vy = ny;
  }
  return normalize(D3(vx, vz, vy));
}
d3 texelDir(int tx, int ty) {  // probe_conv.comp:283-286 with pixelToUv (helpers.glsl:1-4)
  double u = (2.0 * tx + 1.0) / (2.0 * kOct), v = (2.0 * ty + 1.0) / (2.0 * kOct);
  return octDecode(u * 2.0 - 1.0, v * 2.0 - 1.0);
}

// ---- colour and BRDF -------------------------------------------------------------------------------
double toLinear1(double c) { return c < 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4); }  // bindless.glsl:240-247
d3 toLinear(d3 c) { return D3(toLinear1(c.x), toLinear1(c.y), toLinear1(c.z)); }
double distributionGGX(d3 N, d3 H, double r) {  // pbr_light.glsl:10-22
  double a = r * r, a2 = a * a;
  double NdotH = std::max(dot(N, H), 0.0);
  double denom = NdotH * NdotH * (a2 - 1.0) + 1.0;
  return (a2 + 0.001) / (kPi * denom * denom);
}
double schlickGGX(double NdotV, double r) {  // :24-33
  double k = (r + 1.0) * (r + 1.0) / 8.0;
  return NdotV / (NdotV * (1.0 - k) + k);
}
double geometrySmith(d3 N, d3 V, d3 L, double r) {  // :35-43
  return schlickGGX(std::max(dot(N, L), 0.0), r) * schlickGGX(std::max(dot(N, V), 0.0), r);
}
d3 fresnelSchlick(double c, d3 F0) {  // :88-91
  double p = std::pow(clampd(1.0 - c, 0.0, 1.0), 5.0);
  return F0 + (D3(1, 1, 1) - F0) * p;
}
d3 fresnelSchlickRoughness(double c, d3 F0, double r) {  // :93-96
  double p = std::pow(clampd(1.0 - c, 0.0, 1.0), 5.0);
  return F0 + (max3(D3(1.0 - r, 1.0 - r, 1.0 - r), F0) - F0) * p;
}
d3 mixF0(d3 albedo, double metallic) { return D3(0.04, 0.04, 0.04) * (1.0 - metallic) + albedo * metallic; }

d3 calcLight(d3 N, d3 albedo, double metallic, double rough, d3 wp, d3 viewPos, d3 lightDir, double sun) {  // :98-166
  d3 V = normalize(viewPos - wp);
  d3 F0 = mixF0(albedo, metallic);
  d3 L = normalize(-lightDir);
  d3 H = normalize(V + L);
  d3 radiance = D3(sun, sun, sun);
  double NDF = distributionGGX(N, H, rough);
  double G = geometrySmith(N, V, L, rough);
  d3 F = fresnelSchlick(std::max(dot(H, V), 0.0), F0);
  d3 kD = (D3(1, 1, 1) - F) * (1.0 - metallic);
  double NdotL = std::max(dot(N, L), 0.0), NdotV = std::max(dot(N, V), 0.0);
  d3 spec = clamp3(F * (NDF * G) / (4.0 * NdotV * NdotL + 0.0001), 0.0, 1.0);
  return (kD * albedo / kPi + spec) * radiance * NdotL;
}

// ---- scene and BVH ---------------------------------------------------------------------------------
struct Tri {
  d3 v[3];
  int inst, prim, gid;
};
struct Node {
  d3 lo, hi;
  int left, right;  // internal: children; leaf: left = first tri, right = -count
};

struct OracleScene {
  std::vector<Tri> tris;
  std::vector<Node> nodes;
  std::vector<DdgiPackedVertex> verts;
  std::vector<uint32_t> indices;
  std::vector<DdgiMeshInfo> meshes;
  std::vector<DdgiInstance> insts;
  std::vector<DdgiMaterialInfo> mats;
  std::vector<double> w2o;  // 9 per instance: inverse of the 3x3 part, row-major
  std::vector<uint32_t> triOffset;
};

d3 xform(const float* m, d3 p) {
  return D3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}

int buildNode(OracleScene& s, std::vector<int>& idx, int b, int e, std::vector<Tri>& out) {
  Node n;
  n.lo = D3(1e300, 1e300, 1e300);
  n.hi = D3(-1e300, -1e300, -1e300);
  d3 clo = n.lo, chi = n.hi;
  for (int i = b; i < e; ++i) {
    const Tri& t = s.tris[idx[i]];
    d3 c = D3(0, 0, 0);
    for (int k = 0; k < 3; ++k) {
      n.lo = D3(std::min(n.lo.x, t.v[k].x), std::min(n.lo.y, t.v[k].y), std::min(n.lo.z, t.v[k].z));
      n.hi = D3(std::max(n.hi.x, t.v[k].x), std::max(n.hi.y, t.v[k].y), std::max(n.hi.z, t.v[k].z));
      c = c + t.v[k];
    }
    c = c / 3.0;
    clo = D3(std::min(clo.x, c.x), std::min(clo.y, c.y), std::min(clo.z, c.z));
    chi = D3(std::max(chi.x, c.x), std::max(chi.y, c.y), std::max(chi.z, c.z));
  }
  int me = (int)s.nodes.size();
  s.nodes.push_back(n);
  if (e - b <= 4) {
    s.nodes[me].left = (int)out.size();
    s.nodes[me].right = -(e - b);
    for (int i = b; i < e; ++i) out.push_back(s.tris[idx[i]]);
    return me;
  }
  d3 ext = chi - clo;
  int axis = ext.x >= ext.y && ext.x >= ext.z ? 0 : (ext.y >= ext.z ? 1 : 2);
  int mid = (b + e) / 2;
  std::nth_element(idx.begin() + b, idx.begin() + mid, idx.begin() + e, [&](int a, int c) {
    const Tri &ta = s.tris[a], &tc = s.tris[c];
    double ca = comp(ta.v[0], axis) + comp(ta.v[1], axis) + comp(ta.v[2], axis);
    double cc = comp(tc.v[0], axis) + comp(tc.v[1], axis) + comp(tc.v[2], axis);
    return ca < cc || (ca == cc && a < c);
  });
  int l = buildNode(s, idx, b, mid, out);
  int r = buildNode(s, idx, mid, e, out);
  s.nodes[me].left = l;
  s.nodes[me].right = r;
  return me;
}

// ---- exact FP64 watertight test, returning signed barycentrics (no acceptance) ----------------------
struct RayPre {
  d3 o, d, inv;
  int kx, ky, kz;
  double Sx, Sy, Sz;
};
RayPre prep(d3 o, d3 d) {
  RayPre r;
  r.o = o;
  r.d = d;
  double ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
  if (comp(d, kz) < 0.0) std::swap(kx, ky);
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.Sx = comp(d, kx) / comp(d, kz);
  r.Sy = comp(d, ky) / comp(d, kz);
  r.Sz = 1.0 / comp(d, kz);
  r.inv = D3(1.0 / (d.x != 0 ? d.x : 1e-300), 1.0 / (d.y != 0 ? d.y : 1e-300), 1.0 / (d.z != 0 ? d.z : 1e-300));
  return r;
}
// Returns false when the triangle is degenerate for this ray; otherwise t and barycentrics (b0,b1,b2)
// of the ray's intersection with the triangle's plane (any sign).
bool planeHit(const RayPre& r, const Tri& tr, double& t, double& b0, double& b1, double& b2) {
  d3 A = tr.v[0] - r.o, B = tr.v[1] - r.o, C = tr.v[2] - r.o;
  double Ax = comp(A, r.kx) - r.Sx * comp(A, r.kz), Ay = comp(A, r.ky) - r.Sy * comp(A, r.kz);
  double Bx = comp(B, r.kx) - r.Sx * comp(B, r.kz), By = comp(B, r.ky) - r.Sy * comp(B, r.kz);
  double Cx = comp(C, r.kx) - r.Sx * comp(C, r.kz), Cy = comp(C, r.ky) - r.Sy * comp(C, r.kz);
  double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  double det = U + V + W;
  if (det == 0.0) return false;
  double T = U * r.Sz * comp(A, r.kz) + V * r.Sz * comp(B, r.kz) + W * r.Sz * comp(C, r.kz);
  t = T / det;
  b0 = U / det;
  b1 = V / det;
  b2 = W / det;
  return true;
}
bool boxHit(const RayPre& r, const Node& n, double tmin, double tmax, double pad) {
  double t0x = (n.lo.x - pad - r.o.x) * r.inv.x, t1x = (n.hi.x + pad - r.o.x) * r.inv.x;
  double t0y = (n.lo.y - pad - r.o.y) * r.inv.y, t1y = (n.hi.y + pad - r.o.y) * r.inv.y;
  double t0z = (n.lo.z - pad - r.o.z) * r.inv.z, t1z = (n.hi.z + pad - r.o.z) * r.inv.z;
  double tn = std::max(std::max(std::min(t0x, t1x), std::min(t0y, t1y)), std::max(std::min(t0z, t1z), tmin));
  double tf = std::min(std::min(std::max(t0x, t1x), std::max(t0y, t1y)), std::min(std::max(t0z, t1z), tmax));
  return tn <= tf;
}

struct Query {
  // closest exact hit
  int gid = -1, inst = -1, prim = -1;
  double t = 1e300, b1 = 0, b2 = 0, bmin = 0;
  // uncertainty bookkeeping
  double tFuzzyMin = 1e300;   // smallest t of a candidate that is fuzzy-but-not-robust
  double tSecond = 1e300;     // second-smallest t among exact hits of other triangles
  bool anyRobust = false;
};

// Visits every triangle in a box the ray crosses within [tmin - eps, tmax + eps]; the callback may lower
// tmax (closest-hit queries) and returns true to stop.
template <class F>
void visit(const OracleScene& s, const RayPre& r, double tmin, double& tmax, F&& f) {
  if (s.nodes.empty()) return;
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const Node& n = s.nodes[stack[--sp]];
    if (!boxHit(r, n, tmin - kEpsT, tmax + kEpsT, 1e-6)) continue;
    if (n.right < 0) {
      for (int i = 0; i < -n.right; ++i)
        if (f(s.tris[n.left + i])) return;
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.right;
    }
  }
}

void closestHit(const OracleScene& s, d3 o, d3 d, Query& q) {
  RayPre r = prep(o, d);
  double tmax = kTMax;
  visit(s, r, kTMin, tmax, [&](const Tri& tr) {
    double t, b0, b1, b2;
    if (!planeHit(r, tr, t, b0, b1, b2)) return false;
    double bmin = std::min(b0, std::min(b1, b2));
    bool exact = bmin >= 0.0 && t >= kTMin && t <= kTMax;
    bool robust = bmin > kEpsBary && t > kTMin + kEpsT && t < kTMax - kEpsT;
    bool fuzzy = bmin > -kEpsBary && t > kTMin - kEpsT && t < kTMax + kEpsT;
    if (robust) q.anyRobust = true;
    if (fuzzy && !robust) q.tFuzzyMin = std::min(q.tFuzzyMin, t);
    if (exact) {
      if (t < q.t || (t == q.t && tr.gid < q.gid)) {
        if (q.gid >= 0) q.tSecond = std::min(q.tSecond, q.t);
        q.t = t; q.gid = tr.gid; q.inst = tr.inst; q.prim = tr.prim; q.b1 = b1; q.b2 = b2; q.bmin = bmin;
        tmax = std::min(tmax, q.t * (1.0 + kEpsTRel) + kEpsT);
      } else {
        q.tSecond = std::min(q.tSecond, t);
      }
    }
    return false;
  });
}

// Any-hit in [0.1, 50]: returns occlusion and whether an FP32 test could disagree.
bool anyHit(const OracleScene& s, d3 o, d3 d, bool& uncertain) {
  RayPre r = prep(o, d);
  bool robust = false, fuzzyOnly = false;
  double tmax = kTMax;
  visit(s, r, kTMin, tmax, [&](const Tri& tr) {
    double t, b0, b1, b2;
    if (!planeHit(r, tr, t, b0, b1, b2)) return false;
    double bmin = std::min(b0, std::min(b1, b2));
    if (bmin > kEpsBary && t > kTMin + kEpsT && t < kTMax - kEpsT) { robust = true; return true; }
    if (bmin > -kEpsBary && t > kTMin - kEpsT && t < kTMax + kEpsT) fuzzyOnly = true;
    return false;
  });
  if (robust) { uncertain = false; return true; }
  uncertain = fuzzyOnly;
  if (!fuzzyOnly) return false;
  // exact decision for the reported value
  bool exact = false;
  tmax = kTMax;
  visit(s, r, kTMin, tmax, [&](const Tri& tr) {
    double t, b0, b1, b2;
    if (!planeHit(r, tr, t, b0, b1, b2)) return false;
    if (std::min(b0, std::min(b1, b2)) >= 0.0 && t >= kTMin && t <= kTMax) { exact = true; return true; }
    return false;
  });
  return exact;
}

// ---- grid ----------------------------------------------------------------------------------------
struct Grid {
  int X, Y, Z, N, bw, bh, atlasW, atlasH, rayW;
  d3 step;
  double originY;
  uint32_t options;
  bool clampToEdge = false;  // atlas sampler addressing: REPEAT (trace pass) or CLAMP_TO_EDGE (deferred pass)
};
Grid makeGrid(const DdgiGridDesc* d) {
  Grid g;
  g.X = d->dims[0]; g.Y = d->dims[1]; g.Z = d->dims[2];
  g.N = d->raysPerProbe;
  int lg = 0;
  while ((1 << lg) < g.N) ++lg;
  g.bw = 1 << ((lg + 1) / 2);
  g.bh = g.N / g.bw;
  g.atlasW = kPix * g.X;
  g.atlasH = kPix * g.Z * g.Y;
  g.rayW = g.bw * g.X;
  g.step = D3(d->step[0], d->step[1], d->step[2]);
  g.originY = d->originY;
  g.options = d->options;
  return g;
}

// grid frame of the probes: camera-relative (rgen:75-83) or bake tile (rgen:61-73)
void probeFrame(const Grid& g, const DdgiFrame* f, d3& stepv, d3& offv) {
  if (f->flags & DDGI_UBO_BAKE_MODE_ON_FLAG) {
    double t = f->bakeTileInfo[2];
    stepv = D3(t / g.X, 1.0, t / g.Z);
    offv = D3(f->bakeTileInfo[0] * t, g.originY, f->bakeTileInfo[1] * t);
  } else {
    // int() truncation of the FP32 quotient, as the shader computes it
    int cx = (int)(f->cameraPos[0] / (float)g.step.x), cz = (int)(f->cameraPos[2] / (float)g.step.z);
    stepv = g.step;
    offv = D3(cx * g.step.x - g.step.x * g.X / 2.0, g.originY, cz * g.step.z - g.step.z * g.Z / 2.0);
  }
}

// sampleSingleProbe (pbr_light.glsl:168-188) with exact bilinear weights; REPEAT addressing, or
// CLAMP_TO_EDGE for the deferred pass (DeferredLightingRenderPass.cpp:192-199)
d3 sampleSingleProbe(const Grid& g, const double* atlas, int ix, int iy, int iz, d3 n) {
  if (g.options & DDGI_GRID_EDGE_CLAMP) {
    ix = std::min(std::max(ix, 0), g.X - 1);
    iy = std::min(std::max(iy, 0), g.Y - 1);
    iz = std::min(std::max(iz, 0), g.Z - 1);
  }
  int sx = kPix * ix + 1, sy = kPix * g.Z * iy + kPix * iz + 1;
  double ox, oy;
  octEncode(normalize(n), ox, oy);
  double tx = (ox + 1.0) * 0.5 * (kOct - 1), ty = (oy + 1.0) * 0.5 * (kOct - 1);
  double fx0 = std::floor(tx), fy0 = std::floor(ty);
  double fx = tx - fx0, fy = ty - fy0;
  int x0 = sx + (int)fx0, y0 = sy + (int)fy0;
  const bool clampEdge = g.clampToEdge;
  auto wrap = [clampEdge](int v, int m) { return clampEdge ? std::min(std::max(v, 0), m - 1) : ((v % m) + m) % m; };
  int xs[2] = {wrap(x0, g.atlasW), wrap(x0 + 1, g.atlasW)};
  int ys[2] = {wrap(y0, g.atlasH), wrap(y0 + 1, g.atlasH)};
  double wx[2] = {1.0 - fx, fx}, wy[2] = {1.0 - fy, fy};
  d3 r = D3(0, 0, 0);
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const double* t = atlas + 4 * ((size_t)ys[b] * g.atlasW + xs[a]);
      r = r + D3(t[0], t[1], t[2]) * (wx[a] * wy[b]);
    }
  return r;
}

d3 sampleProbe(const Grid& g, const DdgiFrame* f, const double* atlas, d3 wp, d3 n) {  // :240-363
  d3 stepv, offv;
  probeFrame(g, f, stepv, offv);
  int px = std::min(std::max((int)std::floor((wp.x - offv.x) / stepv.x), 0), g.X - 1);
  int py = std::min(std::max((int)std::floor((wp.y - offv.y) / stepv.y), 0), g.Y - 1);
  int pz = std::min(std::max((int)std::floor((wp.z - offv.z) / stepv.z), 0), g.Z - 1);
  d3 base = D3(px, py, pz) * stepv + offv;
  d3 alpha = clamp3((wp - base) / stepv, 0.0, 1.0);
  static const int corners[8][3] = {{0, 0, 0}, {1, 1, 1}, {1, 1, 0}, {1, 0, 0}, {0, 1, 1}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}};
  double sumW = 0.0;
  d3 sumI = D3(0, 0, 0);
  for (auto& c : corners) {
    d3 probePos = base + D3(c[0], c[1], c[2]) * stepv;
    d3 tri = D3(c[0] ? alpha.x : 1.0 - alpha.x, c[1] ? alpha.y : 1.0 - alpha.y, c[2] ? alpha.z : 1.0 - alpha.z);
    d3 dirToProbe = normalize(probePos - wp);
    double cc = std::max(0.0001, (dot(dirToProbe, n) + 1.0) * 0.5);
    double w = cc * cc + 0.2;                       // weightProbe :212
    w = std::max(0.000001, w);                      // :216
    if (w < 0.2) w *= w * w * (1.0 / (0.2 * 0.2));  // :221-224
    w *= tri.x * tri.y * tri.z;                     // :227
    d3 irr = sampleSingleProbe(g, atlas, px + c[0], py + c[1], pz + c[2], n);
    irr = D3(std::sqrt(irr.x), std::sqrt(irr.y), std::sqrt(irr.z));  // :235
    sumI = sumI + irr * w;
    sumW += w;
  }
  d3 net = sumI / sumW;
  net = net * net;  // :360
  return net * (0.5 * kPiSample);
}

d3 calcIndirect(const Grid& g, const DdgiFrame* f, const double* atlas, d3 n, d3 albedo, double metallic,
                double rough, d3 wp, d3 viewPos) {  // :365-388
  d3 V = normalize(viewPos - wp);
  d3 F0 = mixF0(albedo, metallic);
  d3 kS = fresnelSchlickRoughness(std::max(dot(n, V), 0.0), F0, rough * rough);
  d3 kD = (D3(1, 1, 1) - kS) * (1.0 - metallic);
  return kD * (sampleProbe(g, f, atlas, wp, n) * albedo);
}

void lattice(int n, const float rot[9], std::vector<d3>& out) {  // rgen:35-46, 87-88
  out.resize(n);
  for (int i = 0; i < n; ++i) {
    double theta = 2.0 * kPi * (double)i / kGolden;
    double phi = std::acos(1.0 - 2.0 * ((double)i + 0.5) / (double)n);
    d3 v = normalize(D3(std::cos(theta) * std::sin(phi), std::sin(theta) * std::sin(phi), std::cos(phi)));
    out[i] = D3(rot[0] * v.x + rot[3] * v.y + rot[6] * v.z, rot[1] * v.x + rot[4] * v.y + rot[7] * v.z,
                rot[2] * v.x + rot[5] * v.y + rot[8] * v.z);
  }
}

template <class F>
void parallelFor(long long n, int threads, F&& f) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<long long> next(0);
  const long long chunk = 64;
  auto work = [&]() {
    while (true) {
      long long b = next.fetch_add(chunk);
      if (b >= n) return;
      long long e = std::min(n, b + chunk);
      for (long long i = b; i < e; ++i) f(i);
    }
  };
  std::vector<std::thread> ts;
  for (int t = 1; t < threads; ++t) ts.emplace_back(work);
  work();
  for (auto& t : ts) t.join();
}

}  // namespace

// Radiance of a closest hit seen from `origin` (irradiance_probe_update.rchit:137-214; with `mirror`,
// mirror_reflections.rchit:24-117: the normal through mat3(ObjectToWorld) instead of normal * WorldToObject,
// and the DDGI term on UBO_DDGI_FLAG instead of UBO_DDGI_MULTI_FLAG). Returns the world hit position, whether
// the shadow ray toward normalize(-lightDir) hit, and whether that decision is near a tie.
d3 shadeHit(const OracleScene& s, const Grid& g, const DdgiFrame* f, const double* atlas, const Query& q, d3 origin,
            bool mirror, d3& pos, bool& shadowed, bool& sunc) {
  const d3 lightDir = D3(f->lightDir[0], f->lightDir[1], f->lightDir[2]);
  const DdgiInstance& in = s.insts[q.inst];
  const DdgiMeshInfo& m = s.meshes[in.mesh];
  const DdgiPackedVertex* v[3];
  for (int k = 0; k < 3; ++k) v[k] = &s.verts[m.vertexOffset + s.indices[m.indexOffset + 3 * q.prim + k]];
  double b1 = q.b1, b2 = q.b2, b0 = 1.0 - b1 - b2;
  double bb[3] = {b0, b1, b2};
  pos = D3(0, 0, 0);
  d3 nrm = D3(0, 0, 0), col = D3(0, 0, 0);
  for (int k = 0; k < 3; ++k) {
    const DdgiPackedVertex& pv = *v[k];
    pos = pos + D3(pv.d0[0], pv.d0[1], pv.d0[2]) * bb[k];
    col = col + D3(pv.d0[3], pv.d1[0], pv.d1[1]) * bb[k];
    nrm = nrm + D3(pv.d1[2], pv.d1[3], pv.d2[0]) * bb[k];
  }
  pos = xform(in.transform, pos);
  sunc = false;
  shadowed = anyHit(s, pos, normalize(-lightDir), sunc);
  nrm = normalize(nrm);
  d3 normal;
  if (mirror) {
    const float* t = in.transform;  // mat3(ObjectToWorld) * n
    normal = normalize(D3(t[0] * nrm.x + t[1] * nrm.y + t[2] * nrm.z, t[4] * nrm.x + t[5] * nrm.y + t[6] * nrm.z,
                          t[8] * nrm.x + t[9] * nrm.y + t[10] * nrm.z));
  } else {
    const double* wi = &s.w2o[9 * q.inst];
    normal = normalize(D3(nrm.x * wi[0] + nrm.y * wi[3] + nrm.z * wi[6], nrm.x * wi[1] + nrm.y * wi[4] + nrm.z * wi[7],
                          nrm.x * wi[2] + nrm.y * wi[5] + nrm.z * wi[8]));
  }
  d3 color = toLinear(col);
  const DdgiMaterialInfo& mat = s.mats[in.material];
  if ((double)mat.baseColFac[0] + mat.baseColFac[1] + mat.baseColFac[2] > 0.1)
    color = D3(mat.baseColFac[0], mat.baseColFac[1], mat.baseColFac[2]);
  double metallic = mat.metRough[0], rough = mat.metRough[1];
  d3 L = D3(0, 0, 0);
  if (!shadowed) L = calcLight(normal, color, metallic, rough, pos, origin, lightDir, f->sunIntensity);
  if (f->flags & (mirror ? DDGI_UBO_DDGI_FLAG : DDGI_UBO_DDGI_MULTI_FLAG))
    L = L + calcIndirect(g, f, atlas, normal, color, metallic, rough, pos, origin);
  return L + D3(mat.emissive[0], mat.emissive[1], mat.emissive[2]) * (double)mat.emissive[3];
}

extern "C" {

// Builds the FP64 scene: world-space triangles in global-id order (instance order, then primitive).
void* oracle_scene_create(const DdgiSceneDesc* d) {
  OracleScene* s = new OracleScene();
  s->verts.assign(d->vertices, d->vertices + d->numVertices);
  s->indices.assign(d->indices, d->indices + d->numIndices);
  s->meshes.assign(d->meshes, d->meshes + d->numMeshes);
  s->insts.assign(d->instances, d->instances + d->numInstances);
  s->mats.assign(d->materials, d->materials + d->numMaterials);
  int gid = 0;
  for (uint32_t i = 0; i < d->numInstances; ++i) {
    const DdgiInstance& in = d->instances[i];
    const DdgiMeshInfo& m = d->meshes[in.mesh];
    s->triOffset.push_back((uint32_t)gid);
    const float* t = in.transform;
    double a[9] = {t[0], t[1], t[2], t[4], t[5], t[6], t[8], t[9], t[10]};
    double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
    double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    double inv[9] = {c00, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4],
                     c01, a[0] * a[8] - a[2] * a[6], a[2] * a[3] - a[0] * a[5],
                     c02, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]};
    for (double v : inv) s->w2o.push_back(v / det);
    for (uint32_t p = 0; p < m.numIndices / 3; ++p) {
      Tri tr;
      for (int k = 0; k < 3; ++k) {
        const float* pp = d->vertices[m.vertexOffset + d->indices[m.indexOffset + 3 * p + k]].d0;
        tr.v[k] = xform(t, D3(pp[0], pp[1], pp[2]));
      }
      tr.inst = (int)i;
      tr.prim = (int)p;
      tr.gid = gid++;
      s->tris.push_back(tr);
    }
  }
  if (!s->tris.empty()) {
    std::vector<int> idx(s->tris.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
    std::vector<Tri> ordered;
    ordered.reserve(s->tris.size());
    buildNode(*s, idx, 0, (int)idx.size(), ordered);
    s->tris.swap(ordered);
  }
  return s;
}

void oracle_scene_destroy(void* s) { delete static_cast<OracleScene*>(s); }

// Rotated golden-angle lattice in FP64: out = n x 3 doubles.
void oracle_lattice(int n, const float rot[9], double* out) {
  std::vector<d3> v;
  lattice(n, rot, v);
  for (int i = 0; i < n; ++i) {
    out[3 * i] = v[i].x;
    out[3 * i + 1] = v[i].y;
    out[3 * i + 2] = v[i].z;
  }
}

// The value an RGBA16F image holds after a float32 store of v (the ray images of
// IrradianceProbeRayTracingPass.cpp:42-74 are R16G16B16A16_SFLOAT): v rounded to float32, then to the nearest
// binary16 value, ties to even (11-bit significand; subnormal spacing 2^-24 below 2^-14; past 65504 the value
// rounds to infinity from 65520 on).
static double storedHalf(double v) {
  const double x = (double)(float)v;
  if (!std::isfinite(x) || x == 0.0) return x;
  const double ax = std::fabs(x);
  int e = 0;
  std::frexp(ax, &e);                          // ax = m 2^e, m in [0.5, 1): the leading bit is 2^(e-1)
  const int lead = std::max(e - 1, -14);
  const double spacing = std::ldexp(1.0, lead - 10);
  double r = std::nearbyint(ax / spacing) * spacing;  // ax / spacing is exact; nearbyint rounds ties to even
  if (r > 65504.0) r = INFINITY;
  return std::copysign(r, x);
}

// Traces layers [layerBegin, layerEnd) of a grid (rgen + rchit + rmiss). atlasPrev: RGBA doubles of the
// atlas before this frame. Outputs in the ray-image layout (rayW x rayH texels): radiance RGBA doubles,
// hit code (global id * 2 + shadowed, or -1 on a miss) and uncertainty bits (1 primary, 2 shadow).
int oracle_trace(void* scene, const DdgiGridDesc* desc, const DdgiFrame* f, const double* atlasPrev,
                 int layerBegin, int layerEnd, double* rayRad, int32_t* hitOut, uint8_t* uncertainOut,
                 int threads) {
  const OracleScene& s = *static_cast<OracleScene*>(scene);
  Grid g = makeGrid(desc);
  std::vector<d3> dirs;
  lattice(g.N, f->rotation, dirs);
  d3 stepv, offv;
  probeFrame(g, f, stepv, offv);
  d3 sky = toLinear(D3(f->skyColor[0], f->skyColor[1], f->skyColor[2]) * (double)f->skyIntensity);  // rmiss:20
  long long perLayer = (long long)g.X * g.Z * g.N;
  long long total = perLayer * (layerEnd - layerBegin);
  parallelFor(total, threads, [&](long long r) {
    int layer = layerBegin + (int)(r / perLayer);
    long long rem = r % perLayer;
    int p = (int)(rem / g.N), j = (int)(rem % g.N);
    int px = p % g.X, pz = p / g.X;
    d3 origin = D3(px, layer, pz) * stepv + offv;  // rgen:72, :83
    d3 dir = dirs[j];
    Query q;
    closestHit(s, origin, dir, q);
    uint8_t unc = 0;
    if (q.gid >= 0) {
      if (q.bmin < kEpsBary || q.t < kTMin + kEpsT || q.t > kTMax - kEpsT) unc |= 1;
      if (q.tSecond <= q.t * (1.0 + kEpsTRel) + kEpsT) unc |= 1;
    }
    double tLimit = q.gid >= 0 ? q.t * (1.0 + kEpsTRel) + kEpsT : kTMax + kEpsT;
    if (q.tFuzzyMin <= tLimit) unc |= 1;
    d3 L;
    int code = -1;
    if (q.gid < 0) {
      L = sky;
    } else {
      bool sunc = false, shadowed = false;
      d3 pos;
      L = shadeHit(s, g, f, atlasPrev, q, origin, false, pos, shadowed, sunc);
      if (sunc) unc |= 2;
      code = q.gid * 2 + (shadowed ? 1 : 0);
    }
    int rx = px * g.bw + j % g.bw;
    int ry = (layer * g.Z + pz) * g.bh + j / g.bw;
    size_t idx = (size_t)ry * g.rayW + rx;
    if (desc->options & DDGI_GRID_RAYS_RGBA16F) {  // the store into the RGBA16F ray image (rgen:108-109)
      L.x = storedHalf(L.x);
      L.y = storedHalf(L.y);
      L.z = storedHalf(L.z);
    }
    rayRad[4 * idx] = L.x;
    rayRad[4 * idx + 1] = L.y;
    rayRad[4 * idx + 2] = L.z;
    rayRad[4 * idx + 3] = 1.0;
    if (hitOut) hitOut[idx] = code;
    if (uncertainOut) uncertainOut[idx] = unc;
  });
  return 0;
}

// probe_conv.comp:21-90 for layers [layerBegin, layerEnd): atlas (RGBA doubles) updated in place.
// rayRad in the ray-image layout (RGBA doubles); dirs = N x 3 doubles.
int oracle_convolve(const DdgiGridDesc* desc, const double* rayRad, const double* dirs, double* atlas,
                    int layerBegin, int layerEnd, uint32_t flags, double hysteresis, int threads) {
  Grid g = makeGrid(desc);
  bool bake = (flags & DDGI_UBO_BAKE_MODE_ON_FLAG) != 0;
  long long probes = (long long)g.X * g.Z * (layerEnd - layerBegin);
  d3 omega[kOct * kOct];
  for (int t = 0; t < kOct * kOct; ++t) omega[t] = texelDir(t % kOct, t / kOct);
  parallelFor(probes, threads, [&](long long pl) {
    int layer = layerBegin + (int)(pl / (g.X * g.Z));
    int p = (int)(pl % (g.X * g.Z));
    int px = p % g.X, pz = p / g.X;
    for (int t = 0; t < kOct * kOct; ++t) {
      double ar = 0, ag = 0, ab = 0, aw = 0;
      for (int j = 0; j < g.N; ++j) {
        d3 d = D3(dirs[3 * j], dirs[3 * j + 1], dirs[3 * j + 2]);
        double w = std::max(0.0, dot(d, omega[t]));
        if (w > 1e-6) {
          int rx = px * g.bw + j % g.bw, ry = (layer * g.Z + pz) * g.bh + j / g.bw;
          const double* L = rayRad + 4 * ((size_t)ry * g.rayW + rx);
          ar += w * L[0]; ag += w * L[1]; ab += w * L[2]; aw += w;
        }
      }
      int tx = t % kOct, ty = t / kOct;
      double* o = atlas + 4 * ((size_t)(kPix * (layer * g.Z + pz) + 1 + ty) * g.atlasW + (kPix * px + 1 + tx));
      if (bake) {  // :307-319
        double tw = o[3] + aw;
        double r = ar + o[0] * o[3], gg = ag + o[1] * o[3], b = ab + o[2] * o[3];
        if (tw > 1e-6) { r /= tw; gg /= tw; b /= tw; }
        o[0] = r; o[1] = gg; o[2] = b; o[3] = tw;
      } else {  // :321-326
        if (aw > 1e-6) { ar /= aw; ag /= aw; ab /= aw; }
        double a = 1.0 - hysteresis;
        o[0] = ar * a + o[0] * hysteresis;
        o[1] = ag * a + o[1] * hysteresis;
        o[2] = ab * a + o[2] * hysteresis;
        o[3] = aw * a + o[3] * hysteresis;
      }
    }
  });
  return 0;
}

// IrradianceProbeTranslationPass.cpp:83-168 on an RGBA texel array of `texelBytes` per texel.
int oracle_translate(const DdgiGridDesc* desc, const void* in, void* out, int dx, int dz, int texelBytes) {
  Grid g = makeGrid(desc);
  int sx = dx > 0 ? 1 : (dx < 0 ? -1 : 0), sz = dz > 0 ? 1 : (dz < 0 ? -1 : 0);
  int planeH = kPix * g.Z;
  const char* src = static_cast<const char*>(in);
  char* dst = static_cast<char*>(out);
  // full copy into the temp (:83-99), then one region per layer plane (:122-168)
  std::vector<char> tmp(src, src + (size_t)g.atlasW * g.atlasH * texelBytes);
  std::memcpy(dst, src, tmp.size());
  for (int layer = 0; layer < g.Y; ++layer) {
    int w = g.atlasW, h = planeH;
    int srcX = 0, dstX = 0, srcY = layer * planeH, dstY = layer * planeH;
    if (sx > 0) { w -= kPix; srcX = kPix; dstX = 0; }
    else if (sx < 0) { w -= kPix; srcX = 0; dstX = kPix; }
    if (sz > 0) { h -= kPix; srcY += kPix; }
    else if (sz < 0) { h -= kPix; dstY += kPix; }
    for (int y = 0; y < h; ++y)
      std::memcpy(dst + ((size_t)(dstY + y) * g.atlasW + dstX) * texelBytes,
                  tmp.data() + ((size_t)(srcY + y) * g.atlasW + srcX) * texelBytes, (size_t)w * texelBytes);
  }
  return 0;
}

// Ambient term of G-buffer points (deferred_tiled.comp:166-203, 263-299): points are DdgiSurfacePoint
// records, atlas the current atlas in FP64 RGBA, out 3 doubles per point.
int oracle_query_irradiance(const DdgiGridDesc* desc, const DdgiFrame* f, const double* atlas,
                            const DdgiSurfacePoint* pts, int64_t count, double* out) {
  Grid g = makeGrid(desc);
  g.clampToEdge = true;
  const d3 cam = D3(f->cameraPos[0], f->cameraPos[1], f->cameraPos[2]);
  for (int64_t i = 0; i < count; ++i) {
    const DdgiSurfacePoint& p = pts[i];
    const d3 wp = D3(p.position[0], p.position[1], p.position[2]);
    const d3 n = normalize(D3(p.normal[0], p.normal[1], p.normal[2]));  // :177
    const d3 albedo = D3(p.albedo[0], p.albedo[1], p.albedo[2]);
    const double shade = std::min(std::max((double)p.shadow, 0.3), 1.0);
    d3 amb = D3(0, 0, 0);
    if (f->flags & DDGI_UBO_DDGI_FLAG) {
      const d3 d = cam - wp;
      if (std::sqrt(dot(d, d)) > g.X * g.step.x / 2.0)  // :271-273
        amb = amb + albedo * (f->skyIntensity * 0.3 * shade);
      else
        amb = amb + calcIndirect(g, f, atlas, n, albedo, p.metallic, p.roughness, wp, cam);  // :289-295
    } else {
      amb = albedo * (0.3 * shade);  // :298
    }
    out[3 * i] = amb.x;
    out[3 * i + 1] = amb.y;
    out[3 * i + 2] = amb.z;
  }
  return 0;
}

// mirror_reflections.rgen/.rchit/.rmiss on FP64: pts holds 8 floats per point (position, sky, normal, unused),
// out 4 doubles per point (radiance, hit distance); uncertain: bit 0 the reflected ray's hit is near a tie
// or an edge, bit 1 its shadow ray's. The atlas is sampled as by the probe update (REPEAT addressing).
int oracle_mirror_reflections(void* scene, const DdgiGridDesc* desc, const DdgiFrame* f, const double* atlas,
                              const float* pts, int64_t count, double* out, uint8_t* uncertainOut, int threads) {
  const OracleScene& s = *static_cast<OracleScene*>(scene);
  Grid g = makeGrid(desc);
  const d3 cam = D3(f->cameraPos[0], f->cameraPos[1], f->cameraPos[2]);
  const d3 sky = toLinear(D3(f->skyColor[0], f->skyColor[1], f->skyColor[2]) * (double)f->skyIntensity);  // rmiss:20
  parallelFor(count, threads, [&](long long i) {
    const float* p = pts + 8 * i;
    double* o = out + 4 * i;
    uint8_t unc = 0;
    if (p[3] != 0.0f) {  // rgen:52-55
      o[0] = o[1] = o[2] = o[3] = 0.0;
    } else {
      const d3 origin = D3(p[0], p[1], p[2]);
      const d3 n = normalize(D3(p[4], p[5], p[6]));
      const d3 v = normalize(origin - cam);
      const d3 dir = v - n * (2.0 * dot(n, v));  // reflect (rgen:61)
      Query q;
      closestHit(s, origin, dir, q);
      if (q.gid >= 0) {
        if (q.bmin < kEpsBary || q.t < kTMin + kEpsT || q.t > kTMax - kEpsT) unc |= 1;
        if (q.tSecond <= q.t * (1.0 + kEpsTRel) + kEpsT) unc |= 1;
      }
      if (q.tFuzzyMin <= (q.gid >= 0 ? q.t * (1.0 + kEpsTRel) + kEpsT : kTMax + kEpsT)) unc |= 1;
      if (q.gid < 0) {
        o[0] = sky.x; o[1] = sky.y; o[2] = sky.z; o[3] = 1e6;
      } else {
        bool shadowed = false, sunc = false;
        d3 pos;
        const d3 L = shadeHit(s, g, f, atlas, q, origin, true, pos, shadowed, sunc);
        if (sunc) unc |= 2;
        const d3 dd = pos - origin;
        o[0] = L.x; o[1] = L.y; o[2] = L.z; o[3] = std::sqrt(dot(dd, dd));  // rchit:90
      }
    }
    if (uncertainOut) uncertainOut[i] = unc;
  });
  return 0;
}

int oracle_num_triangles(void* scene) { return (int)static_cast<OracleScene*>(scene)->tris.size(); }

// One closest-hit query in [0.1, 50]: returns the global triangle id (-1 on a miss), t, (b1, b2) and
// the uncertainty bit, for known-answer tests of the intersector.
int oracle_closest_hit(void* scene, const double* o, const double* d, double* t, double* b12, int* uncertain) {
  const OracleScene& s = *static_cast<OracleScene*>(scene);
  Query q;
  closestHit(s, D3(o[0], o[1], o[2]), D3(d[0], d[1], d[2]), q);
  int unc = 0;
  if (q.gid >= 0 && (q.bmin < kEpsBary || q.tSecond <= q.t * (1.0 + kEpsTRel) + kEpsT)) unc = 1;
  if (q.tFuzzyMin <= (q.gid >= 0 ? q.t * (1.0 + kEpsTRel) + kEpsT : kTMax + kEpsT)) unc = 1;
  if (t) *t = q.t;
  if (b12) { b12[0] = q.b1; b12[1] = q.b2; }
  if (uncertain) *uncertain = unc;
  return q.gid;
}

}  // extern "C"
