// ORACLE — test infrastructure only. Runs the reference's DDGI shader stages, compiled from their own
// sources as FP64 C++ (build_ref.py writes them to oracle/_ref/gen/stages.inc), on the CPU:
//   ray generation (irradiance_probe_update.rgen main) per ray-image pixel, with traceRayEXT dispatching
//   to the closest-hit (.rchit) or miss (.rmiss) stage the way the ray-tracing pipeline does, and the
//   convolution (probe_conv.comp main) per invocation;
//   the specular GI pass (mirror_reflections.rgen / .rchit / .rmiss) and the RT shadow pass (shadow.rgen /
//   .rchit / .rmiss) per G-buffer point, and the deferred pass's doLight (deferred_tiled.comp) per point with
//   the direct light switched off, which leaves the ambient term of its DDGI block.
// A G-buffer point is given to a stage as a one-pixel G-buffer: ubo.invViewProj is the matrix whose only
// non-zero column is the last one, (point, 1), so calcWorldPos returns the point exactly whatever the depth.
// Which triangle a ray hits is decided by the oracle's exact FP64 closest hit (ddgi_oracle.cpp, compiled
// into the same library); the reference's own hit comes from the closed driver BVH and RT hardware. The
// harness binds the scene records (converted to FP64), the UBO fields, the push constants and the images.
// The stage code uses the reference's compile-time grid (probe_helpers.glsl: 64 x 8 x 64 probes, 256 rays,
// 16 x 16 ray blocks, 8 x 8 texels) and its hysteresis 0.96.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/ddgi.h"
#include "glsl_shim.hpp"

namespace glsl {
thread_local uvec3 gl_LaunchIDEXT;
thread_local uvec3 gl_GlobalInvocationID;
thread_local int gl_InstanceCustomIndexEXT;
thread_local int gl_PrimitiveID;
thread_local mat4x3 gl_ObjectToWorldEXT;
thread_local mat4x3 gl_WorldToObjectEXT;
thread_local dvec3 gl_WorldRayOriginEXT;

// traceRayEXT of each ray-tracing pipeline: the probe update, the specular GI mirror pass, the RT shadow pass
#define DDGI_TRACE_RAY_DECL(name)                                                                                  \
  void name(void* (*payloadAt)(int), const accelerationStructureEXT&, uint flags, uint mask, uint sbt, uint stride, \
            uint miss, const dvec3& origin, double tmin, const dvec3& dir, double tmax, int loc);
DDGI_TRACE_RAY_DECL(traceRay_probe)
DDGI_TRACE_RAY_DECL(traceRay_mirror)
DDGI_TRACE_RAY_DECL(traceRay_shadow)
thread_local uvec3 gl_LocalInvocationID;
}  // namespace glsl

#include "stages.inc"

extern "C" {
void* oracle_scene_create(const DdgiSceneDesc* d);
void oracle_scene_destroy(void* s);
int oracle_closest_hit(void* scene, const double* o, const double* d, double* t, double* b12, int* uncertain);
}

namespace {

struct Scene {
  void* oracle = nullptr;
  std::vector<rchit::PackedVertex> verts;
  std::vector<glsl::uint> indices;
  std::vector<rchit::MeshInfo> meshes;
  std::vector<rchit::MaterialInfo> mats;
  std::vector<rchit::TileInfo> tiles;
  std::vector<DdgiInstance> insts;
  std::vector<uint32_t> triOffset;  // first global triangle id of each instance
};
Scene g_scene;

// The scene records again for the specular GI and deferred stages (their record types are their own).
template <class PV, class MI, class MA, class TI>
struct SceneCopy {
  std::vector<PV> verts;
  std::vector<MI> meshes;
  std::vector<MA> mats;
  std::vector<TI> tiles;
};
SceneCopy<mrchit::PackedVertex, mrchit::MeshInfo, mrchit::MaterialInfo, mrchit::TileInfo> g_mirror;
SceneCopy<deferred::PackedVertex, deferred::MeshInfo, deferred::MaterialInfo, deferred::TileInfo> g_deferred;

glsl::dvec4 v4(const float* f) { return glsl::dvec4(f[0], f[1], f[2], f[3]); }

// object-to-world (3 x 4 row-major) as the shader's mat4x3 (4 columns of 3 rows) and its inverse
void transforms(const float* m, glsl::mat4x3& o2w, glsl::mat4x3& w2o) {
  for (int c = 0; c < 4; ++c) o2w.c[c] = glsl::dvec3(m[c], m[4 + c], m[8 + c]);
  double a[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) a[r][c] = m[4 * r + c];
  double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
               a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
  double inv[3][3];
  inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
  inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
  inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
  inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
  inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
  inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
  inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
  inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
  inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
  const double t[3] = {m[3], m[7], m[11]};
  for (int c = 0; c < 3; ++c) w2o.c[c] = glsl::dvec3(inv[0][c], inv[1][c], inv[2][c]);
  w2o.c[3] = glsl::dvec3(-(inv[0][0] * t[0] + inv[0][1] * t[1] + inv[0][2] * t[2]),
                         -(inv[1][0] * t[0] + inv[1][1] * t[1] + inv[1][2] * t[2]),
                         -(inv[2][0] * t[0] + inv[2][1] * t[1] + inv[2][2] * t[2]));
}

template <class UBO>
void setUbo(UBO& u, const DdgiFrame* f) {
  u.cameraPos = glsl::dvec4(f->cameraPos[0], f->cameraPos[1], f->cameraPos[2], 1.0);
  u.lightDir = glsl::dvec4(f->lightDir[0], f->lightDir[1], f->lightDir[2], 0.0);
  u.bakeTileInfo = glsl::ivec4(f->bakeTileInfo[0], f->bakeTileInfo[1], f->bakeTileInfo[2], 0);
  u.skyColor = glsl::dvec4(f->skyColor[0], f->skyColor[1], f->skyColor[2], 1.0);
  u.sunIntensity = f->sunIntensity;
  u.skyIntensity = f->skyIntensity;
  u.flags = f->flags;
}

}  // namespace

namespace glsl {
// The closest hit of the oracle for a traceRayEXT (the shaders' range [0.1, 50]); the instance it belongs to.
int oracleHit(const dvec3& origin, const dvec3& dir, double b12[2], int* instOut) {
  const double o[3] = {origin.x, origin.y, origin.z}, d[3] = {dir.x, dir.y, dir.z};
  double t = 0;
  int unc = 0;
  const int gid = oracle_closest_hit(g_scene.oracle, o, d, &t, b12, &unc);
  if (gid >= 0) {
    int inst = 0;
    while (inst + 1 < (int)g_scene.triOffset.size() && g_scene.triOffset[inst + 1] <= (uint32_t)gid) ++inst;
    *instOut = inst;
  }
  return gid;
}

// The specular GI pipeline's traceRayEXT (mirror_reflections.rchit / .rmiss; its shadow rays skip the closest
// hit, so a miss clears their shadow flag).
void traceRay_mirror(void* (*payloadAt)(int), const accelerationStructureEXT&, uint flags, uint, uint, uint, uint,
                     const dvec3& origin, double, const dvec3& dir, double, int loc) {
  void* payload = payloadAt(loc);
  double b12[2] = {0, 0};
  int inst = 0;
  const int gid = oracleHit(origin, dir, b12, &inst);
  if (gid < 0) {
    mrmiss::hitPayload* saved = mrmiss::payload__in;
    mrmiss::payload__in = static_cast<mrmiss::hitPayload*>(payload);
    mrmiss::stage_main();
    mrmiss::payload__in = saved;
    return;
  }
  if (flags & gl_RayFlagsSkipClosestHitShaderEXT) return;
  const DdgiInstance& in = g_scene.insts[inst];
  gl_InstanceCustomIndexEXT = (int)(in.material | (in.mesh << 10));
  gl_PrimitiveID = (int)(gid - g_scene.triOffset[inst]);
  transforms(in.transform, gl_ObjectToWorldEXT, gl_WorldToObjectEXT);
  gl_WorldRayOriginEXT = origin;
  mrchit::bary = dvec2(b12[0], b12[1]);
  mrchit::payload__in = static_cast<mrchit::hitPayload*>(payload);
  mrchit::stage_main();  // its shadow ray skips the closest hit: nothing above is overwritten
}

// The RT shadow pipeline's traceRayEXT (shadow.rchit / .rmiss).
void traceRay_shadow(void* (*payloadAt)(int), const accelerationStructureEXT&, uint flags, uint, uint, uint, uint,
                     const dvec3& origin, double, const dvec3& dir, double, int loc) {
  void* payload = payloadAt(loc);
  double b12[2] = {0, 0};
  int inst = 0;
  const int gid = oracleHit(origin, dir, b12, &inst);
  if (gid < 0) {
    srmiss::prd__in = static_cast<srmiss::hitPayload*>(payload);
    srmiss::stage_main();
    return;
  }
  if (flags & gl_RayFlagsSkipClosestHitShaderEXT) return;
  srchit::prd__in = static_cast<srchit::hitPayload*>(payload);
  srchit::stage_main();
}

// The probe update pipeline's traceRayEXT: closest hit -> the closest-hit stage (unless skipped), miss -> the
// miss stage.
void traceRay_probe(void* (*payloadAt)(int), const accelerationStructureEXT&, uint flags, uint, uint, uint, uint,
                    const dvec3& origin, double tmin, const dvec3& dir, double tmax, int loc) {
  (void)tmin;
  (void)tmax;  // the oracle query uses the shaders' range [0.1, 50]
  void* payload = payloadAt(loc);
  const double o[3] = {origin.x, origin.y, origin.z}, d[3] = {dir.x, dir.y, dir.z};
  double t = 0, b12[2] = {0, 0};
  int unc = 0;
  const int gid = oracle_closest_hit(g_scene.oracle, o, d, &t, b12, &unc);
  if (gid < 0) {
    rmiss::payload__in = static_cast<rmiss::hitPayload*>(payload);
    rmiss::stage_main();
    return;
  }
  if (flags & gl_RayFlagsSkipClosestHitShaderEXT) return;
  int inst = 0;
  while (inst + 1 < (int)g_scene.triOffset.size() && g_scene.triOffset[inst + 1] <= (uint32_t)gid) ++inst;
  const DdgiInstance& in = g_scene.insts[inst];
  // the builtins the closest-hit stage reads, saved around the call (a nested trace overwrites them)
  const int savedIdx = gl_InstanceCustomIndexEXT, savedPrim = gl_PrimitiveID;
  const mat4x3 savedO2w = gl_ObjectToWorldEXT, savedW2o = gl_WorldToObjectEXT;
  const dvec3 savedOrigin = gl_WorldRayOriginEXT;
  const dvec2 savedBary = rchit::bary;
  gl_InstanceCustomIndexEXT = (int)(in.material | (in.mesh << 10));
  gl_PrimitiveID = (int)(gid - g_scene.triOffset[inst]);
  transforms(in.transform, gl_ObjectToWorldEXT, gl_WorldToObjectEXT);
  gl_WorldRayOriginEXT = origin;
  rchit::bary = dvec2(b12[0], b12[1]);
  rchit::hitPayload* savedIn = rchit::payload__in;
  rchit::payload__in = static_cast<rchit::hitPayload*>(payload);
  rchit::stage_main();
  rchit::payload__in = savedIn;
  gl_InstanceCustomIndexEXT = savedIdx;
  gl_PrimitiveID = savedPrim;
  gl_ObjectToWorldEXT = savedO2w;
  gl_WorldToObjectEXT = savedW2o;
  gl_WorldRayOriginEXT = savedOrigin;
  rchit::bary = savedBary;
}
}  // namespace glsl

namespace {
// g_scene's records in another stage's record types (the same members)
template <class SC>
void copyScene(SC& s) {
  s.verts.resize(g_scene.verts.size());
  for (size_t i = 0; i < g_scene.verts.size(); ++i) {
    const auto& v = g_scene.verts[i];
    s.verts[i].d0 = v.d0; s.verts[i].d1 = v.d1; s.verts[i].d2 = v.d2; s.verts[i].d3 = v.d3; s.verts[i].d4 = v.d4;
    s.verts[i].d5 = v.d5;
  }
  s.meshes.resize(g_scene.meshes.size());
  for (size_t i = 0; i < g_scene.meshes.size(); ++i) {
    s.meshes[i].vertexOffset = g_scene.meshes[i].vertexOffset;
    s.meshes[i].indexOffset = g_scene.meshes[i].indexOffset;
  }
  s.mats.resize(g_scene.mats.size());
  for (size_t i = 0; i < g_scene.mats.size(); ++i) {
    s.mats[i].baseColFac = g_scene.mats[i].baseColFac;
    s.mats[i].emissive = g_scene.mats[i].emissive;
    s.mats[i].bindlessIndices = g_scene.mats[i].bindlessIndices;
    s.mats[i].metRough = g_scene.mats[i].metRough;
  }
  s.tiles.resize(g_scene.tiles.size());
  for (auto& t : s.tiles) t.ddgiAtlasTex = -1;
}

// ubo.invViewProj that maps every clip-space point to `p` (its only non-zero column is the last).
template <class UBO>
void pointAt(UBO& u, const float p[3]) {
  u.invViewProj = glsl::mat4(0.0);
  u.invViewProj.c[3] = glsl::dvec4(p[0], p[1], p[2], 1.0);
  u.screenWidth = 1;
  u.screenHeight = 1;
}

// one-texel images
struct Texel {
  double v[4] = {0, 0, 0, 0};
  void set(double a, double b, double c, double d) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
  glsl::sampler2D sampler() const {
    glsl::sampler2D s;
    s.data = v;
    s.w = s.h = 1;
    return s;
  }
};
}  // namespace

extern "C" {

// Binds a scene (the records of include/ddgi.h) to the closest-hit stage, converted to FP64.
int ref_scene_set(const DdgiSceneDesc* d) {
  if (g_scene.oracle) oracle_scene_destroy(g_scene.oracle);
  g_scene = Scene{};
  g_scene.oracle = oracle_scene_create(d);
  if (!g_scene.oracle) return -1;
  g_scene.verts.resize(d->numVertices);
  for (uint64_t i = 0; i < d->numVertices; ++i) {
    const DdgiPackedVertex& v = d->vertices[i];
    auto& o = g_scene.verts[i];
    o.d0 = v4(v.d0); o.d1 = v4(v.d1); o.d2 = v4(v.d2); o.d3 = v4(v.d3); o.d4 = v4(v.d4);
    o.d5 = glsl::ivec4(v.d5[0], v.d5[1], v.d5[2], v.d5[3]);
  }
  g_scene.indices.assign(d->indices, d->indices + d->numIndices);
  g_scene.meshes.resize(d->numMeshes);
  for (uint64_t i = 0; i < d->numMeshes; ++i) {
    g_scene.meshes[i].vertexOffset = d->meshes[i].vertexOffset;
    g_scene.meshes[i].indexOffset = d->meshes[i].indexOffset;
  }
  g_scene.mats.resize(d->numMaterials);
  for (uint64_t i = 0; i < d->numMaterials; ++i) {
    const DdgiMaterialInfo& m = d->materials[i];
    auto& o = g_scene.mats[i];
    o.baseColFac = v4(m.baseColFac);
    o.emissive = v4(m.emissive);
    o.bindlessIndices = glsl::ivec4(m.bindlessIndices[0], m.bindlessIndices[1], m.bindlessIndices[2], m.bindlessIndices[3]);
    o.metRough = v4(m.metRough);
  }
  g_scene.tiles.resize(21 * 21);  // no baked tile atlases: every entry -1
  for (auto& t : g_scene.tiles) t.ddgiAtlasTex = -1;
  g_scene.insts.assign(d->instances, d->instances + d->numInstances);
  uint32_t off = 0;
  for (const DdgiInstance& in : g_scene.insts) {
    g_scene.triOffset.push_back(off);
    off += d->meshes[in.mesh].numIndices / 3;
  }
  rchit::vertexBuffer.vertices = g_scene.verts.data();
  rchit::indexBuffer.indices = g_scene.indices.data();
  rchit::meshBuffer.meshes = g_scene.meshes.data();
  rchit::materialBuffer.infos = g_scene.mats.data();
  rchit::tileInfoBuffer.tiles = g_scene.tiles.data();
  copyScene(g_mirror);
  mrchit::vertexBuffer.vertices = g_mirror.verts.data();
  mrchit::indexBuffer.indices = g_scene.indices.data();
  mrchit::meshBuffer.meshes = g_mirror.meshes.data();
  mrchit::materialBuffer.infos = g_mirror.mats.data();
  mrchit::tileInfoBuffer.tiles = g_mirror.tiles.data();
  copyScene(g_deferred);
  deferred::materialBuffer.infos = g_deferred.mats.data();
  deferred::tileInfoBuffer.tiles = g_deferred.tiles.data();
  return 0;
}

void ref_scene_clear(void) {
  if (g_scene.oracle) oracle_scene_destroy(g_scene.oracle);
  g_scene = Scene{};
}

// Runs the ray-generation stage on pixels [x0, x1) x [y0, y1) of one layer's ray image (1024 x 1024).
// rot: mat3(randomRot) column-major; atlasPrev: the previous atlas (RGBA FP64, w x h) bound as probeTex.
// irrOut / dirOut: (x1 - x0) x (y1 - y0) RGBA FP64 texels, row-major.
int ref_trace(const DdgiFrame* f, const float rot[9], int layer, const double* atlasPrev, int atlasW, int atlasH,
              int x0, int y0, int x1, int y1, double* irrOut, double* dirOut) {
  if (!g_scene.oracle) return -1;
  setUbo(rgen::ubo, f);
  setUbo(rchit::ubo, f);
  setUbo(rmiss::ubo, f);
  rgen::pc.randomRot = glsl::mat4(1.0);
  for (int c = 0; c < 3; ++c) rgen::pc.randomRot.c[c] = glsl::dvec4(rot[3 * c], rot[3 * c + 1], rot[3 * c + 2], 0.0);
  rgen::pc.probeLayer = (glsl::uint)layer;
  rchit::probeTex.data = atlasPrev;
  rchit::probeTex.w = atlasW;
  rchit::probeTex.h = atlasH;
  const int w = x1 - x0, h = y1 - y0;
  // the stage stores into full-size images at absolute pixels; bind images that cover the rectangle
  std::vector<double> irr(4ull * 1024 * 1024, 0.0), dir(4ull * 1024 * 1024, 0.0);
  rgen::irradianceIm.data = irr.data();
  rgen::irradianceIm.w = rgen::irradianceIm.h = 1024;
  rgen::dirIm.data = dir.data();
  rgen::dirIm.w = rgen::dirIm.h = 1024;
  for (int y = y0; y < y1; ++y)
    for (int x = x0; x < x1; ++x) {
      glsl::gl_LaunchIDEXT = glsl::uvec3((glsl::uint)x, (glsl::uint)y, 0u);
      rgen::stage_main();
    }
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x)
      for (int c = 0; c < 4; ++c) {
        irrOut[4 * ((size_t)y * w + x) + c] = irr[4 * ((size_t)(y0 + y) * 1024 + x0 + x) + c];
        dirOut[4 * ((size_t)y * w + x) + c] = dir[4 * ((size_t)(y0 + y) * 1024 + x0 + x) + c];
      }
  return 0;
}

// The specular GI pass (mirror_reflections.rgen main) for each DdgiMirrorPoint, with atlas (RGBA FP64,
// atlasW x atlasH) bound as probeTex with the default REPEAT sampler. out: per point (radiance, hit distance)
// as the pass stores into ReflectTex.
int ref_mirror(const DdgiFrame* f, const double* atlas, int atlasW, int atlasH, const DdgiMirrorPoint* pts,
               int64_t count, double* out) {
  if (!g_scene.oracle) return -1;
  setUbo(mrgen::ubo, f);
  setUbo(mrchit::ubo, f);
  setUbo(mrmiss::ubo, f);
  mrchit::probeTex.data = atlas;
  mrchit::probeTex.w = atlasW;
  mrchit::probeTex.h = atlasH;
  mrchit::probeTex.clampToEdge = false;
  Texel depth, g0, g1, lut, res;
  glsl::image2D outIm;
  outIm.data = res.v;
  outIm.w = outIm.h = 1;
  for (int64_t i = 0; i < count; ++i) {
    const DdgiMirrorPoint& p = pts[i];
    pointAt(mrgen::ubo, p.position);
    depth.set(p.sky != 0.0f ? 1.0 : 0.5, 0, 0, 0);
    g0.set(p.normal[0], p.normal[1], p.normal[2], 0.0);
    g1.set(0, 0, 0, 0);
    mrgen::depthIm = depth.sampler();
    mrgen::geom0Im = g0.sampler();
    mrgen::geom1Im = g1.sampler();
    mrgen::lutTex = lut.sampler();
    mrgen::outputIm = outIm;
    res.set(0, 0, 0, 0);
    glsl::gl_LaunchIDEXT = glsl::uvec3(0u, 0u, 0u);
    mrgen::stage_main();
    for (int c = 0; c < 4; ++c) out[4 * i + c] = res.v[c];
  }
  return 0;
}

// The RT shadow pass (shadow.rgen main, UBO_RT_SHADOWS_FLAG set) for each point: float4 (world position, w != 0
// a sky pixel). vis: the value the pass stores into its r32f mask.
int ref_shadow_mask(const DdgiFrame* f, const float* points, int64_t count, double* vis) {
  if (!g_scene.oracle) return -1;
  setUbo(srgen::ubo, f);
  srgen::ubo.flags |= (1u << 3);  // UBO_RT_SHADOWS_FLAG: the pass runs
  Texel depth, res;
  glsl::image2D outIm;
  outIm.data = res.v;
  outIm.w = outIm.h = 1;
  for (int64_t i = 0; i < count; ++i) {
    const float* p = points + 4 * i;
    pointAt(srgen::ubo, p);
    depth.set(p[3] != 0.0f ? 1.0 : 0.5, 0, 0, 0);
    srgen::depth = depth.sampler();
    srgen::outputIm = outIm;
    res.set(-1, 0, 0, 0);
    glsl::gl_LaunchIDEXT = glsl::uvec3(0u, 0u, 0u);
    srgen::stage_main();
    vis[i] = res.v[0];
  }
  return 0;
}

// The deferred pass's doLight (deferred_tiled.comp) for each DdgiSurfacePoint with no point lights, no SSAO, no
// specular GI, exposure 1 and sunIntensity 0, so the stored colour is the ambient term of its DDGI block
// (deferred_tiled.comp:263-299) plus the zero emissive; the point's shadow comes through the RT shadow mask,
// atlas (RGBA FP64) is bound as probeTex with the pass's CLAMP_TO_EDGE sampler. out: count x 3 doubles.
int ref_query_irradiance(const DdgiFrame* f, const double* atlas, int atlasW, int atlasH, const DdgiSurfacePoint* pts,
                         int64_t count, double* out) {
  if (!g_scene.oracle) return -1;
  DdgiFrame fr = *f;
  fr.sunIntensity = 0.0f;
  setUbo(deferred::ubo, &fr);
  deferred::ubo.flags = (f->flags & (1u << 4)) | (1u << 3);  // UBO_DDGI_FLAG as given, UBO_RT_SHADOWS_FLAG
  deferred::ubo.exposure = 1.0;
  deferred::probeTex.data = atlas;
  deferred::probeTex.w = atlasW;
  deferred::probeTex.h = atlasH;
  deferred::probeTex.clampToEdge = true;
  deferred::groupLocalNumIndices = 0;
  Texel i0, i1, i2, depth, mask, res;
  glsl::image2D outIm;
  outIm.data = res.v;
  outIm.w = outIm.h = 1;
  for (int64_t i = 0; i < count; ++i) {
    const DdgiSurfacePoint& p = pts[i];
    pointAt(deferred::ubo, p.position);
    i0.set(p.normal[0], p.normal[1], p.normal[2], p.albedo[0]);
    i1.set(p.albedo[1], p.albedo[2], p.metallic, p.roughness);
    i2.set(0, 0, 0, 0);
    depth.set(0.5, 0, 0, 0);
    mask.set(p.shadow, 0, 0, 0);
    deferred::im0 = i0.sampler();
    deferred::im1 = i1.sampler();
    deferred::im2 = i2.sampler();
    deferred::depth = depth.sampler();
    deferred::rtShadowMask = mask.sampler();
    deferred::outputIm = outIm;
    res.set(0, 0, 0, 0);
    deferred::doLight(glsl::ivec2(0, 0));
    for (int c = 0; c < 3; ++c) out[3 * i + c] = res.v[c];
  }
  return 0;
}

// Runs the convolution stage on invocations [x0, x1) x [y0, y1) of one layer (at most 512 x 512: the
// reference's guard lets one extra row and column through, which read past the ray image; not modelled).
// irrImg / dirImg: the layer's ray images (1024 x 1024 RGBA FP64); atlas: 640 x 5120 RGBA FP64, in place.
int ref_convolve(const DdgiFrame* f, int layer, const double* irrImg, const double* dirImg, double* atlas, int x0,
                 int y0, int x1, int y1) {
  if (x0 < 0 || y0 < 0 || x1 > 512 || y1 > 512) return -1;
  setUbo(conv::ubo, f);
  conv::pc.probeLayer = (glsl::uint)layer;
  conv::irrIm.data = const_cast<double*>(irrImg);
  conv::irrIm.w = conv::irrIm.h = 1024;
  conv::dirIm.data = const_cast<double*>(dirImg);
  conv::dirIm.w = conv::dirIm.h = 1024;
  conv::outputIm.data = atlas;
  conv::outputIm.w = 640;
  conv::outputIm.h = 5120;
  for (int y = y0; y < y1; ++y)
    for (int x = x0; x < x1; ++x) {
      glsl::gl_GlobalInvocationID = glsl::uvec3((glsl::uint)x, (glsl::uint)y, 0u);
      conv::stage_main();
    }
  return 0;
}

}  // extern "C"
