/*
 * ddgi.h — C ABI of the GB300 (sm_103a) DDGI probe-update engine.
 *
 * This boundary replaces three render passes of AneRend and the GPU programs they launch:
 *   IrradianceProbeTranslationPass  (src/anerend/render/passes/IrradianceProbeTranslationPass.cpp:56-186)
 *   IrradianceProbeRayTracingPass   (src/anerend/render/passes/IrradianceProbeRayTracingPass.cpp:28-166,
 *                                    assets/shaders/irradiance_probe_update.{rgen,rchit,rmiss})
 *   IrradianceProbeConvolvePass     (src/anerend/render/passes/IrradianceProbeConvolvePass.cpp:9-143,
 *                                    assets/shaders/probe_conv.comp)
 * The reference drives them through RenderPass::registerToGraph + an exe lambda per frame
 * (src/anerend/render/passes/RenderPass.h:14-35, FrameGraphBuilder.h:22-42); here every entry point is a
 * plain C function that takes plain pointers and sizes and returns an int status (DDGI_OK or a negative
 * DDGI_E* code). No exception crosses the boundary. The last error text is kept per context.
 *
 * Buffer layouts are the reference's:
 *   - ray images ("ProbeRaysIrrTex"/"ProbeRaysDirTex", IrradianceProbeRayTracingPass.cpp:42-74): one RGBA
 *     texel per ray, (bw*X) x (bh*Z) texels per probe layer, the N rays of probe (x,z) in a bw x bh block at
 *     (bw*x, bh*z), ray index = row*bw + col (irradiance_probe_update.rgen:51-58). The reference has N=256,
 *     bw=bh=16; for other N, bw = 2^ceil(log2(N)/2) and bh = N/bw. Layers are stacked vertically.
 *   - atlas ("ProbeRaysConvTex", IrradianceProbeConvolvePass.cpp:62-99): RGBA, width 10*X, height 10*Z*Y,
 *     the 8x8 interior of probe (x,y,z) at texel (10x+1, 10*Z*y + 10z + 1), one texel border, cleared to
 *     (0,0,0,1) (clearConvTex, IrradianceProbeConvolvePass.cpp:9-47).
 *   - scene records: PackedVertex (bindless.glsl:60-68), MeshInfo (bindless.glsl:51-58),
 *     MaterialInfo (bindless.glsl:43-49 = GPUMaterialInfo, GpuBuffers.h:29-36).
 *
 * Streams are passed as void* (a cudaStream_t; NULL = the legacy default stream).
 */
#ifndef DDGI_H
#define DDGI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DDGI_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------------------------------- */
#define DDGI_OK            0
#define DDGI_EINVAL       -1   /* bad argument (null pointer, size mismatch, unsupported value)      */
#define DDGI_ENOMEM       -2   /* device or host allocation failed                                   */
#define DDGI_ETIMEDOUT    -3   /* a bounded device wait gave up                                       */
#define DDGI_EDEVICE      -4   /* CUDA runtime error                                                  */
#define DDGI_EUNSUPPORTED -5   /* feature this library does not support (e.g. textured materials)     */
#define DDGI_EOVERFLOW    -6   /* a device-side bound was hit (traversal stack); work was skipped     */
#define DDGI_EBUSY        -7   /* admission refused (serving: memory budget / slots)                  */

/* ---- scene UBO flag bits: the values of scene_ubo.glsl:1-12 (GpuBuffers.h:108-122) ---------------- */
#define DDGI_UBO_DDGI_FLAG          (1u << 4)
#define DDGI_UBO_DDGI_MULTI_FLAG    (1u << 5)   /* previous-frame probe lookup in the hit shader (rchit:208) */
#define DDGI_UBO_BAKE_MODE_ON_FLAG  (1u << 11)  /* bake: tile origin + accumulate (probe_conv.comp:307-319) */

/* ---- texel formats ----------------------------------------------------------------------------- */
#define DDGI_FORMAT_RGBA32F 0   /* 16 B per texel                                                    */
#define DDGI_FORMAT_RGBA16F 1   /* 8 B per texel, the reference's VK_FORMAT_R16G16B16A16_SFLOAT      */

/* ---- grid options (DdgiGridDesc.options) --------------------------------------------------------- */
#define DDGI_GRID_EDGE_CLAMP   (1u << 0) /* clamp the +1 lookup neighbour at the grid edge instead of
                                            wrapping like the reference's REPEAT sampler does          */
#define DDGI_GRID_WRITE_DIRS   (1u << 1) /* also write the per-ray direction image (ProbeRaysDirTex)     */
#define DDGI_GRID_RECORD_HITS  (1u << 2) /* keep a per-ray hit record (global triangle id, shadow bit)   */
#define DDGI_GRID_RAYS_RGBA16F (1u << 3) /* ray radiance and direction images in RGBA16F, the format of the
                                            reference's ProbeRaysIrrTex / ProbeRaysDirTex
                                            (IrradianceProbeRayTracingPass.cpp:42-74, stored at
                                            irradiance_probe_update.rgen:108-109; round to nearest even),
                                            instead of RGBA32F                                          */

/* ---- scene records --------------------------------------------------------------------------------- */

/* PackedVertex, bindless.glsl:60-68 (96 B): pos=d0.xyz, color=(d0.w,d1.xy), normal=(d1.zw,d2.x),
 * tangent=(d2.yzw,d3.x), jointWeights=(d3.yzw,d4.x), uv=d4.yz, jointIds=d5 (unpackVertex, :98-109). */
typedef struct DdgiPackedVertex {
  float   d0[4], d1[4], d2[4], d3[4], d4[4];
  int32_t d5[4];
} DdgiPackedVertex;

/* MeshInfo, bindless.glsl:51-58 (48 B). The reference's 8-byte blasRef slot carries the mesh's index and
 * vertex counts here, because this engine builds its own BVH instead of referencing a driver BLAS. */
typedef struct DdgiMeshInfo {
  float    minPos[4];
  float    maxPos[4];
  uint32_t vertexOffset;   /* in vertices */
  uint32_t indexOffset;    /* in indices  */
  uint32_t numIndices;     /* multiple of 3 */
  uint32_t numVertices;
} DdgiMeshInfo;

/* MaterialInfo, bindless.glsl:43-49 / GPUMaterialInfo, GpuBuffers.h:29-36 (64 B).
 * Textures are not part of this path: every bindlessIndices entry must be -1 (getSurfaceDataFromMat,
 * bindless.glsl:181-237, then takes baseColFac / metRough / emissive directly). */
typedef struct DdgiMaterialInfo {
  float   baseColFac[4];
  float   emissive[4];        /* rgb * w is the emitted radiance */
  int32_t bindlessIndices[4]; /* metRough, albedo, normal, emissive: all -1 */
  float   metRough[4];        /* r metallic, g roughness */
} DdgiMaterialInfo;

/* One TLAS instance (tlas_update.comp:57-98): a 3x4 row-major object-to-world matrix (VkTransformMatrix
 * order), the mesh and the material. The reference packs material into customIndex bits 0-9 and mesh into
 * bits 10-23 (tlas_update.comp:87-92, decoded at irradiance_probe_update.rchit:137-138); here they are
 * separate 32-bit fields. All instances are double-sided opaque triangles (facing-cull disabled, :87). */
typedef struct DdgiInstance {
  float    transform[12];
  uint32_t mesh;
  uint32_t material;
  uint32_t reserved[2];
} DdgiInstance;

typedef struct DdgiSceneDesc {
  const DdgiPackedVertex* vertices;  uint64_t numVertices;
  const uint32_t*         indices;   uint64_t numIndices;
  const DdgiMeshInfo*     meshes;    uint32_t numMeshes;
  const DdgiInstance*     instances; uint32_t numInstances;
  const DdgiMaterialInfo* materials; uint32_t numMaterials;
} DdgiSceneDesc;

typedef struct DdgiSceneInfo {
  uint64_t numTriangles;   /* instance triangles after flattening */
  uint64_t numNodes;       /* internal BVH nodes */
  uint64_t deviceBytes;    /* device memory held by the scene */
  float    boundsMin[3], boundsMax[3];
} DdgiSceneInfo;

/* ---- probe grid ------------------------------------------------------------------------------------ */

/* Replaces the compile-time constants of probe_helpers.glsl:1-7 (64 x 8 x 64, step (1,2,1), N = 256,
 * 16x16 ray block, 8x8 octahedral texels) and the literals of the three passes. */
typedef struct DdgiGridDesc {
  int32_t  dims[3];        /* X, Y (layers), Z: the reference's NUM_PROBES_PER_PLANE, NUM_PROBE_PLANES, NUM_PROBES_PER_PLANE */
  float    step[3];        /* PROBE_STEP */
  float    originY;        /* world y of layer 0; the reference's grid starts at y = 0 */
  int32_t  raysPerProbe;   /* N, a power of two in [16, 1024]; the reference uses 256 */
  int32_t  atlasFormat;    /* DDGI_FORMAT_* */
  float    hysteresis;     /* probe_conv.comp:325 uses 0.96 */
  uint32_t options;        /* DDGI_GRID_* */
} DdgiGridDesc;

/* Per-frame inputs: the scene UBO fields this path reads (scene_ubo.glsl:14-37, filled at
 * VulkanRenderer.cpp:1201-1242) and the push constants (irradiance_probe_update.rgen:26-29,
 * probe_conv.comp:16-18). */
typedef struct DdgiFrame {
  float    cameraPos[3];
  float    lightDir[3];     /* direction the light travels (the shader lights along -lightDir) */
  float    sunIntensity;
  float    skyColor[3];
  float    skyIntensity;
  uint32_t flags;           /* DDGI_UBO_* bits */
  float    rotation[9];     /* mat3(randomRot), column-major as glm stores it */
  int32_t  layer;           /* probe layer to update, or -1 for every layer */
  int32_t  bakeTileInfo[3]; /* x, y: tile index, z: tile size (bake mode only) */
} DdgiFrame;

/* Launch shape of a grid's trace kernel, picked by the autotuner; the defaults are valid for every grid.
 * No counterpart in the reference (its launch shape is fixed by vkCmdTraceRaysKHR). */
typedef struct DdgiTuning {
  int32_t warpProbes;   /* probes sharing one warp: a power of two in [max(1, 32/N), 32]; default 1 */
  int32_t rayOrder;     /* 0: lattice order; 1: octahedral Morton order of the directions (default) */
  int32_t shadowMode;   /* 0: shadow rays traverse the scene BVH; 1: a BVH built in the sheared ray space of
                           the light direction, rebuilt when the direction changes (default) */
  int32_t convMode;     /* 0: FP32 convolution on CUDA cores (default); 1: tcgen05 tensor cores with FP16
                           radiance and weights; 2: tensor cores with BF16. Tensor-core modes need N % 64 == 0;
                           accumulation and the hysteresis blend stay FP32 */
  int32_t bvhWidth;     /* traversal tree: 8 = 8-wide BVH collapsed from the LBVH (default; 0 means 8);
                           2 = the binary LBVH. Both give the same hits */
  int32_t refillLanes;  /* a warp of the closest-hit traversal takes new rays once this many of its lanes are
                           idle, the shadow traversal's at half as many (1..32; default 8; 0 means 8) */
  int32_t reserved[2];
} DdgiTuning;

/* Device views of the grid's buffers (owned by the grid, or the caller's after ddgi_grid_bind_external). */
typedef struct DdgiGridBuffers {
  void*    atlas;           /* current atlas, atlasFormat texels, atlasWidth x atlasHeight */
  void*    rayRadiance;     /* ray image of rayFormat texels, rayWidth x rayHeight (all layers stacked) */
  void*    rayDirection;    /* ray image of rayFormat texels, or NULL without DDGI_GRID_WRITE_DIRS */
  int32_t* rayHit;          /* per ray (same texel order): global triangle id or -1; NULL unless RECORD_HITS */
  float*   lattice;         /* N x float4 rotated ray directions of the last trace */
  int32_t  atlasWidth, atlasHeight;
  int32_t  rayWidth, rayHeight;
  int32_t  rayBlockW, rayBlockH;
  uint64_t atlasBytes;
  uint64_t rayBytes;        /* bytes of one ray image: rayWidth x rayHeight x (16 or 8) */
  int32_t  rayFormat;       /* DDGI_FORMAT_RGBA32F, or DDGI_FORMAT_RGBA16F with DDGI_GRID_RAYS_RGBA16F */
  int32_t  reserved;
} DdgiGridBuffers;

typedef struct DdgiContext DdgiContext;
typedef struct DdgiScene   DdgiScene;
typedef struct DdgiGrid    DdgiGrid;

/* ---- context ------------------------------------------------------------------------------------- */

/* Selects `device` and creates the context (the analogue of the renderer's device + frame-graph state).
 * Reference: VulkanRenderer::init, VulkanRenderer.cpp:295-407. */
int         ddgi_context_create(int device, DdgiContext** out);
void        ddgi_context_destroy(DdgiContext* ctx);
/* Text of the last failure on this context ("" if none). Valid until the next call on the context. */
const char* ddgi_last_error(const DdgiContext* ctx);
/* Waits for `stream` and returns DDGI_EOVERFLOW / DDGI_ETIMEDOUT if a kernel raised the sticky device
 * error word since the last call (the word is cleared), DDGI_EDEVICE on a CUDA error. */
int         ddgi_sync(DdgiContext* ctx, void* stream);
int         ddgi_abi_version(void);

/* ---- failure detection ------------------------------------------------------------------------------------ */

/* Bounded device waits. The tensor-core convolution's mbarrier waits give up after spinLimit attempts (about
 * 64 ns apart); the kernel then raises DDGI_ETIMEDOUT for the next ddgi_sync, stops issuing work, waits for its
 * own copies and tensor-core work in flight, releases its tensor memory and returns, so the context stays
 * usable. No counterpart in the reference, whose fence waits never time out (VulkanRenderer.cpp:1156, 4825). */
typedef struct DdgiWaitConfig {
  uint32_t spinLimit;    /* attempts per wait before it gives up; 0: the default, 1 << 22 (about 0.3 s) */
  uint32_t stallTest;    /* test hook, 0 in production: nonzero makes each CTA's first accumulator wait wait for
                            a phase that no arrival completes, so that the timeout path runs */
  uint32_t reserved[2];
} DdgiWaitConfig;
int ddgi_context_set_waits(DdgiContext* ctx, const DdgiWaitConfig* cfg);

/* Allocation hook: called with the size before each device allocation of a grid (its buffers at creation, the
 * tensor-core operand buffers on first use, the single-grid trace scratch, the download staging) or of a scene
 * (its records and shading records; the BVH build's own buffers are not covered). A nonzero return refuses the
 * allocation: the call that needed it fails with DDGI_ENOMEM and leaves nothing half-built. The hook may run on
 * the serving loop's worker thread. NULL removes it. No counterpart in the reference, whose allocation failures
 * print and return (VulkanRenderer.cpp:1356-1358). */
typedef int (*DdgiAllocHook)(void* user, uint64_t bytes);
int ddgi_context_set_alloc_hook(DdgiContext* ctx, DdgiAllocHook hook, void* user);

/* ---- scene (replaces BLAS/TLAS builds, VulkanRenderer.cpp:1265-1490, UpdateTLASPass.cpp:128-248) ---- */

/* Copies the host arrays to the device, flattens instances to world-space triangles and builds an LBVH
 * (Morton codes, radix sort, Karras hierarchy, bottom-up bounds). Triangle t of instance i gets the
 * global id triOffset(i) + t, instances in array order. Returns when the build has finished. */
int  ddgi_scene_create(DdgiContext* ctx, const DdgiSceneDesc* desc, void* stream, DdgiScene** out);
void ddgi_scene_destroy(DdgiScene* scene);
int  ddgi_scene_info(const DdgiScene* scene, DdgiSceneInfo* info);

/* ---- grid ---------------------------------------------------------------------------------------- */

/* Allocates the atlas (cleared to (0,0,0,1)), the translation temp ("TempProbeTex"), the ray images and
 * the lattice. The translation state (_lastProbeIdx, IrradianceProbeTranslationPass.h:17) starts at (0,0)
 * and the round-robin layer at 0. */
int  ddgi_grid_create(DdgiContext* ctx, const DdgiGridDesc* desc, DdgiGrid** out);
void ddgi_grid_destroy(DdgiGrid* grid);
int  ddgi_grid_buffers(const DdgiGrid* grid, DdgiGridBuffers* out);

/* Caller-owned device buffers for a grid (zero-copy interop with a renderer that owns the images, as the
 * reference's RenderResourceVault owns "ProbeRaysConvTex", "TempProbeTex", "ProbeRaysIrrTex" and
 * "ProbeRaysDirTex", IrradianceProbeConvolvePass.cpp:62-99, IrradianceProbeTranslationPass.cpp:20-44,
 * IrradianceProbeRayTracingPass.cpp:42-74). Each buffer is tightly packed in the grid's layout (rows of
 * width x texel bytes, no padding), 16-byte aligned, on the grid's device. NULL keeps the current binding. */
typedef struct DdgiGridExternal {
  void*    atlas;         /* the current atlas: atlasBytes of atlasFormat texels                        */
  void*    atlasTemp;     /* the translation temp, atlasBytes; NULL keeps the grid's own                */
  void*    rayRadiance;   /* the ray radiance image: rayBytes of the grid's ray format                  */
  void*    rayDirection;  /* the ray direction image (grids with DDGI_GRID_WRITE_DIRS), rayBytes         */
  uint64_t atlasBytes;    /* must equal DdgiGridBuffers.atlasBytes when atlas or atlasTemp is given      */
  uint64_t rayBytes;      /* must equal DdgiGridBuffers.rayBytes when a ray image is given              */
} DdgiGridExternal;

/* Binds caller-owned buffers in place of the grid's own (which are released): from then on the passes read
 * and write the caller's memory directly, with no copies. A bound atlas is taken as the grid's current
 * atlas as it stands (ddgi_grid_reset clears it). With a bound atlas the translation pass copies the atlas
 * into the temp and shifts it back into the atlas, as the reference's pass does (two copies,
 * IrradianceProbeTranslationPass.cpp:83-168), so the current atlas always stays in the caller's buffer.
 * Waits for `stream` and for the grid's own work before releasing anything. The caller keeps ownership: the
 * buffers must outlive the grid or a later binding. DDGI_EINVAL on a size, alignment or option mismatch. */
int  ddgi_grid_bind_external(DdgiGrid* grid, const DdgiGridExternal* ext, void* stream);
/* Clears the atlas to (0,0,0,1) and the translation state to (0,0). */
int  ddgi_grid_reset(DdgiGrid* grid, void* stream);
/* Device bytes a grid of this description made by ddgi_grid_create holds with the given DdgiTuning.convMode
 * (0 for an invalid desc). It includes 8 bytes per probe ray for the hit and occluder records of the grid's
 * last trace, which seed its next trace (each ray first tests the triangle its probe's ray in the nearest
 * direction hit); grids of the serving loop are traced once and keep none. */
uint64_t ddgi_grid_footprint(const DdgiGridDesc* desc, int convMode);
/* Reads / sets the grid's launch shape (results do not depend on it). */
int  ddgi_grid_get_tuning(const DdgiGrid* grid, DdgiTuning* out);
int  ddgi_grid_set_tuning(DdgiGrid* grid, const DdgiTuning* tuning);

/* IrradianceProbeTranslationPass exe (IrradianceProbeTranslationPass.cpp:56-186): camera probe index by
 * int() truncation of cameraPos.xz/step; if it changed, shift every layer plane of the atlas by
 * sign(dx), sign(dz) probes (10 texels), keeping stale texels on the vacated edge. *moved (may be NULL)
 * receives 1 when a shift was made. */
int  ddgi_translate(DdgiGrid* grid, const float cameraPos[3], int* moved, void* stream);

/* IrradianceProbeRayTracingPass exe + irradiance_probe_update.{rgen,rchit,rmiss}: traces the rays of
 * frame->layer (or of every layer if it is -1) against `scene`, shading hits with Cook-Torrance direct
 * light, a shadow ray and (with DDGI_UBO_DDGI_MULTI_FLAG) the previous-frame probe lookup, and writes the
 * ray-radiance image. */
int  ddgi_trace(DdgiGrid* grid, const DdgiScene* scene, const DdgiFrame* frame, void* stream);

/* IrradianceProbeConvolvePass exe + probe_conv.comp: cosine-weighted sum of the rays of each probe into
 * its 8x8 octahedral texels and the hysteresis blend (bake mode: weighted accumulation). */
int  ddgi_convolve(DdgiGrid* grid, const DdgiFrame* frame, void* stream);

/* translate + trace + convolve, in the reference's pass order (VulkanRenderer.cpp:4473-4475). With
 * frame->layer == -2 the grid picks the layer round-robin like IrradianceProbeRayTracingPass.cpp:111-164. */
int  ddgi_update(DdgiGrid* grid, const DdgiScene* scene, const DdgiFrame* frame, void* stream);

/* Atlas readback / restore in the grid's atlas format (downloadDDGIAtlas, VulkanRenderer.cpp:2706-2771).
 * `bytes` must equal DdgiGridBuffers.atlasBytes. The download is complete when the call returns. */
int  ddgi_atlas_download(DdgiGrid* grid, void* host, uint64_t bytes, void* stream);
int  ddgi_atlas_upload(DdgiGrid* grid, const void* host, uint64_t bytes, void* stream);

/* The same readback without waiting (a per-frame readback that overlaps the next update): the atlas as it
 * stands in `stream`'s order is copied into a device staging buffer, then to `host` on the grid's own copy
 * stream, so later work on `stream` (the next ddgi_update) runs during the copy to the host. The staging
 * buffer (atlasBytes of device memory, outside ddgi_grid_footprint) is allocated on the first call. A
 * further call's snapshot waits on the device until the previous copy to the host has ended. `host` should
 * be pinned memory; it must stay valid, and is complete, once ddgi_atlas_download_wait returns, which
 * blocks until every download issued on the grid has reached the host. */
int  ddgi_atlas_download_async(DdgiGrid* grid, void* host, uint64_t bytes, void* stream);
int  ddgi_atlas_download_wait(DdgiGrid* grid);

/* Baked-atlas persistence in the reference's layout: the atlas as RGBA16F texels, 8 bytes each, width 10 X,
 * height 10 Z Y - the data of the asset::Texture that downloadDDGIAtlas returns (VulkanRenderer.cpp:2706-2771,
 * format RGBA16F_SFLOAT, one mip) - converted from / to the grid's atlas format (round to nearest even).
 * `bytes` must be 8 x atlasWidth x atlasHeight. Both calls are complete when they return. */
int  ddgi_atlas_export_rgba16f(DdgiGrid* grid, void* host, uint64_t bytes, void* stream);
int  ddgi_atlas_import_rgba16f(DdgiGrid* grid, const void* host, uint64_t bytes, void* stream);

/* Reads back the grid's ray buffers into host memory (any pointer may be NULL): radiance is the
 * rayWidth*rayHeight texel ray image in the grid's ray format (DdgiGridBuffers.rayBytes), hits
 * rayWidth*rayHeight int32 (needs DDGI_GRID_RECORD_HITS; global triangle id * 2 + shadowed, or -1 for a miss),
 * lattice N float4. The copy is complete when the call returns. */
int  ddgi_rays_download(DdgiGrid* grid, void* radiance, int32_t* hits, float* lattice, void* stream);

/* ---- dynamic scenes -------------------------------------------------------------------------------------- */

#define DDGI_SCENE_REFIT   0  /* keep the BVH topology, refit its boxes on the device */
#define DDGI_SCENE_REBUILD 1  /* build the BVH again (a fresh build's tree quality) */

/* New object-to-world transforms for all of the scene's instances (numInstances x 12 floats, 3 x 4 row-major
 * as DdgiInstance.transform): the per-frame TLAS update of UpdateTLASPass.cpp:176-205. The scene's BVHs (and
 * its light-space shadow BVH, if built) are refitted or rebuilt; the traced hits are the same either way.
 * Not concurrent with work that reads the scene. Synchronizes `stream`. */
int  ddgi_scene_update_transforms(DdgiScene* scene, const float* transforms, uint64_t numInstances, int mode,
                                  void* stream);
/* New vertex records [first, first + count) (host DdgiPackedVertex, e.g. skinned positions and normals): the
 * dynamic BLAS refit of UpdateBlasPass.cpp:18-19. Same BVH handling and synchronization as above. */
int  ddgi_scene_update_vertices(DdgiScene* scene, const DdgiPackedVertex* vertices, uint64_t first, uint64_t count,
                                int mode, void* stream);

/* ---- ray queries on a scene: the other ray-traced passes ------------------------------------------------- */

typedef struct DdgiRay {    /* 32 bytes */
  float origin[3];
  float tmin;
  float direction[3];       /* any length; t is in units of it, as traceRayEXT's */
  float tmax;
} DdgiRay;
typedef struct DdgiHit {    /* 16 bytes */
  float t, b1, b2;          /* distance and the barycentric weights of the triangle's 2nd and 3rd vertices */
  int32_t triangle;         /* global triangle id (instance order, primitive order), -1 for a miss */
} DdgiHit;
#define DDGI_RAY_ANY_HIT (1u << 0) /* stop at the first hit (gl_RayFlagsTerminateOnFirstHitEXT); t, b of it */

/* Closest (or any) hit of each ray in [tmin, tmax] against the scene's BVH: the traceRayEXT of the reference's
 * other ray-traced passes, on the same traversal as the probe update (watertight test, double-sided, ties
 * to the lowest global triangle id). rays / hits: device arrays of `count` records. Stream-ordered. */
int  ddgi_trace_rays(DdgiScene* scene, const DdgiRay* rays, uint64_t count, uint32_t flags, DdgiHit* hits,
                     void* stream);

/* The RT shadow pass (shadow.rgen:29-82, shadow.rmiss, shadow.rchit): for each point a ray from the point
 * along -frame->lightDir over [0.1, 50], terminating on the first hit; visibility 1 on a miss, 0 on a hit.
 * points: device float4 per point (xyz world position; w != 0 marks a sky pixel, depth == 1, which gets 1
 * without a ray); visibility: device float per point. Stream-ordered. */
int  ddgi_shadow_mask(DdgiScene* scene, const DdgiFrame* frame, const float* points, uint64_t count,
                      float* visibility, void* stream);

/* ---- atlas consumer: indirect diffuse light of G-buffer points ------------------------------------------- */

/* One G-buffer point (48 bytes): what deferred_tiled.comp:166-194 reads for a pixel. `normal` need not be
 * unit length (the shader normalises it); `shadow` is the direct-light visibility the pass computed (1 lit). */
typedef struct DdgiSurfacePoint {
  float position[3];
  float metallic;
  float normal[3];
  float roughness;
  float albedo[3];
  float shadow;
} DdgiSurfacePoint;

/* Ambient term of each point from the grid's current atlas: the DDGI block of deferred_tiled.comp:263-299 with
 * the CLAMP_TO_EDGE sampler the deferred pass binds (DeferredLightingRenderPass.cpp:192-199), no baked tile
 * atlases. With DDGI_UBO_DDGI_FLAG in frame->flags: calcIndirectDiffuseLight seen from frame->cameraPos, or
 * skyIntensity * 0.3 * albedo * clamp(shadow, 0.3, 1) beyond X * step.x / 2 from the camera; without it:
 * 0.3 * albedo * clamp(shadow, 0.3, 1). points: device array of `count` records; ambient: device array of
 * `count` float4 (rgb, w = 0). Stream-ordered; no counterpart call in the reference (a shader block). */
int  ddgi_query_irradiance(DdgiGrid* grid, const DdgiFrame* frame, const DdgiSurfacePoint* points, uint64_t count,
                           float* ambient, void* stream);

/* ---- specular GI: mirror reflections of G-buffer points ---------------------------------------------------- */

/* One G-buffer point for the mirror pass (32 bytes): its world position (calcWorldPos of the depth sample,
 * mirror_reflections.rgen:28-36), `sky` != 0 for a sky pixel (depth == 1), and the normal of Geometry0Image
 * (need not be unit length; the shader normalises it). */
typedef struct DdgiMirrorPoint {
  float position[3];
  float sky;
  float normal[3];
  float reserved;
} DdgiMirrorPoint;

/* The specular GI ray-traced pass (SpecularGIRTPass.cpp:111-128, mirror_reflections.rgen/.rchit/.rmiss): per
 * point a ray from the point along reflect(normalize(point - frame->cameraPos), normalize(normal)) over
 * [0.1, 50], closest hit; a hit is shaded as the probe update's (a shadow ray along normalize(-lightDir),
 * calcLight when lit, the DDGI indirect term from the grid's current atlas when DDGI_UBO_DDGI_FLAG is set,
 * emissive) with the normal through mat3(ObjectToWorld); the atlas is sampled with REPEAT addressing, the
 * default sampler the pass binds, and the grid's DDGI_GRID_EDGE_CLAMP neighbour rule. out: device float4 per point,
 * (radiance, hit distance); a miss gives (linear sky, 1e6), a sky point 0. FP32 where the reference stores
 * RGBA16F "ReflectTex". Stream-ordered. */
int  ddgi_mirror_reflections(DdgiGrid* grid, DdgiScene* scene, const DdgiFrame* frame, const DdgiMirrorPoint* points,
                             uint64_t count, float* out, void* stream);

/* ---- batched form: many grids in one persistent trace launch and one convolution launch ---------------- */

typedef struct DdgiBatch DdgiBatch;
typedef struct DdgiBatchItem {
  DdgiGrid*        grid;    /* each grid at most once per batch */
  const DdgiScene* scene;
} DdgiBatchItem;

/* Launch shape of a batch (picked by the autotuner, anerend_gb300/autotune.py). No counterpart in the
 * reference, whose passes run one grid with a fixed launch shape. */
typedef struct DdgiBatchTuning {
  int32_t warpProbes;    /* as DdgiTuning.warpProbes, raised per grid to 32/N where needed (default 2) */
  int32_t rayOrder;      /* as DdgiTuning.rayOrder (default 1) */
  int32_t shadowMode;    /* as DdgiTuning.shadowMode (default 1) */
  int32_t convMode;      /* as DdgiTuning.convMode (default 0); tensor-core batches hold at most 64 items */
  int32_t blocksPerSm;   /* resident 128-thread blocks per SM of the persistent trace (1..8, default 8) */
  int32_t refillLanes;   /* a warp of the closest-hit traversal takes new rays from the queue once this many of
                            its 32 lanes are idle, the shadow traversal's at half as many (1..32, default 8) */
  int32_t useGraph;      /* capture the launch sequence into a CUDA graph once its shape repeats (default 1) */
  int32_t bvhWidth;      /* as DdgiTuning.bvhWidth (default 8) */
} DdgiBatchTuning;

typedef struct DdgiBatchStats {
  uint64_t rays;           /* primary rays of the last update */
  uint32_t translations;   /* grids translated by the last update */
  uint32_t graphLaunches;  /* updates replayed from the captured graph (cumulative) */
  uint32_t eagerLaunches;  /* updates launched without the graph (cumulative) */
  uint32_t reserved;
} DdgiBatchStats;

/* Creates a batch over `n` (grid, scene) items of one context and applies the default tuning to its grids. */
int  ddgi_batch_create(DdgiContext* ctx, const DdgiBatchItem* items, int n, DdgiBatch** out);
void ddgi_batch_destroy(DdgiBatch* batch);
int  ddgi_batch_get_tuning(const DdgiBatch* batch, DdgiBatchTuning* out);
int  ddgi_batch_set_tuning(DdgiBatch* batch, const DdgiBatchTuning* tuning);
int  ddgi_batch_stats(const DdgiBatch* batch, DdgiBatchStats* out);
/* ddgi_update for every item with frames[i] (translate unless baking, trace, convolve), as one persistent
 * trace launch over all items' rays and one convolution launch, replayed from a CUDA graph once the batch's
 * shape repeats. Results equal the items' individual ddgi_update calls up to FP32 rounding order. */
int  ddgi_batch_update(DdgiBatch* batch, const DdgiFrame* frames, void* stream);

/* ---- serving: continuous batching of probe-update requests ------------------------------------------------ */

typedef struct DdgiServer DdgiServer;

#define DDGI_SERVE_FIFO           0  /* admit in arrival order */
#define DDGI_SERVE_SHORTEST_FIRST 1  /* admit the request with the fewest rays first; a request's ray count is
                                        scaled down as it waits (aging), so large ones are not starved */

typedef struct DdgiServerConfig {
  uint64_t memoryBudget;  /* device bytes of request grids admitted at once (ddgi_grid_footprint less the seeding records) */
  int32_t  maxBatch;      /* requests per launch (1..64) */
  int32_t  inFlight;      /* launches running at once, each on its own stream (1..8) */
  int32_t  convMode;      /* DdgiTuning.convMode of the served grids */
  uint32_t maxBatchMRays; /* rays per launch, in millions, admitted at most (a request larger than that runs
                             alone); 0: no limit. Short launches free their slot sooner, so later arrivals
                             wait less behind large ones */
  int32_t  policy;        /* DDGI_SERVE_*; 0 is FIFO */
  float    agingMs;       /* shortest-first: a request that has waited w ms ranks as rays x max(0, 1 - w / agingMs),
                             so after agingMs it goes ahead of every younger request (0: 50 ms) */
  int32_t  reserved[2];
} DdgiServerConfig;

/* One probe update of a grid of its own over a resident scene. The grid starts cleared, is translated,
 * traced and convolved once, and its atlas is copied to atlasOut (pinned host memory of the grid's
 * atlasBytes; NULL discards it) before the request completes. */
typedef struct DdgiRequest {
  const DdgiScene* scene;
  DdgiGridDesc     grid;
  DdgiFrame        frame;
  void*            atlasOut;
  uint64_t         tag;
} DdgiRequest;

#define DDGI_REQUEST_QUEUED    0
#define DDGI_REQUEST_RUNNING   1
#define DDGI_REQUEST_DONE      2
#define DDGI_REQUEST_FAILED   -1
#define DDGI_REQUEST_REJECTED -2

typedef struct DdgiRequestStatus {
  int32_t state;          /* DDGI_REQUEST_* */
  int32_t error;          /* status code of a failed or rejected request */
  double  submitSeconds, admitSeconds, doneSeconds;  /* server clock */
} DdgiRequestStatus;

typedef struct DdgiServerStats {
  uint64_t submitted, completed, rejected, failed, batches, rays, peakBytes;
  double   p50LatencyMs, p99LatencyMs, meanLatencyMs, maxLatencyMs, elapsedSeconds;
} DdgiServerStats;

/* Starts the serving loop's worker thread. No counterpart in the reference, which updates one grid per
 * frame inside its render loop. */
int  ddgi_server_create(DdgiContext* ctx, const DdgiServerConfig* cfg, DdgiServer** out);
/* Queues a request (thread-safe, non-blocking). DDGI_EBUSY when it alone exceeds the memory budget. */
int  ddgi_server_submit(DdgiServer* server, const DdgiRequest* request, uint64_t* id);
int  ddgi_server_status(DdgiServer* server, uint64_t id, DdgiRequestStatus* out);
/* Waits until every submitted request has finished; DDGI_ETIMEDOUT after timeoutSeconds. */
int  ddgi_server_drain(DdgiServer* server, double timeoutSeconds);
int  ddgi_server_stats(DdgiServer* server, DdgiServerStats* out);
/* Stops the worker (queued requests fail with DDGI_EBUSY), waits for running launches, frees everything. */
void ddgi_server_destroy(DdgiServer* server);

/* ---- raw kernels on caller-owned device memory ------------------------------------------------------- */

/* The golden-angle ray set of irradiance_probe_update.rgen:35-46 rotated by mat3(rot) (rgen:87-88),
 * computed in FP64 on the device and stored as N float4 (x, y, z, 0). */
int  ddgi_fibonacci_lattice(int numRays, const float rot[9], float* dirs, void* stream);

/* probe_conv.comp on device buffers: rayRadiance in the ray-image layout of `desc` (RGBA32F texels, or RGBA16F
 * with DDGI_GRID_RAYS_RGBA16F in desc->options), dirs = N float4 lattice, atlas in desc->atlasFormat. Updates
 * layers [layerBegin, layerEnd). flags: DDGI_UBO_* bits. */
int  ddgi_convolve_raw(const DdgiGridDesc* desc, const void* rayRadiance, const float* dirs, void* atlas,
                       int layerBegin, int layerEnd, uint32_t flags, void* stream);

/* ddgi_convolve_raw for callers that cannot allocate device memory while they update probes (renderers
 * that reserve all memory before the frame loop and forbid allocation inside a frame; processes whose
 * device memory is committed to a budget). It has no counterpart in the reference. The weight scratch
 * lives in a static device array of DDGI_NOALLOC_MAX_RAYS x 64 + 64 floats (131,328 bytes, held on every
 * GPU that loads the library until exit); the call allocates nothing. Returns DDGI_EINVAL when
 * desc->raysPerProbe exceeds DDGI_NOALLOC_MAX_RAYS. The first call on a device looks up the array's
 * address: make it before any stream capture. All calls share the array; calls that overlap on the GPU
 * race on it and must be ordered by the caller. */
#define DDGI_NOALLOC_MAX_RAYS 512
int  ddgi_convolve_raw_noalloc(const DdgiGridDesc* desc, const void* rayRadiance, const float* dirs,
                               void* atlas, int layerBegin, int layerEnd, uint32_t flags, void* stream);

/* 16-bit element formats of the tensor-core convolution's radiance and weights */
#define DDGI_ELEM_F16  0
#define DDGI_ELEM_BF16 1

/* probe_conv.comp as a tcgen05 tensor-core GEMM: D_c[probe][texel] = sum_j R_c[probe][j] W[texel][j] per
 * channel c, FP32 accumulation in tensor memory, then the FP32 normalisation and hysteresis blend (or bake
 * accumulation) into `atlas`. radiance16: planar 16-bit radiance, 3 x P rows of N values, row c * P + p
 * with p = (layer * Z + z) * X + x and P = X * Y * Z (see ddgi_pack_rays16). desc->raysPerProbe must be a
 * multiple of 64. Timeouts of the kernel's bounded waits are reported by ddgi_sync(ctx). */
int  ddgi_convolve_tc_raw(DdgiContext* ctx, const DdgiGridDesc* desc, const void* radiance16, int elemFormat,
                          const float* dirs, void* atlas, int layerBegin, int layerEnd, uint32_t flags,
                          void* stream);
/* Converts the ray image (the format of desc, as ddgi_convolve_raw) of layers [layerBegin, layerEnd) into the
 * planar 16-bit layout above. */
int  ddgi_pack_rays16(const DdgiGridDesc* desc, const void* rayRadiance, void* radiance16, int elemFormat,
                      int layerBegin, int layerEnd, void* stream);

/* The translation copy of IrradianceProbeTranslationPass.cpp:83-168 from atlasIn to atlasOut (distinct
 * buffers, desc->atlasFormat): atlasOut = atlasIn shifted by (sign(dx), sign(dz)) probes per layer plane. */
int  ddgi_translate_raw(const DdgiGridDesc* desc, const void* atlasIn, void* atlasOut, int dx, int dz,
                        void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DDGI_H */
