// LBVH build on the device. Replaces the driver-built BLAS/TLAS of the reference
// (VulkanRenderer.cpp:1265-1490, UpdateTLASPass.cpp:128-248, tlas_update.comp:57-98) with one flat BVH
// over world-space instance triangles:
//   1. flatten   instance triangles to world space (object-to-world applied once, like the TLAS does per ray)
//   2. morton    30-bit codes of the triangle-box centroids inside the centroid bounds
//   3. sort      (code, triangle) pairs with an LSD radix sort written here (8-bit digits, stable)
//   4. karras    hierarchy from the sorted codes (Karras 2012, "Maximizing parallelism in the construction
//                of BVHs, octrees and k-d trees"), equal codes split by index
//   5. bounds    bottom-up AABBs, the second child to arrive at a node computes it (atomic counters)
//   6. pack      nodes into the four-float4 traversal layout, triangles into leaf order
//   7. collapse  the binary tree into the 8-wide tree on the host (wbvh.h); triangle records are laid
//                out in the wide tree's leaf order and the binary tree's leaf ids are renumbered to match
#include "ddgi_common.cuh"
#include "lbvh.h"
#include "wbvh.h"

#include <cstring>
#include <utility>
#include <vector>

namespace ddgi {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;

DDGI_D uint32_t orderedBits(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
DDGI_HD float orderedFloat(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
#else
  uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  float f;
  memcpy(&f, &v, 4);
  return f;
#endif
}

DDGI_D float3 xform(const float* m, float3 p) {
  return f3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}

// 1. world-space triangles in global-id order, plus centroid bounds (ordered-int atomics).
__global__ void k_flatten(const InstanceGPU* __restrict__ inst, int numInst,
                          const DdgiMeshInfo* __restrict__ meshes, const uint32_t* __restrict__ indices,
                          const DdgiPackedVertex* __restrict__ verts, uint64_t numIndices, uint64_t numVerts,
                          int numTris, float4* __restrict__ trisOut, uint32_t* __restrict__ centroidBounds,
                          uint32_t* __restrict__ err) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  float3 c = f3(0.f, 0.f, 0.f);
  bool valid = g < numTris;
  if (valid) {
    int lo = 0, hi = numInst - 1;
    while (lo < hi) {  // last instance whose triOffset <= g
      int mid = (lo + hi + 1) >> 1;
      if ((int)inst[mid].triOffset <= g) lo = mid; else hi = mid - 1;
    }
    const InstanceGPU& in = inst[lo];
    int prim = g - (int)in.triOffset;
    const DdgiMeshInfo& m = meshes[in.mesh];
    float3 w[3];
    for (int k = 0; k < 3; ++k) {
      uint64_t ii = (uint64_t)m.indexOffset + 3ull * prim + k;
      uint32_t vi = ii < numIndices ? indices[ii] : 0u;
      uint64_t vv = (uint64_t)m.vertexOffset + vi;
      if (ii >= numIndices || vv >= numVerts) { atomicOr(err, DDGI_DEVERR_BOUNDS); vv = 0; }
      const float* d0 = verts[vv].d0;
      w[k] = xform(in.o2w, f3(d0[0], d0[1], d0[2]));
    }
    trisOut[3 * g + 0] = make_float4(w[0].x, w[0].y, w[0].z, __int_as_float(g));
    trisOut[3 * g + 1] = make_float4(w[1].x, w[1].y, w[1].z, __int_as_float(lo));
    trisOut[3 * g + 2] = make_float4(w[2].x, w[2].y, w[2].z, __int_as_float(prim));
    float3 bl = f3(fminf(w[0].x, fminf(w[1].x, w[2].x)), fminf(w[0].y, fminf(w[1].y, w[2].y)),
                   fminf(w[0].z, fminf(w[1].z, w[2].z)));
    float3 bh = f3(fmaxf(w[0].x, fmaxf(w[1].x, w[2].x)), fmaxf(w[0].y, fmaxf(w[1].y, w[2].y)),
                   fmaxf(w[0].z, fmaxf(w[1].z, w[2].z)));
    c = (bl + bh) * 0.5f;
  }
  // block reduction of centroid min/max through shared memory, then one atomic per block and axis
  __shared__ uint32_t smin[3], smax[3];
  if (threadIdx.x < 3) { smin[threadIdx.x] = 0xffffffffu; smax[threadIdx.x] = 0u; }
  __syncthreads();
  if (valid) {
    atomicMin(&smin[0], orderedBits(c.x)); atomicMax(&smax[0], orderedBits(c.x));
    atomicMin(&smin[1], orderedBits(c.y)); atomicMax(&smax[1], orderedBits(c.y));
    atomicMin(&smin[2], orderedBits(c.z)); atomicMax(&smax[2], orderedBits(c.z));
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    atomicMin(&centroidBounds[threadIdx.x], smin[threadIdx.x]);
    atomicMax(&centroidBounds[3 + threadIdx.x], smax[threadIdx.x]);
  }
}

DDGI_D uint32_t expandBits10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

// 2. Morton codes of triangle-box centroids.
__global__ void k_morton(const float4* __restrict__ tris, int n, const uint32_t* __restrict__ cb,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  float3 lo = f3(orderedFloat(cb[0]), orderedFloat(cb[1]), orderedFloat(cb[2]));
  float3 hi = f3(orderedFloat(cb[3]), orderedFloat(cb[4]), orderedFloat(cb[5]));
  float4 a = tris[3 * g], b = tris[3 * g + 1], c = tris[3 * g + 2];
  float3 bl = f3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
  float3 bh = f3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
  float3 cen = (bl + bh) * 0.5f;
  float3 ext = hi - lo;
  float nx = ext.x > 0.f ? (cen.x - lo.x) / ext.x : 0.f;
  float ny = ext.y > 0.f ? (cen.y - lo.y) / ext.y : 0.f;
  float nz = ext.z > 0.f ? (cen.z - lo.z) / ext.z : 0.f;
  uint32_t ix = (uint32_t)clampf(nx * 1024.f, 0.f, 1023.f);
  uint32_t iy = (uint32_t)clampf(ny * 1024.f, 0.f, 1023.f);
  uint32_t iz = (uint32_t)clampf(nz * 1024.f, 0.f, 1023.f);
  keys[g] = (expandBits10(ix) << 2) | (expandBits10(iy) << 1) | expandBits10(iz);
  vals[g] = (uint32_t)g;
}

// 3. LSD radix sort, 8-bit digits. Each tile of 4096 keys: histogram -> global scan -> stable scatter.
__global__ void k_radix_hist(const uint32_t* __restrict__ keys, int n, int shift, int numTiles,
                             uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * kSortTile;
  for (int i = 0; i < kSortItems; ++i) {
    size_t idx = base + (size_t)i * kSortThreads + threadIdx.x;
    if (idx < (size_t)n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * numTiles + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of `len` counters by one block of 1024 threads
__global__ void k_scan_single(uint32_t* __restrict__ data, int len) {
  __shared__ uint32_t part[1024];
  int t = threadIdx.x;
  int per = (len + 1023) / 1024;
  int b = t * per, e = min(len, b + per);
  uint32_t s = 0;
  for (int i = b; i < e; ++i) s += data[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint32_t v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - s;  // exclusive prefix of this thread's chunk
  for (int i = b; i < e; ++i) {
    uint32_t v = data[i];
    data[i] = run;
    run += v;
  }
}

DDGI_D uint32_t blockExclusiveScan256(uint32_t v, uint32_t* warpSums, uint32_t& total) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warpSums[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t s = lane < 8 ? warpSums[lane] : 0u;
    for (int o = 1; o < 8; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < 8) warpSums[lane] = s;  // inclusive warp prefix
  }
  __syncthreads();
  uint32_t before = w > 0 ? warpSums[w - 1] : 0u;
  total = warpSums[7];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(
    const uint32_t* __restrict__ keysIn, const uint32_t* __restrict__ valsIn, int n, int shift, int numTiles,
    const uint32_t* __restrict__ histScan, uint32_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut) {
  __shared__ uint32_t sk[kSortTile];
  __shared__ uint32_t sv[kSortTile];
  __shared__ uint32_t warpSums[8];
  __shared__ uint32_t digitStart[256];
  __shared__ uint32_t digitCount[256];
  size_t base = (size_t)blockIdx.x * kSortTile;
  // blocked arrangement: thread t owns local items [16t, 16t+16); invalid items get the largest key
  for (int i = 0; i < kSortItems; ++i) {
    int li = i * kSortThreads + threadIdx.x;  // coalesced load, then placed by local index
    size_t idx = base + li;
    sk[li] = idx < (size_t)n ? keysIn[idx] : 0xffffffffu;
    sv[li] = idx < (size_t)n ? valsIn[idx] : 0xffffffffu;
  }
  digitCount[threadIdx.x] = 0;
  __syncthreads();
  uint32_t k[kSortItems], v[kSortItems];
  for (int i = 0; i < kSortItems; ++i) {
    k[i] = sk[threadIdx.x * kSortItems + i];
    v[i] = sv[threadIdx.x * kSortItems + i];
  }
  // stable split on each of the 8 digit bits
  for (int bit = 0; bit < 8; ++bit) {
    uint32_t zeros = 0;
    for (int i = 0; i < kSortItems; ++i) zeros += ((k[i] >> (shift + bit)) & 1u) ^ 1u;
    uint32_t totalZeros;
    uint32_t zBefore = blockExclusiveScan256(zeros, warpSums, totalZeros);
    __syncthreads();
    uint32_t zi = zBefore;
    uint32_t pos0 = threadIdx.x * kSortItems;
    for (int i = 0; i < kSortItems; ++i) {
      uint32_t b = (k[i] >> (shift + bit)) & 1u;
      uint32_t dst;
      if (!b) { dst = zi; ++zi; }
      else { dst = totalZeros + (pos0 + i - zi); }
      sk[dst] = k[i];
      sv[dst] = v[i];
    }
    __syncthreads();
    for (int i = 0; i < kSortItems; ++i) {
      k[i] = sk[threadIdx.x * kSortItems + i];
      v[i] = sv[threadIdx.x * kSortItems + i];
    }
    __syncthreads();
  }
  // count valid items per digit (padding items carry value 0xffffffff and sort last)
  for (int i = 0; i < kSortItems; ++i) {
    if (v[i] != 0xffffffffu) atomicAdd(&digitCount[(k[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  {
    uint32_t tot;
    uint32_t ex = blockExclusiveScan256(digitCount[threadIdx.x], warpSums, tot);
    digitStart[threadIdx.x] = ex;
  }
  __syncthreads();
  for (int i = 0; i < kSortItems; ++i) {
    uint32_t li = threadIdx.x * kSortItems + i;
    if (v[i] == 0xffffffffu) continue;
    uint32_t d = (k[i] >> shift) & 255u;
    uint32_t dst = histScan[(size_t)d * numTiles + blockIdx.x] + (li - digitStart[d]);
    keysOut[dst] = k[i];
    valsOut[dst] = v[i];
  }
}

// 4. Karras hierarchy. delta = common prefix length of the augmented keys (code, index).
DDGI_D int delta(const uint32_t* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint32_t a = keys[i], b = keys[j];
  if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
  return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* __restrict__ keys, int n, int2* __restrict__ children,
                         int* __restrict__ parentInternal, int* __restrict__ parentLeaf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(keys, n, i, j);
  int s = 0;
  int divider = 2;
  for (int t = (l + divider - 1) / divider; ; ) {
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
    divider <<= 1;
    t = (l + divider - 1) / divider;
  }
  int gamma = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  int c0 = (lo == gamma) ? ~gamma : gamma;
  int c1 = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  children[i] = make_int2(c0, c1);
  if (c0 < 0) parentLeaf[~c0] = i; else parentInternal[c0] = i;
  if (c1 < 0) parentLeaf[~c1] = i; else parentInternal[c1] = i;
}

// 5. bottom-up bounds
__global__ void k_bounds(const float4* __restrict__ trisLeaf, int n, const int2* __restrict__ children,
                         const int* __restrict__ parentInternal, const int* __restrict__ parentLeaf,
                         float4* __restrict__ nodeLo, float4* __restrict__ nodeHi, int* __restrict__ flags) {
  int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= n) return;
  int cur = parentLeaf[L];
  while (cur >= 0) {
    __threadfence();
    if (atomicAdd(&flags[cur], 1) == 0) return;  // first arrival: the sibling finishes this node
    __threadfence();
    int2 ch = children[cur];
    float3 lo = f3(3e38f, 3e38f, 3e38f), hi = f3(-3e38f, -3e38f, -3e38f);
    int cs[2] = {ch.x, ch.y};
    for (int k = 0; k < 2; ++k) {
      int c = cs[k];
      if (c < 0) {
        int leaf = ~c;
        for (int v = 0; v < 3; ++v) {
          float4 p = trisLeaf[3 * leaf + v];
          lo = f3(fminf(lo.x, p.x), fminf(lo.y, p.y), fminf(lo.z, p.z));
          hi = f3(fmaxf(hi.x, p.x), fmaxf(hi.y, p.y), fmaxf(hi.z, p.z));
        }
      } else {
        float4 a = __ldcg(&nodeLo[c]), b = __ldcg(&nodeHi[c]);
        lo = f3(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z));
        hi = f3(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z));
      }
    }
    __stcg(&nodeLo[cur], make_float4(lo.x, lo.y, lo.z, 0.f));
    __stcg(&nodeHi[cur], make_float4(hi.x, hi.y, hi.z, 0.f));
    cur = parentInternal[cur];
  }
}

__global__ void k_gather_tris(const float4* __restrict__ trisIn, const uint32_t* __restrict__ order, int n,
                              float4* __restrict__ trisOut) {
  int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= n) return;
  uint32_t g = order[L];
  trisOut[3 * L + 0] = trisIn[3 * g + 0];
  trisOut[3 * L + 1] = trisIn[3 * g + 1];
  trisOut[3 * L + 2] = trisIn[3 * g + 2];
}

DDGI_D void leafBox(const float4* tris, int leaf, float3& lo, float3& hi) {
  float4 a = tris[3 * leaf], b = tris[3 * leaf + 1], c = tris[3 * leaf + 2];
  lo = f3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
  hi = f3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
}

// 6. pack internal nodes into the traversal layout
__global__ void k_pack(const float4* __restrict__ trisLeaf, int n, const int2* __restrict__ children,
                       const float4* __restrict__ nodeLo, const float4* __restrict__ nodeHi,
                       float4* __restrict__ nodes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int2 ch = children[i];
  float3 lo[2], hi[2];
  int cs[2] = {ch.x, ch.y};
  for (int k = 0; k < 2; ++k) {
    if (cs[k] < 0) leafBox(trisLeaf, ~cs[k], lo[k], hi[k]);
    else { lo[k] = xyz(nodeLo[cs[k]]); hi[k] = xyz(nodeHi[cs[k]]); }
  }
  nodes[4 * i + 0] = make_float4(lo[0].x, hi[0].x, lo[0].y, hi[0].y);
  nodes[4 * i + 1] = make_float4(lo[1].x, hi[1].x, lo[1].y, hi[1].y);
  nodes[4 * i + 2] = make_float4(lo[0].z, hi[0].z, lo[1].z, hi[1].z);
  nodes[4 * i + 3] = make_float4(__int_as_float(ch.x), __int_as_float(ch.y), 0.f, 0.f);
}

inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// Builds the BVH into `out` (device arrays allocated here with cudaMalloc, released by lbvhFree).
// Scratch is allocated and freed inside; the call synchronizes `stream` before returning.
cudaError_t lbvhBuild(const InstanceGPU* dInst, int numInst, const DdgiMeshInfo* dMeshes,
                      const uint32_t* dIndices, uint64_t numIndices, const DdgiPackedVertex* dVerts,
                      uint64_t numVerts, int numTris, uint32_t* dErr, cudaStream_t stream, LbvhResult* out) {
  *out = LbvhResult{};
  out->numTris = numTris;
  if (numTris == 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  float4* trisRaw = nullptr;
  uint32_t *keysA = nullptr, *keysB = nullptr, *valsA = nullptr, *valsB = nullptr, *hist = nullptr, *cb = nullptr;
  int2* children = nullptr;
  int *parentI = nullptr, *parentL = nullptr, *flags = nullptr;
  float4 *nodeLo = nullptr, *nodeHi = nullptr;
  int n = numTris;
  int numTiles = (n + kSortTile - 1) / kSortTile;
  int ni = n > 1 ? n - 1 : 1;
#define DDGI_TRY(x) do { e = (x); if (e != cudaSuccess) goto done; } while (0)
  DDGI_TRY(cudaMalloc(&trisRaw, sizeof(float4) * 3 * (size_t)n));
  DDGI_TRY(cudaMalloc(&out->tris, sizeof(float4) * 3 * (size_t)n));
  DDGI_TRY(cudaMalloc(&keysA, 4ull * n));
  DDGI_TRY(cudaMalloc(&keysB, 4ull * n));
  DDGI_TRY(cudaMalloc(&valsA, 4ull * n));
  DDGI_TRY(cudaMalloc(&valsB, 4ull * n));
  DDGI_TRY(cudaMalloc(&hist, 4ull * 256 * numTiles));
  DDGI_TRY(cudaMalloc(&cb, 4ull * 6));
  DDGI_TRY(cudaMalloc(&children, sizeof(int2) * ni));
  DDGI_TRY(cudaMalloc(&parentI, sizeof(int) * ni));
  DDGI_TRY(cudaMalloc(&parentL, sizeof(int) * n));
  DDGI_TRY(cudaMalloc(&flags, sizeof(int) * ni));
  DDGI_TRY(cudaMalloc(&nodeLo, sizeof(float4) * ni));
  DDGI_TRY(cudaMalloc(&nodeHi, sizeof(float4) * ni));
  DDGI_TRY(cudaMalloc(&out->nodes, sizeof(float4) * 4 * (size_t)ni));
  {
    uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    DDGI_TRY(cudaMemcpyAsync(cb, init, sizeof(init), cudaMemcpyHostToDevice, stream));
  }
  k_flatten<<<blocks(n, 256), 256, 0, stream>>>(dInst, numInst, dMeshes, dIndices, dVerts, numIndices, numVerts,
                                                n, trisRaw, cb, dErr);
  k_morton<<<blocks(n, 256), 256, 0, stream>>>(trisRaw, n, cb, keysA, valsA);
  for (int shift = 0; shift < 32; shift += 8) {
    k_radix_hist<<<numTiles, kSortThreads, 0, stream>>>(keysA, n, shift, numTiles, hist);
    k_scan_single<<<1, 1024, 0, stream>>>(hist, 256 * numTiles);
    k_radix_scatter<<<numTiles, kSortThreads, 0, stream>>>(keysA, valsA, n, shift, numTiles, hist, keysB, valsB);
    std::swap(keysA, keysB);
    std::swap(valsA, valsB);
  }
  k_gather_tris<<<blocks(n, 256), 256, 0, stream>>>(trisRaw, valsA, n, out->tris);
  DDGI_TRY(cudaMemsetAsync(parentI, 0xff, sizeof(int) * ni, stream));
  DDGI_TRY(cudaMemsetAsync(parentL, 0xff, sizeof(int) * n, stream));
  DDGI_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * ni, stream));
  if (n > 1) {
    k_karras<<<blocks(n - 1, 256), 256, 0, stream>>>(keysA, n, children, parentI, parentL);
    k_bounds<<<blocks(n, 256), 256, 0, stream>>>(out->tris, n, children, parentI, parentL, nodeLo, nodeHi, flags);
    k_pack<<<blocks(n - 1, 256), 256, 0, stream>>>(out->tris, n, children, nodeLo, nodeHi, out->nodes);
  }
  DDGI_TRY(cudaGetLastError());
  {
    uint32_t hb[6];
    DDGI_TRY(cudaMemcpyAsync(hb, cb, sizeof(hb), cudaMemcpyDeviceToHost, stream));
    DDGI_TRY(cudaStreamSynchronize(stream));
    for (int k = 0; k < 3; ++k) {
      out->centroidLo[k] = orderedFloat(hb[k]);
      out->centroidHi[k] = orderedFloat(hb[3 + k]);
    }
  }
  out->numNodes = n > 1 ? n - 1 : 0;
  {
    std::vector<float4> hn(4 * (size_t)out->numNodes), ht(3 * (size_t)n);
    if (out->numNodes)
      DDGI_TRY(cudaMemcpyAsync(hn.data(), out->nodes, sizeof(float4) * hn.size(), cudaMemcpyDeviceToHost, stream));
    DDGI_TRY(cudaMemcpyAsync(ht.data(), out->tris, sizeof(float4) * ht.size(), cudaMemcpyDeviceToHost, stream));
    DDGI_TRY(cudaStreamSynchronize(stream));
    std::vector<float4> wide;
    std::vector<int> order, slotRef;
    if (!wbvh::collapse(hn.data(), ht.data(), n, wide, order, &slotRef)) {
      e = cudaErrorUnknown;
      goto done;
    }
    std::vector<int> inv(n);
    for (int k = 0; k < n; ++k) inv[order[k]] = k;
    std::vector<float4> ht2(ht.size());
    for (int k = 0; k < n; ++k)
      for (int v = 0; v < 3; ++v) ht2[3 * k + v] = ht[3 * (size_t)order[k] + v];
    for (int i = 0; i < out->numNodes; ++i) {
      int c0 = wbvh::asIntH(hn[4 * i + 3].x), c1 = wbvh::asIntH(hn[4 * i + 3].y);
      if (c0 < 0) hn[4 * i + 3].x = wbvh::asFloatH((uint32_t)~inv[~c0]);
      if (c1 < 0) hn[4 * i + 3].y = wbvh::asFloatH((uint32_t)~inv[~c1]);
    }
    for (int& r : slotRef)
      if (r != wbvh::kEmptySlot && r < 0) r = ~inv[~r];
    std::vector<int> parI(std::max(1, out->numNodes), -1), parL(n, -1);
    for (int i = 0; i < out->numNodes; ++i)
      for (int k = 0; k < 2; ++k) {
        int c = wbvh::asIntH(k ? hn[4 * i + 3].y : hn[4 * i + 3].x);
        if (c >= 0) parI[c] = i; else parL[~c] = i;
      }
    DDGI_TRY(cudaMalloc(&out->parentInternal, sizeof(int) * parI.size()));
    DDGI_TRY(cudaMalloc(&out->parentLeaf, sizeof(int) * parL.size()));
    DDGI_TRY(cudaMalloc(&out->slotRef, sizeof(int) * slotRef.size()));
    DDGI_TRY(cudaMemcpyAsync(out->parentInternal, parI.data(), sizeof(int) * parI.size(), cudaMemcpyHostToDevice, stream));
    DDGI_TRY(cudaMemcpyAsync(out->parentLeaf, parL.data(), sizeof(int) * parL.size(), cudaMemcpyHostToDevice, stream));
    DDGI_TRY(cudaMemcpyAsync(out->slotRef, slotRef.data(), sizeof(int) * slotRef.size(), cudaMemcpyHostToDevice, stream));
    out->numWNodes = (int)(wide.size() / kWideNodeF4);
    DDGI_TRY(cudaMalloc(&out->wnodes, sizeof(float4) * wide.size()));
    DDGI_TRY(cudaMemcpyAsync(out->wnodes, wide.data(), sizeof(float4) * wide.size(), cudaMemcpyHostToDevice, stream));
    DDGI_TRY(cudaMemcpyAsync(out->tris, ht2.data(), sizeof(float4) * ht2.size(), cudaMemcpyHostToDevice, stream));
    if (out->numNodes)
      DDGI_TRY(cudaMemcpyAsync(out->nodes, hn.data(), sizeof(float4) * hn.size(), cudaMemcpyHostToDevice, stream));
    DDGI_TRY(cudaStreamSynchronize(stream));
  }
done:
#undef DDGI_TRY
  cudaFree(trisRaw);
  cudaFree(keysA); cudaFree(keysB); cudaFree(valsA); cudaFree(valsB);
  cudaFree(hist); cudaFree(cb); cudaFree(children); cudaFree(parentI); cudaFree(parentL); cudaFree(flags);
  cudaFree(nodeLo); cudaFree(nodeHi);
  if (e != cudaSuccess) lbvhFree(out);
  return e;
}

namespace {

// Refit 1: the triangle records again from the object-space vertices (the arithmetic of k_flatten); the
// record keeps its global id, instance and primitive in .w.
__global__ void k_refit_tris(float4* __restrict__ tris, int n, const InstanceGPU* __restrict__ inst,
                             const DdgiMeshInfo* __restrict__ meshes, const uint32_t* __restrict__ indices,
                             const DdgiPackedVertex* __restrict__ verts, uint64_t numIndices, uint64_t numVerts,
                             uint32_t* __restrict__ err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int in = __float_as_int(tris[3 * k + 1].w), prim = __float_as_int(tris[3 * k + 2].w);
  const InstanceGPU& I = inst[in];
  const DdgiMeshInfo& m = meshes[I.mesh];
  for (int v = 0; v < 3; ++v) {
    uint64_t ii = (uint64_t)m.indexOffset + 3ull * prim + v;
    uint32_t vi = ii < numIndices ? indices[ii] : 0u;
    uint64_t vv = (uint64_t)m.vertexOffset + vi;
    if (ii >= numIndices || vv >= numVerts) { atomicOr(err, DDGI_DEVERR_BOUNDS); vv = 0; }
    const float* d0 = verts[vv].d0;
    const float3 w = xform(I.o2w, f3(d0[0], d0[1], d0[2]));
    const float keep = tris[3 * k + v].w;
    tris[3 * k + v] = make_float4(w.x, w.y, w.z, keep);
  }
}

DDGI_D void recordBox(const float4* tris, int rec, float3& lo, float3& hi) {
  const float4 a = __ldcg(&tris[3 * rec]), b = __ldcg(&tris[3 * rec + 1]), c = __ldcg(&tris[3 * rec + 2]);
  lo = f3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
  hi = f3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
}

// Refit 2: binary boxes bottom-up, the second child to arrive at a node computes it (as k_bounds).
__global__ void k_refit_binary(const float4* __restrict__ tris, int n, float4* __restrict__ nodes,
                               const int* __restrict__ parentInternal, const int* __restrict__ parentLeaf,
                               float4* __restrict__ nodeLo, float4* __restrict__ nodeHi, int* __restrict__ flags) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int cur = parentLeaf[k];
  while (cur >= 0) {
    __threadfence();
    if (atomicAdd(&flags[cur], 1) == 0) return;
    __threadfence();
    const float4 n3 = __ldcg(&nodes[4 * cur + 3]);
    const int cs[2] = {__float_as_int(n3.x), __float_as_int(n3.y)};
    float3 lo[2], hi[2];
    for (int c = 0; c < 2; ++c) {
      if (cs[c] < 0) {
        recordBox(tris, ~cs[c], lo[c], hi[c]);
      } else {
        lo[c] = xyz(__ldcg(&nodeLo[cs[c]]));
        hi[c] = xyz(__ldcg(&nodeHi[cs[c]]));
      }
    }
    __stcg(&nodes[4 * cur + 0], make_float4(lo[0].x, hi[0].x, lo[0].y, hi[0].y));
    __stcg(&nodes[4 * cur + 1], make_float4(lo[1].x, hi[1].x, lo[1].y, hi[1].y));
    __stcg(&nodes[4 * cur + 2], make_float4(lo[0].z, hi[0].z, lo[1].z, hi[1].z));
    __stcg(&nodeLo[cur], make_float4(fminf(lo[0].x, lo[1].x), fminf(lo[0].y, lo[1].y), fminf(lo[0].z, lo[1].z), 0.f));
    __stcg(&nodeHi[cur], make_float4(fmaxf(hi[0].x, hi[1].x), fmaxf(hi[0].y, hi[1].y), fmaxf(hi[0].z, hi[1].z), 0.f));
    cur = parentInternal[cur];
  }
}

#if !DDGI_WIDE_QUANT
// Refit 3: every wide slot takes the box of the binary subtree it holds (FP32 node layout).
__global__ void k_refit_wide(float4* __restrict__ wnodes, int numWide, const int* __restrict__ slotRef,
                             const float4* __restrict__ tris, const float4* __restrict__ nodeLo,
                             const float4* __restrict__ nodeHi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= numWide * 8) return;
  const int node = i >> 3, sl = i & 7;
  const int ref = slotRef[i];
  if (ref == INT_MIN) return;
  float3 lo, hi;
  if (ref < 0) {
    recordBox(tris, ~ref, lo, hi);
  } else {
    lo = xyz(nodeLo[ref]);
    hi = xyz(nodeHi[ref]);
  }
  float* f = reinterpret_cast<float*>(wnodes + (size_t)node * kWideNodeF4);
  const int c = (sl >> 2), q = sl & 3;  // plane row p -> float4 1 + 2p + c, component q
  f[4 * (1 + 0 + c) + q] = lo.x;
  f[4 * (1 + 2 + c) + q] = hi.x;
  f[4 * (1 + 4 + c) + q] = lo.y;
  f[4 * (1 + 6 + c) + q] = hi.y;
  f[4 * (1 + 8 + c) + q] = lo.z;
  f[4 * (1 + 10 + c) + q] = hi.z;
}
#endif

#if DDGI_WIDE_QUANT
// Refit 3 (quantized layout): one thread per wide node re-quantizes its slots against the union of their
// refitted boxes, by the collapse's rules (quantizeSlots); the header (nd[1]) stays.
__global__ void k_refit_wide_quant(float4* __restrict__ wnodes, int numWide, const int* __restrict__ slotRef,
                                   const float4* __restrict__ tris, const float4* __restrict__ nodeLo,
                                   const float4* __restrict__ nodeHi) {
  const int node = blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= numWide) return;
  float lo[8][3], hi[8][3];
  uint32_t used = 0;
  for (int sl = 0; sl < 8; ++sl) {
    const int ref = slotRef[(size_t)node * 8 + sl];
    float3 l = f3(0.f, 0.f, 0.f), h = f3(0.f, 0.f, 0.f);
    if (ref != INT_MIN) {
      used |= 1u << sl;
      if (ref < 0) {
        recordBox(tris, ~ref, l, h);
      } else {
        l = xyz(nodeLo[ref]);
        h = xyz(nodeHi[ref]);
      }
    }
    lo[sl][0] = l.x; lo[sl][1] = l.y; lo[sl][2] = l.z;
    hi[sl][0] = h.x; hi[sl][1] = h.y; hi[sl][2] = h.z;
  }
  quantizeSlots(lo, hi, used, wnodes + (size_t)node * kWideNodeF4);
}
#endif

}  // namespace

cudaError_t lbvhRefit(LbvhResult* r, const InstanceGPU* dInst, const DdgiMeshInfo* dMeshes, const uint32_t* dIndices,
                      uint64_t numIndices, const DdgiPackedVertex* dVerts, uint64_t numVerts, uint32_t* dErr,
                      cudaStream_t stream) {
  const int n = r->numTris;
  if (n <= 0) return cudaSuccess;
  k_refit_tris<<<blocks(n, 256), 256, 0, stream>>>(r->tris, n, dInst, dMeshes, dIndices, dVerts, numIndices, numVerts,
                                                   dErr);
  float4* box = nullptr;
  int* flags = nullptr;
  const int ni = std::max(1, r->numNodes);
  cudaError_t e = cudaMallocAsync(&box, sizeof(float4) * 2 * (size_t)ni, stream);
  if (e == cudaSuccess) e = cudaMallocAsync(&flags, sizeof(int) * (size_t)ni, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)ni, stream);
  if (e == cudaSuccess && r->numNodes > 0)
    k_refit_binary<<<blocks(n, 256), 256, 0, stream>>>(r->tris, n, r->nodes, r->parentInternal, r->parentLeaf, box,
                                                       box + ni, flags);
#if DDGI_WIDE_QUANT
  if (e == cudaSuccess)
    k_refit_wide_quant<<<blocks(r->numWNodes, 128), 128, 0, stream>>>(r->wnodes, r->numWNodes, r->slotRef, r->tris,
                                                                      box, box + ni);
#else
  if (e == cudaSuccess)
    k_refit_wide<<<blocks((long long)r->numWNodes * 8, 256), 256, 0, stream>>>(r->wnodes, r->numWNodes, r->slotRef,
                                                                             r->tris, box, box + ni);
#endif
  if (e == cudaSuccess) e = cudaGetLastError();
  if (box) cudaFreeAsync(box, stream);
  if (flags) cudaFreeAsync(flags, stream);
  cudaError_t s = cudaStreamSynchronize(stream);
  return e != cudaSuccess ? e : s;
}

void lbvhFree(LbvhResult* r) {
  if (r->tris) cudaFree(r->tris);
  if (r->nodes) cudaFree(r->nodes);
  if (r->wnodes) cudaFree(r->wnodes);
  cudaFree(r->parentInternal);
  cudaFree(r->parentLeaf);
  cudaFree(r->slotRef);
  r->tris = nullptr;
  r->nodes = nullptr;
  r->wnodes = nullptr;
  r->parentInternal = r->parentLeaf = r->slotRef = nullptr;
}

}  // namespace ddgi
