// CPU check of the wide-BVH collapse and of both traversals (host build of traverse.cuh):
// a binary BVH in the device layout is built here by median splits, collapsed with wbvh::collapse, and
// closest-hit / any-hit queries through both trees are compared with a brute-force loop over all triangle
// records that uses the same watertight test and the same tie rule. Built by tests/test_wide_bvh.py with
// g++ -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "wbvh.h"

using namespace ddgi;

namespace {

struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  float uni() { return (float)((next() >> 40) * (1.0 / 16777216.0)); }
};

float asF(int i) { float f; std::memcpy(&f, &i, 4); return f; }

struct Tri {
  float v[3][3];
  int gid;
};

// binary BVH in the device layout over records in leaf order; returns the node index of the subtree
struct Bvh2Builder {
  std::vector<Tri>& tris;
  std::vector<int> idx;
  std::vector<float4> nodes;
  int nextNode = 0;
  std::vector<int> leafOrder;

  explicit Bvh2Builder(std::vector<Tri>& t) : tris(t) {}

  wbvh::Box boxOf(int lo, int hi) {
    wbvh::Box b{{3e38f, 3e38f, 3e38f}, {-3e38f, -3e38f, -3e38f}};
    for (int i = lo; i < hi; ++i)
      for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) {
          b.lo[a] = std::min(b.lo[a], tris[idx[i]].v[v][a]);
          b.hi[a] = std::max(b.hi[a], tris[idx[i]].v[v][a]);
        }
    return b;
  }
  // returns child id: >= 0 internal node, < 0 ~record
  int build(int lo, int hi) {
    if (hi - lo == 1) {
      leafOrder.push_back(idx[lo]);
      return ~((int)leafOrder.size() - 1);
    }
    int node = nextNode++;
    wbvh::Box b = boxOf(lo, hi);
    int ax = 0;
    for (int a = 1; a < 3; ++a)
      if (b.hi[a] - b.lo[a] > b.hi[ax] - b.lo[ax]) ax = a;
    int mid = (lo + hi) / 2;
    std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi, [&](int x, int y) {
      float cx = tris[x].v[0][ax] + tris[x].v[1][ax] + tris[x].v[2][ax];
      float cy = tris[y].v[0][ax] + tris[y].v[1][ax] + tris[y].v[2][ax];
      return cx < cy || (cx == cy && x < y);
    });
    int c0 = build(lo, mid);
    int c1 = build(mid, hi);
    wbvh::Box b0 = boxOf(lo, mid), b1 = boxOf(mid, hi);
    nodes[4 * node + 0] = make_float4(b0.lo[0], b0.hi[0], b0.lo[1], b0.hi[1]);
    nodes[4 * node + 1] = make_float4(b1.lo[0], b1.hi[0], b1.lo[1], b1.hi[1]);
    nodes[4 * node + 2] = make_float4(b0.lo[2], b0.hi[2], b1.lo[2], b1.hi[2]);
    nodes[4 * node + 3] = make_float4(asF(c0), asF(c1), 0.f, 0.f);
    return node;
  }
};

struct Box64 {
  double lo[3], hi[3];
};

bool sameHit(const HitInfo& a, const HitInfo& b) {
  if ((a.leaf >= 0) != (b.leaf >= 0)) return false;
  if (a.leaf < 0) return true;
  return a.gid == b.gid && a.t == b.t && a.b1 == b.b1 && a.b2 == b.b2;
}

}  // namespace

// stats[0] wide nodes, [1] triangles, [2] closest mismatches binary, [3] closest mismatches wide,
// [4] any-hit mismatches wide, [5] structure errors, [6] rays with a hit, [7] error-word bits
extern "C" int wbvh_check(int numTris, int numRays, uint64_t seed, int dupEvery, long long* stats) {
  for (int i = 0; i < 8; ++i) stats[i] = 0;
  Rng rng{seed};
  std::vector<Tri> tris(numTris);
  for (int i = 0; i < numTris; ++i) {
    Tri& t = tris[i];
    if (dupEvery > 0 && i > 0 && i % dupEvery == 0) {  // exact duplicate of the previous triangle: t ties
      t = tris[i - 1];
    } else if (i % 97 == 5) {  // degenerate (zero-area) triangle
      float c[3] = {rng.uni() * 20 - 10, rng.uni() * 20 - 10, rng.uni() * 20 - 10};
      for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) t.v[v][a] = c[a] + (a == 0 ? 0.3f * v : 0.0f);
    } else {
      float c[3] = {rng.uni() * 20 - 10, rng.uni() * 20 - 10, rng.uni() * 20 - 10};
      for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) t.v[v][a] = c[a] + (rng.uni() - 0.5f) * 1.5f;
    }
    t.gid = i;
  }
  Bvh2Builder bb(tris);
  bb.idx.resize(numTris);
  for (int i = 0; i < numTris; ++i) bb.idx[i] = i;
  bb.nodes.resize(4 * (size_t)std::max(1, numTris - 1));
  if (numTris > 1) bb.build(0, numTris);
  else bb.leafOrder.push_back(0);
  std::vector<float4> recs(3 * (size_t)numTris);
  for (int r = 0; r < numTris; ++r) {
    const Tri& t = tris[bb.leafOrder[r]];
    recs[3 * r + 0] = make_float4(t.v[0][0], t.v[0][1], t.v[0][2], asF(t.gid));
    recs[3 * r + 1] = make_float4(t.v[1][0], t.v[1][1], t.v[1][2], asF(0));
    recs[3 * r + 2] = make_float4(t.v[2][0], t.v[2][1], t.v[2][2], asF(t.gid));
  }
  std::vector<float4> wide;
  std::vector<int> order;
  if (!wbvh::collapse(bb.nodes.data(), recs.data(), numTris, wide, order)) {
    stats[5] = 1;
    return 1;
  }
  const int numWide = (int)(wide.size() / kWideNodeF4);
  stats[0] = numWide;
  stats[1] = numTris;
  // permutation check, then reorder records and remap the binary leaves
  std::vector<int> inv(numTris, -1);
  for (int k = 0; k < (int)order.size(); ++k) {
    if (order[k] < 0 || order[k] >= numTris || inv[order[k]] >= 0) { stats[5]++; continue; }
    inv[order[k]] = k;
  }
  if (stats[5]) return 1;
  std::vector<float4> recs2(recs.size());
  for (int k = 0; k < numTris; ++k)
    for (int v = 0; v < 3; ++v) recs2[3 * k + v] = recs[3 * order[k] + v];
  std::vector<float4> nodes2 = bb.nodes;
  for (int n = 0; n + 1 < numTris; ++n) {
    int c0 = wbvh::asIntH(nodes2[4 * n + 3].x), c1 = wbvh::asIntH(nodes2[4 * n + 3].y);
    if (c0 < 0) c0 = ~inv[~c0];
    if (c1 < 0) c1 = ~inv[~c1];
    nodes2[4 * n + 3].x = asF(c0);
    nodes2[4 * n + 3].y = asF(c1);
  }
  // structure: every slot's box contains every record below it; indices in range; each record once
  {
    std::vector<std::pair<int, Box64>> st;
    Box64 all{{-3e38, -3e38, -3e38}, {3e38, 3e38, 3e38}};
    st.push_back({0, all});
    int visited = 0;
    std::vector<int> seen(numTris, 0);
    while (!st.empty()) {
      auto [n, pb] = st.back();
      st.pop_back();
      if (n < 0 || n >= numWide) { stats[5]++; continue; }
      ++visited;
      const float4* nd = wide.data() + (size_t)n * kWideNodeF4;
      uint32_t childBase, triBase, imask, lmask;
      wbvh::nodeHeader(nd, childBase, triBase, imask, lmask);
      if (imask & lmask) stats[5]++;
      int rank = 0, leafRank = 0;
      for (int s = 0; s < 8; ++s) {
        const bool internal = (imask >> s) & 1u, leaf = (lmask >> s) & 1u;
        if (!internal && !leaf) continue;
        double blo[3], bhi[3];
        wbvh::slotBox(nd, s, blo, bhi);
        Box64 b{{blo[0], blo[1], blo[2]}, {bhi[0], bhi[1], bhi[2]}};
        // every triangle below a slot must lie in the slot's box: carry the intersection of the boxes
        // on the path (a quantized child node may reach one step past its parent's slot box)
        for (int a = 0; a < 3; ++a) {
          b.lo[a] = std::max(b.lo[a], pb.lo[a]);
          b.hi[a] = std::min(b.hi[a], pb.hi[a]);
        }
        if (internal) {
          st.push_back({(int)(childBase + rank), b});
          ++rank;
        } else {
          const int k = (int)triBase + leafRank++;  // one record per leaf slot, in slot order
          if (k >= numTris) { stats[5]++; continue; }
          seen[k]++;
          for (int v = 0; v < 3; ++v) {
            float4 p = recs2[3 * k + v];
            float q[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; ++a)
              if (q[a] < b.lo[a] || q[a] > b.hi[a]) stats[5]++;
          }
        }
      }
    }
    for (int k = 0; k < numTris; ++k)
      if (seen[k] != 1) stats[5]++;
    if (visited != numWide) stats[5]++;
  }
  BvhRef bref{nodes2.data(), wide.data(), recs2.data(), numTris, std::max(0, numTris - 1), numWide};
  uint32_t err = 0;
  for (int q = 0; q < numRays; ++q) {
    float3 o = f3(rng.uni() * 24 - 12, rng.uni() * 24 - 12, rng.uni() * 24 - 12);
    float3 d;
    if (q % 11 == 3) {  // axis-aligned rays, including negative zero components
      int a = q % 3;
      float sgn = (q & 8) ? -1.0f : 1.0f;
      d = f3(a == 0 ? sgn : -0.0f, a == 1 ? sgn : 0.0f, a == 2 ? sgn : -0.0f);
    } else if (q % 7 == 2 && numTris > 0) {  // aimed at a vertex or an edge midpoint of a triangle
      const Tri& t = tris[rng.next() % numTris];
      int v = q % 3;
      float3 target = f3(t.v[v][0], t.v[v][1], t.v[v][2]);
      if (q & 16) target = (target + f3(t.v[(v + 1) % 3][0], t.v[(v + 1) % 3][1], t.v[(v + 1) % 3][2])) * 0.5f;
      d = target - o;
      float l = std::sqrt(dot3(d, d));
      d = l > 0 ? d / l : f3(0, 0, 1);
    } else {
      float z = rng.uni() * 2 - 1, ph = rng.uni() * 6.2831853f, s = std::sqrt(std::max(0.0f, 1 - z * z));
      d = f3(s * std::cos(ph), s * std::sin(ph), z);
    }
    if (q % 13 == 6 && numTris > 0) {  // origin straight below a vertex: +z rays through vertices and edges
      const Tri& t = tris[rng.next() % numTris];
      o = f3(t.v[q % 3][0], t.v[q % 3][1], t.v[q % 3][2] - 3.0f);
    }
    WRay r = makeRay(o, d);
    HitInfo bf;
    bf.leaf = -1; bf.gid = INT_MAX; bf.t = 50.0f;
    for (int k = 0; k < numTris; ++k) testTri<false>(bref, r, k, 0.1f, bf);
    HitInfo h2, hw, ha;
    traverse<false>(bref, r, 0.1f, 50.0f, h2, &err);
    traverseWide<false>(bref, r, 0.1f, 50.0f, hw, &err);
    bool any = traverseWide<true>(bref, r, 0.1f, 50.0f, ha, &err);
    HitInfo hs;  // the node test with the scale formed from the node's exponent
    traverseWide<false, false, true>(bref, r, 0.1f, 50.0f, hs, &err);
    if (!sameHit(bf, h2)) stats[2]++;
    if (!sameHit(bf, hw)) stats[3]++;
    if (!sameHit(hw, hs)) stats[3]++;
    if (any != (bf.leaf >= 0) || (any && !(ha.t >= 0.1f && ha.t <= 50.0f))) stats[4]++;
    if (bf.leaf >= 0) stats[6]++;
    // the same origin along exactly +z through the specialised box test (light-space shadow rays)
    if (q % 3 == 0) {
      WRay rz = makeRay(o, f3(0.f, 0.f, 1.f));
      HitInfo bz;
      bz.leaf = -1; bz.gid = INT_MAX; bz.t = 50.0f;
      for (int k = 0; k < numTris; ++k) testTri<false>(bref, rz, k, 0.1f, bz);
      HitInfo hz, az;
      traverseWide<false, true>(bref, rz, 0.1f, 50.0f, hz, &err);
      bool anyz = traverseWide<true, true>(bref, rz, 0.1f, 50.0f, az, &err);
      HitInfo sz;
      const bool anys = traverseWide<true, true, true>(bref, rz, 0.1f, 50.0f, sz, &err);
      if (!sameHit(bz, hz)) stats[3]++;
      if (anys != anyz) stats[4]++;
      if (anyz != (bz.leaf >= 0)) stats[4]++;
    }
  }
  stats[7] = err;
  return (int)(stats[2] + stats[3] + stats[4] + stats[5] + (err ? 1 : 0));
}

// divFast (the ray-slot mapping's division by an invariant divisor) against integer division: random
// dividends below 2^31 and divisors up to 2^24, and dividends at the multiples of the divisor and one below.
extern "C" long long divfast_check(int numCases, uint64_t seed) {
  Rng rng{seed};
  long long bad = 0;
  for (int c = 0; c < numCases; ++c) {
    const uint32_t d = (c % 3 == 0) ? 1u + (uint32_t)(rng.next() % 64) : 1u + (uint32_t)(rng.next() % (1u << 24));
    const uint32_t m = divMagic(d);
    uint32_t as[4];
    as[0] = (uint32_t)(rng.next() % (1ull << 31));
    const uint32_t k = (uint32_t)(rng.next() % ((1ull << 31) / d));
    as[1] = k * d;
    as[2] = k * d ? k * d - 1 : 0;
    as[3] = 0x7fffffffu;
    for (uint32_t a : as) bad += divFast(a, d, m) != a / d;
  }
  return bad;
}

// makeRay against makeRayPacked(packRayDir(d)) (the per-direction record the lattice kernel writes): every field
// bit for bit, on random directions and on directions with zero, signed-zero and tied components.
extern "C" long long raydir_check(int numCases, uint64_t seed) {
  Rng rng{seed};
  long long bad = 0;
  auto same = [](float a, float b) { uint32_t x, y; std::memcpy(&x, &a, 4); std::memcpy(&y, &b, 4); return x == y; };
  auto same3 = [&](float3 a, float3 b) { return same(a.x, b.x) && same(a.y, b.y) && same(a.z, b.z); };
  for (int c = 0; c < numCases; ++c) {
    float3 d = f3(2.0f * rng.uni() - 1.0f, 2.0f * rng.uni() - 1.0f, 2.0f * rng.uni() - 1.0f);
    if (c % 5 == 1) d.x = (c & 8) ? -0.0f : 0.0f;
    if (c % 7 == 2) d.y = d.z;
    if (c % 11 == 3) d = f3(0.0f, 0.0f, (c & 16) ? -1.0f : 1.0f);
    const float3 o = f3(20.0f * rng.uni() - 10.0f, 20.0f * rng.uni() - 10.0f, 20.0f * rng.uni() - 10.0f);
    const WRay a = makeRay(o, d), b = makeRayPacked(o, packRayDir(d));
    const bool ok = same3(a.o, b.o) && same3(a.invd, b.invd) && same3(a.nAdd, b.nAdd) && same3(a.fAdd, b.fAdd) &&
                    same3(a.invd15, b.invd15) && same3(a.invdM, b.invdM) && a.kx == b.kx && a.ky == b.ky &&
                    a.kz == b.kz && same(a.Sx, b.Sx) && same(a.Sy, b.Sy) && same(a.Sz, b.Sz);
    bad += !ok;
  }
  return bad;
}
