// Collapse of the binary LBVH into the 8-wide BVH that traverseWide reads (node layout in traverse.cuh).
// Host code, run once per built BVH; the binary tree comes from the device build.
//
// Each wide node starts from one binary subtree and repeatedly opens the open child (subtree of more
// than kWideLeafMax triangles) with the largest surface area until it has 8 children or none is left to
// open. Children of kWideLeafMax (one) triangle become leaf slots; their records are laid out contiguously
// per wide node in slot order (triBase + leaf slots below); larger children become wide nodes, numbered in
// breadth-first order so the internal children of a node are consecutive (childBase + internal slots below);
// the header holds the internal- and leaf-slot masks. Children are
// placed in slots by a greedy octant assignment (slot s = the child lying most toward the corner with
// sign bits s). The method follows the greedy variant of Ylitie, Karras, Laine 2017 ("Efficient
// incoherent ray traversal on GPUs through compressed wide BVHs"); child boxes are stored as FP32 planes
// or, in the default layout, as bytes on a per-node power-of-two grid (quantizeSlots).
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "traverse.cuh"

namespace ddgi {

// Quantized wide node (the DDGI_WIDE_QUANT layout): from the boxes of the used slots (bit sl of `used`)
// writes nd[0] = (origin, biased exponents) and the byte planes nd[2..4]; nd[1], the header, is the
// caller's. Origin = the union's minimum; per axis the smallest e with 255 * 2^e >= extent (e = -100 for
// a flat axis), limited to [-126, 126]; slot planes rounded outward, floor / ceil of (plane - origin) / 2^e
// in double arithmetic on the float boxes (exact). Unused slots get zero bytes. The host collapse and
// the device refit both call it.
DDGI_HD void quantizeSlots(const float lo[8][3], const float hi[8][3], uint32_t used, float4* nd) {
  float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int sl = 0; sl < 8; ++sl)
    if (used >> sl & 1u)
      for (int a = 0; a < 3; ++a) {
        nlo[a] = fminf(nlo[a], lo[sl][a]);
        nhi[a] = fmaxf(nhi[a], hi[sl][a]);
      }
  if (!used)
    for (int a = 0; a < 3; ++a) nlo[a] = nhi[a] = 0.0f;
  uint32_t eb = 0, words[12];
  for (int a = 0; a < 3; ++a) {
    const double ext = (double)nhi[a] - (double)nlo[a];
    int e = -100;
    if (ext > 0.0) {
      e = ilogb(ext) - 7;  // ext in [2^k, 2^(k+1)) and 255 * 2^(k-8) < 2^k: e is k - 7 or k - 6
      if (ldexp(255.0, e) < ext) ++e;
    }
    e = e < -126 ? -126 : e > 126 ? 126 : e;
    const double sc = ldexp(1.0, e);
    uint32_t wl[2] = {0u, 0u}, wh[2] = {0u, 0u};
    for (int sl = 0; sl < 8; ++sl) {
      if (!(used >> sl & 1u)) continue;
      const double ql = floor(((double)lo[sl][a] - (double)nlo[a]) / sc);
      const double qh = ceil(((double)hi[sl][a] - (double)nlo[a]) / sc);
      wl[sl >> 2] |= (uint32_t)fmax(0.0, fmin(255.0, ql)) << (8 * (sl & 3));
      wh[sl >> 2] |= (uint32_t)fmax(0.0, fmin(255.0, qh)) << (8 * (sl & 3));
    }
    eb |= (uint32_t)(e + 127) << (8 * a);
    words[2 * a] = wl[0];
    words[2 * a + 1] = wl[1];
    words[6 + 2 * a] = wh[0];
    words[6 + 2 * a + 1] = wh[1];
  }
  nd[0] = make_float4(nlo[0], nlo[1], nlo[2], asFloatHd(eb));
  for (int k = 0; k < 3; ++k)
    nd[2 + k] = make_float4(asFloatHd(words[4 * k]), asFloatHd(words[4 * k + 1]), asFloatHd(words[4 * k + 2]),
                            asFloatHd(words[4 * k + 3]));
}

namespace wbvh {

struct Box {
  float lo[3], hi[3];
};

inline float area(const Box& b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}

inline Box merge(const Box& a, const Box& b) {
  Box r;
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = std::min(a.lo[k], b.lo[k]);
    r.hi[k] = std::max(a.hi[k], b.hi[k]);
  }
  return r;
}

inline int asIntH(float f) { int i; std::memcpy(&i, &f, 4); return i; }
inline float asFloatH(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

struct Cand {
  int ref;    // binary child id: >= 0 internal node, < 0 triangle record ~ref
  Box box;
  int count;  // triangles below
};

constexpr int kEmptySlot = INT_MIN;  // slotRef of an empty slot

// nodes2: numTris - 1 binary nodes (4 float4 each, root 0; none when numTris == 1); tris: numTris records.
// Output: wide nodes (kWideNodeF4 float4 each, root 0), `order` (new record index -> old record index) and,
// if asked, slotRef: per wide node 8 binary child ids, the subtree each slot holds (>= 0 binary node, < 0
// ~record in the OLD record order, kEmptySlot for an empty slot) - what a refit reads the slot boxes from.
// Returns false only for numTris <= 0.
inline bool collapse(const float4* nodes2, const float4* tris, int numTris, std::vector<float4>& out,
                     std::vector<int>& order, std::vector<int>* slotRef = nullptr) {
  out.clear();
  order.clear();
  if (slotRef) slotRef->clear();
  if (numTris <= 0) return false;
  const int numNodes2 = numTris - 1;
  auto childOf = [&](int node, int k) { return asIntH(k == 0 ? nodes2[4 * node + 3].x : nodes2[4 * node + 3].y); };
  auto childBox = [&](int node, int k) {
    const float4 a = nodes2[4 * node + k], z = nodes2[4 * node + 2];
    Box b;
    b.lo[0] = a.x; b.hi[0] = a.y; b.lo[1] = a.z; b.hi[1] = a.w;
    b.lo[2] = k == 0 ? z.x : z.z;
    b.hi[2] = k == 0 ? z.y : z.w;
    return b;
  };
  auto triBox = [&](int rec) {
    Box b;
    const float4 v[3] = {tris[3 * rec], tris[3 * rec + 1], tris[3 * rec + 2]};
    for (int k = 0; k < 3; ++k) {
      float c0 = k == 0 ? v[0].x : (k == 1 ? v[0].y : v[0].z);
      float c1 = k == 0 ? v[1].x : (k == 1 ? v[1].y : v[1].z);
      float c2 = k == 0 ? v[2].x : (k == 1 ? v[2].y : v[2].z);
      b.lo[k] = std::min(c0, std::min(c1, c2));
      b.hi[k] = std::max(c0, std::max(c1, c2));
    }
    return b;
  };

  // triangle counts of the binary subtrees (iterative post-order)
  std::vector<int> count(numNodes2 > 0 ? numNodes2 : 1, 0);
  if (numNodes2 > 0) {
    std::vector<std::pair<int, int>> st;  // (node, state)
    st.push_back({0, 0});
    while (!st.empty()) {
      auto& top = st.back();
      const int n = top.first;
      if (top.second == 0) {
        top.second = 1;
        for (int k = 0; k < 2; ++k) {
          int c = childOf(n, k);
          if (c >= 0) st.push_back({c, 0});
        }
      } else {
        int s = 0;
        for (int k = 0; k < 2; ++k) {
          int c = childOf(n, k);
          s += c >= 0 ? count[c] : 1;
        }
        count[n] = s;
        st.pop_back();
      }
    }
  }
  auto cand = [&](int parent, int k) {
    Cand c;
    c.ref = childOf(parent, k);
    c.box = childBox(parent, k);
    c.count = c.ref >= 0 ? count[c.ref] : 1;
    return c;
  };
  auto gather = [&](const Cand& c, std::vector<int>& recs) {  // triangle records below a candidate
    std::vector<int> st{c.ref};
    while (!st.empty()) {
      int r = st.back();
      st.pop_back();
      if (r < 0) { recs.push_back(~r); continue; }
      st.push_back(childOf(r, 1));
      st.push_back(childOf(r, 0));
    }
  };

  struct Job {
    std::vector<Cand> kids;  // the children of the wide node before opening
    int index;
  };
  std::vector<Job> queue;
  {
    Job root;
    root.index = 0;
    if (numNodes2 == 0) {
      root.kids.push_back(Cand{~0, triBox(0), 1});
    } else {
      root.kids.push_back(cand(0, 0));
      root.kids.push_back(cand(0, 1));
    }
    queue.push_back(root);
  }
  out.resize(kWideNodeF4);
  int numWide = 1;
  for (size_t qi = 0; qi < queue.size(); ++qi) {
    std::vector<Cand> kids = std::move(queue[qi].kids);
    const int index = queue[qi].index;
    // open the largest open child while slots remain
    while ((int)kids.size() < 8) {
      int best = -1;
      float bestA = -1.0f;
      for (int i = 0; i < (int)kids.size(); ++i) {
        if (kids[i].ref >= 0 && kids[i].count > kWideLeafMax && area(kids[i].box) > bestA) {
          best = i;
          bestA = area(kids[i].box);
        }
      }
      if (best < 0) break;
      const int r = kids[best].ref;
      kids[best] = cand(r, 0);
      kids.push_back(cand(r, 1));
    }
    // octant slots: greedy on the score dot(centre_i - centre_node, corner_s)
    const int nk = (int)kids.size();
    Box nb = kids[0].box;
    for (int i = 1; i < nk; ++i) nb = merge(nb, kids[i].box);
    float nc[3];
    for (int a = 0; a < 3; ++a) nc[a] = 0.5f * (nb.lo[a] + nb.hi[a]);
    int slotOf[8], kidOf[8];
    for (int s = 0; s < 8; ++s) kidOf[s] = -1;
    for (int i = 0; i < nk; ++i) slotOf[i] = -1;
    for (int step = 0; step < nk; ++step) {
      float bestS = -3.0e38f;
      int bi = -1, bs = -1;
      for (int i = 0; i < nk; ++i) {
        if (slotOf[i] >= 0) continue;
        float d[3];
        for (int a = 0; a < 3; ++a) d[a] = 0.5f * (kids[i].box.lo[a] + kids[i].box.hi[a]) - nc[a];
        for (int s = 0; s < 8; ++s) {
          if (kidOf[s] >= 0) continue;
          float sc = ((s & 1) ? d[0] : -d[0]) + ((s & 2) ? d[1] : -d[1]) + ((s & 4) ? d[2] : -d[2]);
          if (sc > bestS) { bestS = sc; bi = i; bs = s; }
        }
      }
      slotOf[bi] = bs;
      kidOf[bs] = bi;
    }
    // leaves: one record each, laid out per node in slot order; internal children: consecutive wide nodes
    const uint32_t triBase = (uint32_t)order.size();
    const int childBase = numWide;
    uint32_t imask = 0, lmask = 0;
    int rank = 0;
    for (int s = 0; s < 8; ++s) {
      const int i = kidOf[s];
      if (i < 0) continue;
      if (kids[i].count <= kWideLeafMax) {
        std::vector<int> recs;
        gather(kids[i], recs);
        for (int rec : recs) order.push_back(rec);
        lmask |= 1u << s;
      } else {
        imask |= 1u << s;
        Job j;
        j.index = childBase + rank;
        j.kids.push_back(cand(kids[i].ref, 0));
        j.kids.push_back(cand(kids[i].ref, 1));
        queue.push_back(std::move(j));
        ++rank;
      }
    }
    numWide += rank;
    out.resize((size_t)numWide * kWideNodeF4);
    if (slotRef) {
      slotRef->resize((size_t)numWide * 8, kEmptySlot);
      for (int sl = 0; sl < 8; ++sl) (*slotRef)[(size_t)index * 8 + sl] = kidOf[sl] >= 0 ? kids[kidOf[sl]].ref : kEmptySlot;
    }
    float4* nd = out.data() + (size_t)index * kWideNodeF4;
    const uint32_t masks = imask | (lmask << 8);
#if DDGI_WIDE_QUANT
    float slo[8][3], shi[8][3];
    uint32_t used = 0;
    for (int sl = 0; sl < 8; ++sl) {
      const int i = kidOf[sl];
      for (int a = 0; a < 3; ++a) {
        slo[sl][a] = i >= 0 ? kids[i].box.lo[a] : 0.0f;
        shi[sl][a] = i >= 0 ? kids[i].box.hi[a] : 0.0f;
      }
      if (i >= 0) used |= 1u << sl;
    }
    quantizeSlots(slo, shi, used, nd);
    nd[1] = make_float4(asFloatH((uint32_t)childBase), asFloatH(triBase), asFloatH(masks), 0.0f);
#else
    nd[0] = make_float4(asFloatH((uint32_t)childBase), asFloatH(triBase), asFloatH(masks), 0.0f);
    float pl[6][8];
    for (int s = 0; s < 8; ++s) {
      const int i = kidOf[s];
      for (int a = 0; a < 3; ++a) {
        pl[2 * a][s] = i >= 0 ? kids[i].box.lo[a] : 0.0f;
        pl[2 * a + 1][s] = i >= 0 ? kids[i].box.hi[a] : 0.0f;
      }
    }
    for (int p = 0; p < 6; ++p) {
      nd[1 + 2 * p] = make_float4(pl[p][0], pl[p][1], pl[p][2], pl[p][3]);
      nd[2 + 2 * p] = make_float4(pl[p][4], pl[p][5], pl[p][6], pl[p][7]);
    }
#endif
  }
  return (int)order.size() == numTris;
}

// Header words (child base, record base, internal-slot mask, leaf-slot mask) and the exact box of slot `sl`
// of a wide node (host checks).
inline void nodeHeader(const float4* nd, uint32_t& childBase, uint32_t& triBase, uint32_t& imask, uint32_t& lmask) {
  const float4 h = nd[DDGI_WIDE_QUANT ? 1 : 0];
  childBase = (uint32_t)asIntH(h.x);
  triBase = (uint32_t)asIntH(h.y);
  imask = (uint32_t)asIntH(h.z) & 0xffu;
  lmask = ((uint32_t)asIntH(h.z) >> 8) & 0xffu;
}
inline void slotBox(const float4* nd, int sl, double lo[3], double hi[3]) {
#if DDGI_WIDE_QUANT
  const uint32_t eb = (uint32_t)asIntH(nd[0].w);
  const float p[3] = {nd[0].x, nd[0].y, nd[0].z};
  const uint32_t* w = reinterpret_cast<const uint32_t*>(nd + 2);
  auto q = [&](int word0) { return (double)((w[word0 + sl / 4] >> (8 * (sl % 4))) & 0xffu); };
  for (int a = 0; a < 3; ++a) {
    const double s = std::ldexp(1.0, (int)((eb >> (8 * a)) & 0xffu) - 127);
    lo[a] = (double)p[a] + q(2 * a) * s;
    hi[a] = (double)p[a] + q(6 + 2 * a) * s;
  }
#else
  const float* f = reinterpret_cast<const float*>(nd);
  for (int a = 0; a < 3; ++a) {
    lo[a] = f[4 * (1 + 4 * a) + sl];
    hi[a] = f[4 * (3 + 4 * a) + sl];
  }
#endif
}

}  // namespace wbvh
}  // namespace ddgi
