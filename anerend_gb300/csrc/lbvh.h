// LBVH build interface (see lbvh.cu).
#pragma once
#include "ddgi_common.cuh"

namespace ddgi {

struct LbvhResult {
  float4* nodes = nullptr;  // 4 float4 per internal node (numNodes of them), root = 0
  float4* tris = nullptr;   // 3 float4 per triangle record, in the wide tree's leaf order
  float4* wnodes = nullptr; // kWideNodeF4 float4 per 8-wide node (numWNodes of them), root = 0
  // refit state: parents of binary nodes and records, and the binary subtree of every wide slot
  int* parentInternal = nullptr;  // numNodes
  int* parentLeaf = nullptr;      // numTris (record order)
  int* slotRef = nullptr;         // 8 per wide node: >= 0 binary node, < 0 ~record, INT_MIN empty
  int numTris = 0;
  int numNodes = 0;
  int numWNodes = 0;
  float centroidLo[3] = {0, 0, 0}, centroidHi[3] = {0, 0, 0};
};

cudaError_t lbvhBuild(const InstanceGPU* dInst, int numInst, const DdgiMeshInfo* dMeshes,
                      const uint32_t* dIndices, uint64_t numIndices, const DdgiPackedVertex* dVerts,
                      uint64_t numVerts, int numTris, uint32_t* dErr, cudaStream_t stream, LbvhResult* out);
void lbvhFree(LbvhResult* r);
// Refits `r` in place for new instance transforms and / or vertex positions (same topology): the triangle
// records are transformed again from the object-space vertices, then binary and wide boxes are rebuilt
// bottom-up. Synchronizes `stream`.
cudaError_t lbvhRefit(LbvhResult* r, const InstanceGPU* dInst, const DdgiMeshInfo* dMeshes, const uint32_t* dIndices,
                      uint64_t numIndices, const DdgiPackedVertex* dVerts, uint64_t numVerts, uint32_t* dErr,
                      cudaStream_t stream);

}  // namespace ddgi
