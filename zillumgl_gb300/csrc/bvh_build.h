// bvh_build.h — host MTBVH construction (binned SAH, one triangle per leaf,
// depth-first node order, six threaded hit/miss tables).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace zgl {

constexpr int32_t kLeafMask = (int32_t)0x80000000u;

// PackedBVH plus the subtree sizes, in the reference layout
// (src/accelerator/BVH.h:13-17):
//   bounds      float[M*6]   pMin.xyz, pMax.xyz of node i (DFS pre-order)
//   sizeIndices int32[M]     subtree node count, or prim | 0x80000000 at a leaf
//   hitTable    int32[6*M*3] per face f, entry k: {node, prim or -1, miss}
struct HostBVH {
    int64_t ntri = 0;
    int64_t M = 0;
    std::vector<float> bounds;
    std::vector<int32_t> sizeIndices;
    std::vector<int32_t> hitTable;
};

// Builds the tree bit-identically to BVH::quickBuild + BVH::buildHitTable
// (src/accelerator/BVH.cpp:217-296, :298-345).  Subtrees are built in
// parallel on `nthreads` host threads; the result does not depend on the
// thread count because every node depends only on its own primitive range.
void build_bvh(const float* vertices, const uint32_t* indices, int64_t ntri, HostBVH& out,
               int nthreads);

// The same build into caller arrays (M = 2*ntri - 1): bounds float[M*6],
// sizeIndices int32[M], hitTable int32[6*M*3]; every entry is written.
void build_bvh_into(const float* vertices, const uint32_t* indices, int64_t ntri, float* bounds,
                    int32_t* sizeIndices, int32_t* hitTable, int nthreads);

}  // namespace zgl
