// ref_bvh_shim.cpp — C ABI over the reference's own MTBVH builder.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_oracle.py copies the reference's
// src/accelerator/{BVH.h, BVH.cpp, AABB.h, AABB.cpp} and src/util/{Error.h,
// Timer.h, NamespaceDecl.h} unchanged into oracle/_ref/src/, puts the
// stand-in headers of oracle/refstub/ (glm, core/Buffer.h, core/Model.h)
// beside them, and compiles them with this file into oracle/_ref/.  The
// builder that runs here is therefore BVH::build() itself
// (src/accelerator/BVH.cpp:116-144): quickBuild (:217-296) and buildHitTable
// (:298-345), with the AABB operations of src/accelerator/AABB.cpp.
#include <cstdint>
#include <vector>

#include "accelerator/BVH.h"

extern "C" {

// PackedBVH of BVH(vertices, indices).build(): bounds as float[M][6]
// (pMin.xyz, pMax.xyz), hitTable as int32[6][M][3].  Returns M, or -1 for an
// empty mesh, which the reference does not handle (its tree size
// primInfo.size() * 2 - 1 wraps around).
int64_t ref_bvh_build(const float* vertices, int64_t n_vertices, const uint32_t* indices, int64_t n_triangles,
                      float* bounds, int32_t* hit_table) {
    if (n_triangles <= 0) return -1;
    std::vector<glm::vec3> v((size_t)n_vertices);
    for (int64_t i = 0; i < n_vertices; i++)
        v[(size_t)i] = glm::vec3(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]);
    std::vector<uint32_t> idx(indices, indices + 3 * n_triangles);
    PackedBVH p = BVH(v, idx).build();
    const int64_t M = (int64_t)p.bounds.size();
    for (int64_t k = 0; k < M; k++) {
        const AABB& b = p.bounds[(size_t)k];
        float* o = bounds + 6 * k;
        o[0] = b.pMin.x;
        o[1] = b.pMin.y;
        o[2] = b.pMin.z;
        o[3] = b.pMax.x;
        o[4] = b.pMax.y;
        o[5] = b.pMax.z;
    }
    for (size_t i = 0; i < p.hitTable.size(); i++) hit_table[i] = p.hitTable[i];
    return M;
}

}  // extern "C"
