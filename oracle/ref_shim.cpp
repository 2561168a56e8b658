// ref_shim.cpp — exposes the two reference headers that compile on their own
// (src/math/AliasTable.h and src/math/SobolMatrices256x32.h) through a C ABI so
// that tests can pin the oracle and the product against the reference code
// itself.  Compiled by oracle/build_oracle.py from the headers where they lie
// in the reference tree; the output goes to oracle/_ref/ and is never
// committed.  TEST INFRASTRUCTURE ONLY.
#include <cstdint>
#include <vector>

#include "math/AliasTable.h"
#include "math/SobolMatrices256x32.h"

extern "C" {

// AliasTable::build<int32_t>(pdf) (src/math/AliasTable.h:12-54).
int32_t ref_alias_build(const float* pdf, int32_t n, int32_t* alias, float* prob) {
    std::vector<float> p(pdf, pdf + n);
    auto res = AliasTable::build<int32_t>(p);
    for (int32_t i = 0; i < n; i++) {
        alias[i] = res.first[(size_t)i];
        prob[i] = res.second[(size_t)i];
    }
    return n;
}

// SobolMatrices[256 * 32] (src/math/SobolMatrices256x32.h:5-7).
int32_t ref_sobol_matrices(uint32_t* out, int32_t cap) {
    int32_t n = SobolMatricesDim * SobolMatricesSize;
    for (int32_t i = 0; i < n && i < cap; i++) out[i] = SobolMatrices[i];
    return n;
}

}  // extern "C"
