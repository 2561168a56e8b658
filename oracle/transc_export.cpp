// transc_export.cpp — C ABI over the oracle's transcendental functions so that
// tests can check their accuracy and compare them with the CUDA copies.
// TEST INFRASTRUCTURE ONLY.
#include <cstdint>

#include "oracle_transc.h"

extern "C" {

// op: 0 sin, 1 cos, 2 atan2(a, b), 3 log, 4 exp2, 5 pow(a, b), 6 atan(a)
void orc_transc(int32_t op, const float* a, const float* b, float* out, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        float x = a[i], y = b ? b[i] : 0.0f, r = 0.0f;
        switch (op) {
            case 0: r = orc::zsin(x); break;
            case 1: r = orc::zcos(x); break;
            case 2: r = orc::zatan2(x, y); break;
            case 3: r = orc::zlog(x); break;
            case 4: r = orc::zexp2(x); break;
            case 5: r = orc::zpow(x, y); break;
            case 6: r = orc::zatan(x); break;
        }
        out[i] = r;
    }
}

}  // extern "C"
