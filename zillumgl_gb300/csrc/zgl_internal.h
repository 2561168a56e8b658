// zgl_internal.h — shared plumbing of libzgl: status/error reporting and
// CUDA error checks.  Every C entry point returns a zgl_status and records a
// thread-local message; nothing aborts (the reference's Error::check aborts,
// src/util/Error.h:35-42).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/zgl.h"

namespace zgl {

void set_error(const char* fmt, ...);
void clear_error();

struct Error {
    zgl_status code;
};

// Throwing helpers, used inside a try block of each entry point.
[[noreturn]] void fail(zgl_status code, const char* fmt, ...);

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation) fail(ZGL_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
        fail(ZGL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
}

// A named range over an entry point, shown on nsys / ncu timelines (NVTX;
// costs nothing unless a tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace zgl

#define ZGL_CUDA(call) ::zgl::cuda_check((call), #call)
#define ZGL_RANGE(name) ::zgl::NvtxRange zgl_nvtx_range_(name)

// Wraps the body of an extern "C" entry point.
#define ZGL_API_BEGIN \
    try {             \
        ::zgl::clear_error();
#define ZGL_API_END                                            \
    }                                                          \
    catch (const ::zgl::Error& e) {                            \
        return e.code;                                         \
    }                                                          \
    catch (const std::bad_alloc&) {                            \
        ::zgl::set_error("host allocation failed");            \
        return ZGL_ERR_OOM;                                    \
    }                                                          \
    catch (...) {                                              \
        ::zgl::set_error("unexpected internal exception");     \
        return ZGL_ERR_STATE;                                  \
    }                                                          \
    return ZGL_OK;
