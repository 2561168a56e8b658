// common.cpp — error reporting and version of libzgl.
#include <cstdarg>
#include <cstdio>
#include <new>

#include "zgl_internal.h"

namespace zgl {

thread_local char g_last_error[1024] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

void clear_error() { g_last_error[0] = '\0'; }

void fail(zgl_status code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    throw Error{code};
}

}  // namespace zgl

extern "C" {

int32_t zgl_version(void) { return 100; }

const char* zgl_last_error(void) { return zgl::g_last_error; }

}  // extern "C"
