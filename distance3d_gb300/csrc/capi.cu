// capi.cu -- ABI version and the per-thread error message.
#include <stdarg.h>
#include <stdio.h>

#include "capi_util.h"

namespace {
thread_local char g_error[512] = "";
}

namespace d3d {
void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}
}  // namespace d3d

extern "C" int d3d_abi_version(void) { return D3D_ABI_VERSION; }

extern "C" const char* d3d_last_error(void) { return g_error; }
