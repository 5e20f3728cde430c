// Error reporting and version of the C ABI (include/angelo_gb.h).
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace angelo {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

}  // namespace angelo

extern "C" const char *angelo_last_error_string(void) { return angelo::g_err; }

extern "C" int angelo_version(void) { return 1; }
