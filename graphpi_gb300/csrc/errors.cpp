// Thread-local last-error message of the C ABI (gpm_last_error).  Shared by
// the engine library and the standalone generator library.
#include <cstdarg>
#include <cstdio>
#include <string>

#include "gpm_internal.h"

namespace gpm {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

}  // namespace gpm

extern "C" GPM_API const char* gpm_last_error(void) { return gpm::g_last_error.c_str(); }
