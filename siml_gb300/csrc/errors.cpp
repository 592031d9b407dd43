// Thread-local last-error message behind siml_last_error().
#include <cstdarg>
#include <cstdio>
#include <string>

#include "siml_internal.h"

namespace siml {

static thread_local std::string t_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return code;
}

void clear_error() { t_last_error.clear(); }

}  // namespace siml

extern "C" const char* siml_last_error(void) { return siml::t_last_error.c_str(); }
