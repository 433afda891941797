// Error reporting and version string of the library.
#include <stdarg.h>

#include "gbcommon.cuh"

static thread_local char g_err[512] = "";

void gb_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" const char *gb_last_error(void) { return g_err; }

extern "C" const char *gb_version(void)
{
    return "gb300conv 0.1 sm_103a (fp64 paths built with -fmad=false; explicit fma only)";
}
