// Library-wide entry points: last-error message and version.
#include <stdio.h>
#include <string.h>

#include "ngt_host.cuh"

namespace ngt {
namespace {
thread_local char g_msg[512] = "";
}
void set_error_v(const char* fmt, va_list ap) { vsnprintf(g_msg, sizeof(g_msg), fmt, ap); }
}  // namespace ngt

extern "C" const char* ngt_last_error_message(void) { return ngt::g_msg; }
extern "C" int ngt_version(void) { return 1; }
