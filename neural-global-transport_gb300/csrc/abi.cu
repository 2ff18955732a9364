// Library-wide entry points: last-error message, version and argument-struct sizes.
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

extern "C" size_t ngt_struct_size(const char* name) {
  if (!name) return 0;
  struct Entry {
    const char* name;
    size_t size;
  };
  static const Entry kSizes[] = {
      {"ngt_sample_lut_args", sizeof(ngt_sample_lut_args)},
      {"ngt_sample_lut_grad_args", sizeof(ngt_sample_lut_grad_args)},
      {"ngt_sample_transform_args", sizeof(ngt_sample_transform_args)},
      {"ngt_sample_transform_grad_args", sizeof(ngt_sample_transform_grad_args)},
      {"ngt_lod_args", sizeof(ngt_lod_args)},
      {"ngt_raymarch_args", sizeof(ngt_raymarch_args)},
      {"ngt_raymarch_grad_args", sizeof(ngt_raymarch_grad_args)},
      {"ngt_reduce_blend_args", sizeof(ngt_reduce_blend_args)},
      {"ngt_reduce_blend_grad_args", sizeof(ngt_reduce_blend_grad_args)},
      {"ngt_advect_args", sizeof(ngt_advect_args)},
      {"ngt_advect_grad_args", sizeof(ngt_advect_grad_args)},
      {"ngt_advect_velocity_args", sizeof(ngt_advect_velocity_args)},
      {"ngt_advect_velocity_grad_args", sizeof(ngt_advect_velocity_grad_args)},
  };
  for (const Entry& e : kSizes)
    if (strcmp(e.name, name) == 0) return e.size;
  return 0;
}
