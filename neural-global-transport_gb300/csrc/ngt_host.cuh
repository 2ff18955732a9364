// Host-side helpers shared by the entry points: error reporting, launch checks.
#pragma once

#include <stdarg.h>
#include <stdio.h>

#include "ngt_ops.h"

namespace ngt {

void set_error_v(const char* fmt, va_list ap);

inline int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  set_error_v(fmt, ap);
  va_end(ap);
  return code;
}

inline int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(NGT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return NGT_OK;
}

inline bool valid_channels(int64_t c) { return c == 1 || c == 2 || c == 4; }

inline bool positive_shape(const int64_t* s, int n) {
  for (int i = 0; i < n; ++i)
    if (s[i] <= 0) return false;
  return true;
}

inline unsigned ceil_div_u(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace ngt
