// Host-side helpers shared by the entry points: error reporting, launch checks.
#pragma once

#include <stdarg.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#include <initializer_list>

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

// Bytes of one stored value (NGT_F32 / F64 / BF16 / F16) and of one value of the
// type the kernels compute, write images and accumulate gradients in (float;
// double for F64).
inline size_t storage_bytes(int dtype) { return dtype == NGT_F64 ? 8 : dtype == NGT_F32 ? 4 : 2; }
inline size_t arith_bytes(int dtype) { return dtype == NGT_F64 ? 8 : 4; }

// Device buffers start on a multiple of their element size; workspaces and
// camera blocks on kScratchAlign bytes (they hold 16-byte vector data).  A
// misaligned buffer would fault in the kernels, so it is rejected here.
constexpr size_t kScratchAlign = 16;

struct NamedPtr {
  const char* name;
  const void* p;
};

// NGT_ERR_INVALID_ARGUMENT naming the first of ``ptrs`` that is not a multiple
// of ``bytes``; null pointers pass (each caller checks the ones it needs).
inline int check_aligned(const char* op, size_t bytes, std::initializer_list<NamedPtr> ptrs) {
  for (const NamedPtr& q : ptrs)
    if (reinterpret_cast<uintptr_t>(q.p) % bytes != 0)
      return fail(NGT_ERR_INVALID_ARGUMENT, "%s: %s is not aligned to %zu bytes", op, q.name, bytes);
  return NGT_OK;
}

}  // namespace ngt
