// Host execution of the reference's CUDA device code (test infrastructure).
//
// The reference's samplers, blends, transforms and kernel bodies are plain
// CUDA C++; compiled as host C++ after this prelude they run sequentially on
// the CPU: the CUDA qualifiers become empty, thread / block indices are
// globals that the harness driver sets before calling a kernel body for each
// thread, atomics are plain read-modify-writes (execution is sequential), and
// copies to __constant__ symbols are memcpy into ordinary globals.
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <iostream>
#include <algorithm>
#undef __device__
#define __device__
#undef __host__
#define __host__
#undef __constant__
#define __constant__
#undef __global__
#define __global__
#undef __launch_bounds__
#define __launch_bounds__(...)
using std::max;
using std::min;

static uint3 threadIdx, blockIdx;
static dim3 blockDim, gridDim;

static inline float atomicAdd(float* a, float v) { float o = *a; *a = o + v; return o; }
static inline unsigned atomicInc(unsigned* a, unsigned m) { unsigned o = *a; *a = (o >= m) ? 0u : o + 1u; return o; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
static inline float __fsub_rn(float a, float b) { return a - b; }

template <class S>
static inline cudaError_t ref_memcpy_to_symbol(S& sym, const void* src, size_t n, size_t off = 0,
                                               cudaMemcpyKind = cudaMemcpyHostToDevice) {
  std::memcpy(reinterpret_cast<char*>(&sym) + off, src, n);
  return cudaSuccess;
}
#define cudaMemcpyToSymbol ref_memcpy_to_symbol
#define checkCudaErrors(x) (x)

// Run ``body`` once per thread of a grid, in block-major order.
template <class F>
static void emu_launch(dim3 grid, dim3 block, F&& body) {
  gridDim = grid;
  blockDim = block;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = make_uint3(bx, by, bz);
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx) {
              threadIdx = make_uint3(tx, ty, tz);
              body();
            }
      }
}
