// Deterministic gather form of the trilinear scatter adjoint.
//
// The atomic scatter (one float atomicAdd per sample corner) gives results that
// depend on the order the atomics land.  Here the samples are bucketed by the
// cell of their floor corner (counting sort: integer counts, a prefix sum, a fill
// and a per-bucket sort by sample index), then every voxel sums the contributions
// of the samples in the 8 buckets whose floor cell can reach it, in a fixed order.
// Same sums in the same order on every run: bit-reproducible gradients.
//
// A sample source provides, for sample s, its position (cell-centred, xyz) and
// its C-channel value; it returns false for samples that contribute nothing.
#pragma once

#include <algorithm>

#include "ngt_common.cuh"

namespace ngt {
namespace {  // kernels here are instantiated per translation unit

constexpr int kGatherBlock = 256;
constexpr int kScanBlock = 1024;

// floor cell of a sample, as a key in a (dims [+1 for BORDER]) lattice
template <class S>
__device__ __forceinline__ int64_t home_key(const Tri<S>& t, const S p[3], const Dims& d, int bm) {
  int h[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int n = a == 0 ? d.x : (a == 1 ? d.y : d.z);
    const int f = to_int_rz(floor(p[a]));
    if (bm == BORDER) h[a] = f + 1;  // floor in [-1, n-1] for samples inside the domain
    else h[a] = t.i0[a];             // clamped or wrapped floor corner
    (void)n;
  }
  const int ex = bm == BORDER ? 1 : 0;
  return (int64_t(h[2]) * (d.y + ex) + h[1]) * (d.x + ex) + h[0];
}

__host__ __device__ __forceinline__ int64_t key_count(const Dims& d, int bm) {
  const int ex = bm == BORDER ? 1 : 0;
  return int64_t(d.x + ex) * (d.y + ex) * (d.z + ex);
}

template <int C, class S, class SRC>
__global__ void __launch_bounds__(kGatherBlock) k_gather_count(SRC src, int64_t nsamples, Dims d, int bm,
                                                               int* __restrict__ keys, int* __restrict__ count) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= nsamples) return;
  S p[3], g[C];
  int key = -1;
  if (src(s, p, g)) {
    const Tri<S> t = tri_setup(p[0], p[1], p[2], d, bm);
    if (!(bm == BORDER && !t.inside)) {
      key = int(home_key(t, p, d, bm));
      atomicAdd(count + key, 1);
    }
  }
  keys[s] = key;
}

// exclusive scan of n ints in three passes (block scan, scan of block sums, add)
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(const int* __restrict__ in, int* __restrict__ out,
                                                            int* __restrict__ sums, int64_t n) {
  __shared__ int warp_tot[kScanBlock / 32];
  const int64_t i = int64_t(blockIdx.x) * kScanBlock + threadIdx.x;
  const int v = i < n ? in[i] : 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  const int incl = x + (w > 0 ? warp_tot[w - 1] : 0);
  if (i < n) out[i] = incl - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_sums(int* __restrict__ sums, int64_t nb, int* __restrict__ total) {
  // one block: serial over chunks of kScanBlock, carrying the running total
  __shared__ int warp_tot[kScanBlock / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += kScanBlock) {
    const int64_t i = base + threadIdx.x;
    const int v = i < nb ? sums[i] : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    const int incl = x + (w > 0 ? warp_tot[w - 1] : 0);
    const int c = carry;
    if (i < nb) sums[i] = c + incl - v;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_add(int* __restrict__ out, const int* __restrict__ sums, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

__global__ void __launch_bounds__(kGatherBlock) k_gather_fill(const int* __restrict__ keys, int64_t nsamples,
                                                              const int* __restrict__ offset, int* __restrict__ cursor,
                                                              int* __restrict__ list) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= nsamples) return;
  const int key = keys[s];
  if (key < 0) return;
  const int pos = atomicAdd(cursor + key, 1);
  list[offset[key] + pos] = int(s);
}

// order each bucket by sample index (buckets hold a handful of samples)
__global__ void __launch_bounds__(kGatherBlock) k_gather_sort(const int* __restrict__ offset,
                                                              const int* __restrict__ count, int* __restrict__ list,
                                                              int64_t nkeys) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= nkeys) return;
  int* b = list + offset[k];
  const int n = count[k];
  for (int i = 1; i < n; ++i) {
    const int v = b[i];
    int j = i - 1;
    while (j >= 0 && b[j] > v) {
      b[j + 1] = b[j];
      --j;
    }
    b[j + 1] = v;
  }
}

// grad[v] = sum over the buckets of v - {0,1}^3 of the corner weights that land on v
template <int C, class S, class SRC>
__global__ void __launch_bounds__(kGatherBlock) k_gather_sum(SRC src, Dims d, int bm, const int* __restrict__ offset,
                                                             const int* __restrict__ count,
                                                             const int* __restrict__ list, S* __restrict__ grad,
                                                             int accumulate) {
  const int64_t v = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= d.count()) return;
  const int vx = int(v % d.x), vy = int((v / d.x) % d.y), vz = int(v / (int64_t(d.x) * d.y));
  const int ex = bm == BORDER ? 1 : 0;
  S acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = S(0);
  for (int k = 0; k < 8; ++k) {
    int h[3] = {vx - (k & 1), vy - ((k >> 1) & 1), vz - ((k >> 2) & 1)};
    const int n[3] = {d.x, d.y, d.z};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (bm == WRAP) h[a] = wrap_index(h[a], n[a]);
      else if (bm == BORDER) h[a] += 1;
      else ok = ok && h[a] >= 0;
    }
    if (!ok) continue;
    // with wrap on an axis of size 1 or 2, two offsets can name the same bucket
    bool dup = false;
    for (int k2 = 0; k2 < k && bm == WRAP; ++k2) {
      int h2[3] = {vx - (k2 & 1), vy - ((k2 >> 1) & 1), vz - ((k2 >> 2) & 1)};
      bool same = true;
#pragma unroll
      for (int a = 0; a < 3; ++a) same = same && wrap_index(h2[a], n[a]) == h[a];
      dup = dup || same;
    }
    if (dup) continue;
    const int64_t key = (int64_t(h[2]) * (d.y + ex) + h[1]) * (d.x + ex) + h[0];
    const int o = offset[key], cnt = count[key];
    for (int j = 0; j < cnt; ++j) {
      const int s = list[o + j];
      S p[3], g[C];
      src(s, p, g);
      const Tri<S> t = tri_setup(p[0], p[1], p[2], d, bm);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        bool valid;
        const int64_t idx = tri_corner(t, q, d, valid);
        if (!valid || idx != v) continue;
        const S w = tri_weight(t, q);
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = add_rn(acc[c], mul_rn(g[c], w));
      }
    }
  }
#pragma unroll
  for (int c = 0; c < C; ++c) {
    if (accumulate) grad[v * C + c] = add_rn(grad[v * C + c], acc[c]);
    else grad[v * C + c] = acc[c];
  }
}

// Workspace of one deterministic gather over ``nsamples`` samples into a grid d.
struct GatherWork {
  int* keys;     // nsamples
  int* count;    // nkeys
  int* offset;   // nkeys
  int* cursor;   // nkeys
  int* list;     // nsamples
  int* sums;     // ceil(nkeys / kScanBlock)
};

__host__ inline size_t gather_bytes(int64_t nsamples, const Dims& d, int bm) {
  const int64_t nk = key_count(d, bm);
  const int64_t nb = (nk + kScanBlock - 1) / kScanBlock;
  return size_t(2 * nsamples + 3 * nk + nb + 64) * sizeof(int);
}

__host__ inline GatherWork gather_layout(void* ws, int64_t nsamples, const Dims& d, int bm) {
  const int64_t nk = key_count(d, bm);
  int* p = static_cast<int*>(ws);
  GatherWork w;
  w.keys = p;
  p += nsamples;
  w.count = p;
  p += nk;
  w.offset = p;
  p += nk;
  w.cursor = p;
  p += nk;
  w.list = p;
  p += nsamples;
  w.sums = p;
  return w;
}

// Enqueue the full deterministic adjoint: grad (+)= gather of the sources' samples.
// Returns the status of the enqueueing (the launches' own errors surface in the
// caller's launch check).
template <int C, class S, class SRC>
__host__ inline cudaError_t gather_adjoint(const SRC& src, int64_t nsamples, const Dims& d, int bm, void* ws, S* grad,
                                           int accumulate, cudaStream_t st) {
  const int64_t nk = key_count(d, bm);
  const int64_t nb = (nk + kScanBlock - 1) / kScanBlock;
  GatherWork w = gather_layout(ws, nsamples, d, bm);
  cudaError_t e = cudaMemsetAsync(w.count, 0, size_t(nk) * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.cursor, 0, size_t(nk) * sizeof(int), st);
  if (e != cudaSuccess) return e;
  const unsigned gs = unsigned((nsamples + kGatherBlock - 1) / kGatherBlock);
  k_gather_count<C, S, SRC><<<gs, kGatherBlock, 0, st>>>(src, nsamples, d, bm, w.keys, w.count);
  k_scan_blocks<<<unsigned(nb), kScanBlock, 0, st>>>(w.count, w.offset, w.sums, nk);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(w.sums, nb, nullptr);
  k_scan_add<<<unsigned(nb), kScanBlock, 0, st>>>(w.offset, w.sums, nk);
  k_gather_fill<<<gs, kGatherBlock, 0, st>>>(w.keys, nsamples, w.offset, w.cursor, w.list);
  k_gather_sort<<<unsigned((nk + kGatherBlock - 1) / kGatherBlock), kGatherBlock, 0, st>>>(w.offset, w.count, w.list,
                                                                                            nk);
  k_gather_sum<C, S, SRC><<<unsigned((d.count() + kGatherBlock - 1) / kGatherBlock), kGatherBlock, 0, st>>>(
      src, d, bm, w.offset, w.count, w.list, grad, accumulate);
  return cudaSuccess;
}

// ------------------------------------------------------------ fixed-point form
// The same adjoint as a scatter whose sums do not depend on the order of the
// additions: every contribution g * w is rounded to an integer at the scale 2^E
// and added with a 64-bit integer atomic (integer addition is associative), and a
// last pass converts the sums.  A first pass takes the largest |value| of the
// samples, g_max < 2^eg; a sample's corner weights to one cell sum to at most 1,
// so no cell's sum passes nsamples * g_max, and E = 62 - eg - en with
// nsamples <= 2^en keeps it below 2^62 while resolving each contribution to
// 2^(en - 62) of g_max.  One pass over the samples, against the counting sort's
// count, scan, fill and sort and a sum that sets every sample up again for each
// of its eight corner cells.  A value that is not finite makes every cell of the
// result NaN (the float scatter would spread it to some).

__host__ inline size_t fixed_bytes(const Dims& d, int C) { return size_t(d.count()) * size_t(C) * 8 + 256; }

__device__ __forceinline__ int fixed_exponent(unsigned gmax_bits, int64_t nsamples) {
  const float g = __uint_as_float(gmax_bits);
  if (!(g > 0.0f)) return 0;
  int eg;
  frexpf(g, &eg);  // g = m * 2^eg, m in [0.5, 1): every |value| (rounded to float: at most g) is below 2^eg
  const unsigned long long n = (unsigned long long)(nsamples > 1 ? nsamples : 1);
  const int en = n > 1 ? 64 - __clzll(n - 1) : 0;
  return 62 - eg - en;
}

template <int C, class S, class SRC>
__global__ void __launch_bounds__(kGatherBlock) k_fixed_max(SRC src, int64_t nsamples, unsigned* __restrict__ gmax) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned m = 0u;  // bits of |value| as float: ordered as integers, NaN and inf above every finite value
  S p[3], g[C];
  if (s < nsamples && src(s, p, g)) {
#pragma unroll
    for (int c = 0; c < C; ++c) m = max(m, __float_as_uint(fabsf(float(g[c]))));
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(gmax, m);
}

template <int C, class S, class SRC>
__global__ void __launch_bounds__(kGatherBlock) k_fixed_scatter(SRC src, int64_t nsamples, Dims d, int bm,
                                                                const unsigned* __restrict__ gmax,
                                                                unsigned long long* __restrict__ fix) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= nsamples) return;
  const unsigned gb = *gmax;
  if (gb == 0u || gb >= 0x7f800000u) return;  // all zero, or not finite
  const int e = fixed_exponent(gb, nsamples);
  S p[3], g[C];
  if (!src(s, p, g)) return;
  const Tri<S> t = tri_setup(p[0], p[1], p[2], d, bm);
  if (bm == BORDER && !t.inside) return;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    bool valid;
    const int64_t idx = tri_corner(t, q, d, valid);
    if (!valid) continue;
    const S w = tri_weight(t, q);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const long long v = fixed_of(mul_rn(g[c], w), e);
      if (v) atomicAdd(fix + idx * C + c, (unsigned long long)v);
    }
  }
}

template <class S>
__global__ void k_fixed_convert(const unsigned long long* __restrict__ fix, const unsigned* __restrict__ gmax,
                                int64_t nsamples, S* __restrict__ grad, int64_t n, int accumulate) {
  const unsigned gb = *gmax;
  const int e = fixed_exponent(gb, nsamples);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    S v;
    fixed_value((long long)fix[i], e, v);
    if (gb >= 0x7f800000u) v = S(NAN);
    grad[i] = accumulate ? add_rn(grad[i], v) : v;
  }
}

// Enqueue the fixed-point deterministic adjoint: grad (+)= the samples' scatter.
// ``ws``: fixed_bytes(d, C) bytes, 8-byte aligned.  Returns the status of the
// enqueueing (the launches' own errors surface in the caller's launch check).
template <int C, class S, class SRC>
__host__ inline cudaError_t fixed_adjoint(const SRC& src, int64_t nsamples, const Dims& d, int bm, void* ws, S* grad,
                                          int accumulate, cudaStream_t st) {
  unsigned long long* fix = static_cast<unsigned long long*>(ws);
  unsigned* gmax = reinterpret_cast<unsigned*>(fix + d.count() * C);
  const cudaError_t e = cudaMemsetAsync(ws, 0, fixed_bytes(d, C), st);
  if (e != cudaSuccess) return e;
  const unsigned gs = unsigned((nsamples + kGatherBlock - 1) / kGatherBlock);
  k_fixed_max<C, S, SRC><<<gs, kGatherBlock, 0, st>>>(src, nsamples, gmax);
  k_fixed_scatter<C, S, SRC><<<gs, kGatherBlock, 0, st>>>(src, nsamples, d, bm, gmax, fix);
  const int64_t n = d.count() * C;
  const unsigned nb = unsigned(std::min<int64_t>((n + 255) / 256, 152 * 16));
  k_fixed_convert<S><<<nb, 256, 0, st>>>(fix, gmax, nsamples, grad, n, accumulate);
  return cudaSuccess;
}

}  // namespace
}  // namespace ngt
