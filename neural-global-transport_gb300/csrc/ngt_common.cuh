// Shared device code of the grid operators (sm_103a).
//
// Layout: grids are NDHWC with x fastest; a single grid slice is addressed as
// ((z*H + y)*W + x)*C + c.  Positions are xyz in cell units with cell centres
// at integer coordinates (callers subtract the cell-centre offset first).
//
// Sampler arithmetic uses explicitly rounded operations (no FMA contraction)
// in the order of the reference's interpolation code, so that a float32
// evaluation matches an op-by-op IEEE evaluation bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace ngt {

enum Boundary : int { BORDER = 0, CLAMP = 1, WRAP = 2 };
enum Filter : int { NEAREST = 0, LINEAR = 1, FMIN = 2, FMAX = 3, QUADRATIC = 4 };
enum Blend : int { BEER_LAMBERT = 0, ALPHA = 2, ALPHA_ADDITIVE = 3, ADDITIVE = 4 };

// Start value of the running extremum (vectormath.hpp:13-19: 3.40282e+38 narrowed to float).
constexpr float kFloatMax = 3.40282e38f;

// ------------------------------------------------------------ exact arithmetic
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// a + t*(b-a), rounded after every operation (vectormath_helper.hpp:246-248)
template <class S>
__device__ __forceinline__ S lerp_rn(S a, S b, S t) { return add_rn(a, mul_rn(t, sub_rn(b, a))); }

// ------------------------------------------------------------ storage types
// Compute scalar of a storage type: double stays double, everything else is float.
template <class T> struct Compute { typedef float type; };
template <> struct Compute<double> { typedef double type; };

template <class T>
__device__ __forceinline__ typename Compute<T>::type ld(const T* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }
template <>
__device__ __forceinline__ float ld<__half>(const __half* p) { return __half2float(__ldg(p)); }

template <class T>
__device__ __forceinline__ T from_compute(typename Compute<T>::type v) { return T(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_compute<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <>
__device__ __forceinline__ __half from_compute<__half>(float v) { return __float2half_rn(v); }

template <class S> __device__ __forceinline__ void atomic_add(S* p, S v) { atomicAdd(p, v); }

// ------------------------------------------------------ fixed-point sums
// A value at the scale 2^e as a 64-bit integer (for order-independent integer
// atomic sums), and an integer sum back, in the data's own arithmetic: float data
// never goes through double (slow on this GPU); scaling by a power of two is
// exact, so the integer is the one a double evaluation would give.
__device__ __forceinline__ long long fixed_of(float v, int e) { return __float2ll_rn(ldexpf(v, e)); }
__device__ __forceinline__ long long fixed_of(double v, int e) { return __double2ll_rn(ldexp(v, e)); }
__device__ __forceinline__ void fixed_value(long long q, int e, float& v) { v = ldexpf(__ll2float_rn(q), -e); }
__device__ __forceinline__ void fixed_value(long long q, int e, double& v) { v = ldexp(__ll2double_rn(q), -e); }

// --------------------------------------------------------------- grid dims
struct Dims {
  int x, y, z;  // W, H, D
  __device__ __host__ int64_t count() const { return int64_t(x) * y * z; }
};

// Cell-parallel launches without integer division: threads (bx, by) over x and
// y, blockIdx.z over z; bx a multiple of 32, so a warp is 32 consecutive x cells
// of one row.
struct CellLaunch {
  dim3 grid, block;
};

inline CellLaunch cell_launch(const Dims& d) {
  const int bx = d.x >= 256 ? 256 : ((d.x + 31) / 32) * 32;
  int by = 256 / bx;
  if (by > d.y) by = d.y;
  CellLaunch l;
  l.block = dim3(unsigned(bx), unsigned(by), 1);
  l.grid = dim3(unsigned((d.x + bx - 1) / bx), unsigned((d.y + by - 1) / by), unsigned(d.z));
  return l;
}

// This thread's cell of a cell_launch grid; false for padding threads.
__device__ __forceinline__ bool launch_cell(const Dims& d, int& x, int& y, int& z) {
  x = int(blockIdx.x * blockDim.x + threadIdx.x);
  y = int(blockIdx.y * blockDim.y + threadIdx.y);
  z = int(blockIdx.z);
  return x < d.x && y < d.y;
}

__device__ __forceinline__ int64_t flat(int x, int y, int z, const Dims& d) {
  return (int64_t(z) * d.y + y) * d.x + x;
}

__device__ __forceinline__ int wrap_index(int i, int n) {
  int m = i % n;
  return m < 0 ? m + n : m;
}

// float -> int conversion as the reference's int casts: truncation toward zero,
// saturating (NaN -> 0), so any index stays representable before clamping.
template <class S> __device__ __forceinline__ int to_int_rz(S v);
template <> __device__ __forceinline__ int to_int_rz<float>(float v) { return __float2int_rz(v); }
template <> __device__ __forceinline__ int to_int_rz<double>(double v) { return __double2int_rz(v); }

// ------------------------------------------------------------- trilinear setup
// Corner indices / validity / weights of a trilinear lookup (sampling.hpp:371-465,
// sampling_v2.hpp:37-124).  BORDER: a sample outside 0 <= p+0.5 < dims reads the
// constant 0; inside, out-of-range corners read 0.  CLAMP clamps, WRAP wraps.
template <class S>
struct Tri {
  int i0[3], i1[3];
  bool ok0[3], ok1[3];
  S w[3];
  bool inside;
};

template <class S>
__device__ __forceinline__ Tri<S> tri_setup(S px, S py, S pz, const Dims& d, int bm) {
  Tri<S> t;
  const S p[3] = {px, py, pz};
  const int n[3] = {d.x, d.y, d.z};
  t.inside = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const S f = floor(p[a]);
    const S c = ceil(p[a]);
    t.w[a] = sub_rn(p[a], f);
    int i0 = to_int_rz(f), i1 = to_int_rz(c);
    bool ok0 = true, ok1 = true;
    if (bm == BORDER) {
      const S q = add_rn(p[a], S(0.5));
      t.inside = t.inside && (q >= S(0)) && (q < S(n[a]));
      ok0 = (i0 > -1) && (i0 < n[a]);
      ok1 = (i1 > -1) && (i1 < n[a]);
      i0 = ok0 ? i0 : 0;
      i1 = ok1 ? i1 : 0;
    } else if (bm == CLAMP) {
      i0 = min(max(i0, 0), n[a] - 1);
      i1 = min(max(i1, 0), n[a] - 1);
    } else {
      i0 = wrap_index(i0, n[a]);
      i1 = wrap_index(i1, n[a]);
    }
    t.i0[a] = i0;
    t.i1[a] = i1;
    t.ok0[a] = ok0;
    t.ok1[a] = ok1;
  }
  return t;
}

// corner k in reference order: x fastest, then y, then z
template <class S>
__device__ __forceinline__ int64_t tri_corner(const Tri<S>& t, int k, const Dims& d, bool& valid) {
  const int sx = k & 1, sy = (k >> 1) & 1, sz = (k >> 2) & 1;
  valid = (sx ? t.ok1[0] : t.ok0[0]) && (sy ? t.ok1[1] : t.ok0[1]) && (sz ? t.ok1[2] : t.ok0[2]);
  return flat(sx ? t.i1[0] : t.i0[0], sy ? t.i1[1] : t.i0[1], sz ? t.i1[2] : t.i0[2], d);
}

template <class S>
__device__ __forceinline__ S tri_weight(const Tri<S>& t, int k) {
  const S cw0 = t.w[0], cw1 = t.w[1], cw2 = t.w[2];
  const S a = (k & 1) ? cw0 : sub_rn(S(1), cw0);
  const S b = ((k >> 1) & 1) ? cw1 : sub_rn(S(1), cw1);
  const S c = ((k >> 2) & 1) ? cw2 : sub_rn(S(1), cw2);
  return mul_rn(mul_rn(a, b), c);
}

// Read the 8 corners of C channels (out-of-range corners read 0).
template <int C, class T, class S>
__device__ __forceinline__ void tri_fetch(const T* __restrict__ g, const Tri<S>& t, const Dims& d, S v[8][C]) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    bool ok;
    const int64_t i = tri_corner(t, k, d, ok);
#pragma unroll
    for (int c = 0; c < C; ++c) v[k][c] = ok ? S(ld(g + i * C + c)) : S(0);
  }
}

// x within each (y, z) pair, then y, then z (sampling.hpp:389-430)
template <int C, class S>
__device__ __forceinline__ void tri_combine(const S v[8][C], const Tri<S>& t, S out[C]) {
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const S v00 = lerp_rn(v[0][c], v[1][c], t.w[0]);
    const S v01 = lerp_rn(v[2][c], v[3][c], t.w[0]);
    const S v0 = lerp_rn(v00, v01, t.w[1]);
    const S v10 = lerp_rn(v[4][c], v[5][c], t.w[0]);
    const S v11 = lerp_rn(v[6][c], v[7][c], t.w[0]);
    const S v1 = lerp_rn(v10, v11, t.w[1]);
    out[c] = lerp_rn(v0, v1, t.w[2]);
  }
}

template <int C, class T, class S>
__device__ __forceinline__ void read_linear(const T* __restrict__ g, S px, S py, S pz, const Dims& d, int bm,
                                            S out[C]) {
  const Tri<S> t = tri_setup(px, py, pz, d, bm);
  if (bm == BORDER && !t.inside) {
#pragma unroll
    for (int c = 0; c < C; ++c) out[c] = S(0);
    return;
  }
  S v[8][C];
  tri_fetch<C>(g, t, d, v);
  tri_combine<C>(v, t, out);
}

// Spatial derivative of the trilinear read (read3DGrad, sampling.hpp:470-565).
template <int C, class S>
__device__ __forceinline__ void tri_gradient(const S v[8][C], const Tri<S>& t, S dx[C], S dy[C], S dz[C]) {
  const S wx = t.w[0], wy = t.w[1], wz = t.w[2];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    // v index: x + 2y + 4z
    dx[c] = lerp_rn(lerp_rn(sub_rn(v[1][c], v[0][c]), sub_rn(v[3][c], v[2][c]), wy),
                    lerp_rn(sub_rn(v[5][c], v[4][c]), sub_rn(v[7][c], v[6][c]), wy), wz);
    dy[c] = lerp_rn(lerp_rn(sub_rn(v[2][c], v[0][c]), sub_rn(v[3][c], v[1][c]), wx),
                    lerp_rn(sub_rn(v[6][c], v[4][c]), sub_rn(v[7][c], v[5][c]), wx), wz);
    dz[c] = lerp_rn(lerp_rn(sub_rn(v[4][c], v[0][c]), sub_rn(v[5][c], v[1][c]), wx),
                    lerp_rn(sub_rn(v[6][c], v[2][c]), sub_rn(v[7][c], v[3][c]), wx), wy);
  }
}

// Nearest read: index = int(p + 0.5), truncating (sampling.hpp:569-584).
template <class S>
__device__ __forceinline__ bool nearest_index(S px, S py, S pz, const Dims& d, int bm, int64_t& idx) {
  int i[3] = {to_int_rz(add_rn(px, S(0.5))), to_int_rz(add_rn(py, S(0.5))), to_int_rz(add_rn(pz, S(0.5)))};
  const int n[3] = {d.x, d.y, d.z};
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (bm == BORDER) {
      ok = ok && i[a] >= 0 && i[a] < n[a];
    } else if (bm == CLAMP) {
      i[a] = min(max(i[a], 0), n[a] - 1);
    } else {
      i[a] = wrap_index(i[a], n[a]);
    }
  }
  idx = ok ? flat(i[0], i[1], i[2], d) : 0;
  return ok;
}

template <int C, class T, class S>
__device__ __forceinline__ void read_nearest(const T* __restrict__ g, S px, S py, S pz, const Dims& d, int bm,
                                             S out[C]) {
  int64_t i;
  const bool ok = nearest_index(px, py, pz, d, bm, i);
#pragma unroll
  for (int c = 0; c < C; ++c) out[c] = ok ? S(ld(g + i * C + c)) : S(0);
}

// MIN / MAX over the 8 corners (sampling.hpp:585-704).  BORDER: 0 outside the
// domain; the running value starts at 0 when any corner is out of range, else at
// +-FLOAT_MAX; only in-range corners compete.  ``arg`` receives the winning corner
// per channel (-1 for the start value), for the adjoint.
template <int C, class T, class S>
__device__ __forceinline__ void read_extremum(const T* __restrict__ g, S px, S py, S pz, const Dims& d, int bm,
                                              bool is_max, S out[C], int arg[C], int64_t cidx[8]) {
  const Tri<S> t = tri_setup(px, py, pz, d, bm);
  bool any_bad = false;
  bool okk[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    cidx[k] = tri_corner(t, k, d, okk[k]);
    any_bad = any_bad || !okk[k];
  }
  const S start = (bm == BORDER && any_bad) ? S(0) : (is_max ? S(-kFloatMax) : S(kFloatMax));
#pragma unroll
  for (int c = 0; c < C; ++c) {
    out[c] = start;
    arg[c] = -1;
  }
  if (bm == BORDER && !t.inside) {
#pragma unroll
    for (int c = 0; c < C; ++c) out[c] = S(0);
    return;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (!okk[k]) continue;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const S v = S(ld(g + cidx[k] * C + c));
      const bool better = is_max ? (v > out[c]) : (v < out[c]);
      if (better) {
        out[c] = v;
        arg[c] = k;
      }
    }
  }
}

// read_extremum's MIN and MAX of the same position in one pass over the corners.
template <int C, class T, class S>
__device__ __forceinline__ void read_minmax(const T* __restrict__ g, S px, S py, S pz, const Dims& d, int bm,
                                           S mn[C], S mx[C]) {
  const Tri<S> t = tri_setup(px, py, pz, d, bm);
  bool any_bad = false;
  bool okk[8];
  int64_t cidx[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    cidx[k] = tri_corner(t, k, d, okk[k]);
    any_bad = any_bad || !okk[k];
  }
  const bool zero = bm == BORDER && any_bad;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    mn[c] = zero ? S(0) : S(kFloatMax);
    mx[c] = zero ? S(0) : S(-kFloatMax);
  }
  if (bm == BORDER && !t.inside) {
#pragma unroll
    for (int c = 0; c < C; ++c) mn[c] = mx[c] = S(0);
    return;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (!okk[k]) continue;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const S v = S(ld(g + cidx[k] * C + c));
      if (v < mn[c]) mn[c] = v;
      if (v > mx[c]) mx[c] = v;
    }
  }
}

// Adjoint of read_linear for a warp whose lanes hold consecutive x cells (all 32
// lanes call it; ``active`` lanes scatter): when a lane's upper-x corners are the
// next lane's lower-x corners (same cells, same validity), that lane adds them
// to its own before the atomics, so neighbouring samples share one atomic per
// corner.  Same sums as scatter_linear up to the order of the additions.
template <int C, class S>
__device__ __forceinline__ void scatter_linear_warp(S* __restrict__ grad, const Tri<S>& t, const Dims& d, int bm,
                                                    const S g[C], bool active) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const bool on = active && !(bm == BORDER && !t.inside);
  // corner values: lo[j] at x = i0x, hi[j] at x = i1x, j = (y, z) in reference order
  S lo[4][C], hi[4][C];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const S wl = tri_weight(t, 2 * j), wh = tri_weight(t, 2 * j + 1);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      lo[j][c] = on ? mul_rn(g[c], wl) : S(0);
      hi[j][c] = on ? mul_rn(g[c], wh) : S(0);
    }
  }
  // does the previous lane's upper-x column coincide with my lower-x column?
  const int okyz = int(t.ok0[1]) | (int(t.ok1[1]) << 1) | (int(t.ok0[2]) << 2) | (int(t.ok1[2]) << 3);
  const int prev_y0 = __shfl_up_sync(full, t.i0[1], 1), prev_y1 = __shfl_up_sync(full, t.i1[1], 1);
  const int prev_z0 = __shfl_up_sync(full, t.i0[2], 1), prev_z1 = __shfl_up_sync(full, t.i1[2], 1);
  const int prev_ok = __shfl_up_sync(full, okyz | (int(t.ok1[0]) << 4) | (int(on) << 5), 1);
  const int prev_x1 = __shfl_up_sync(full, t.i1[0], 1);
  const bool take = on && lane > 0 && prev_x1 == t.i0[0] && prev_y0 == t.i0[1] && prev_y1 == t.i1[1] &&
                    prev_z0 == t.i0[2] && prev_z1 == t.i1[2] && prev_ok == (okyz | (int(t.ok0[0]) << 4) | (1 << 5));
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const S r = __shfl_up_sync(full, hi[j][c], 1);
      if (take) lo[j][c] += r;
    }
  const bool given = __shfl_down_sync(full, take, 1) && lane < 31;
  if (!on) return;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    bool ok;
    const int64_t il = tri_corner(t, 2 * j, d, ok);
    if (ok) {
#pragma unroll
      for (int c = 0; c < C; ++c) atomic_add(grad + il * C + c, lo[j][c]);
    }
    if (!given) {
      const int64_t ih = tri_corner(t, 2 * j + 1, d, ok);
      if (ok) {
#pragma unroll
        for (int c = 0; c < C; ++c) atomic_add(grad + ih * C + c, hi[j][c]);
      }
    }
  }
}

template <int C, class S>
__device__ __forceinline__ void scatter_linear_warp(S* __restrict__ grad, S px, S py, S pz, const Dims& d, int bm,
                                                    const S g[C], bool active) {
  scatter_linear_warp<C>(grad, tri_setup(px, py, pz, d, bm), d, bm, g, active);
}

// Quadratic B-spline weight (sampling.hpp:247-256)
template <class S>
__device__ __forceinline__ S bspline2(S dist) {
  if (dist < S(0.5)) return S(0.75) - dist * dist;
  if (dist < S(1.5)) {
    const S t = S(1.5) - dist;
    return S(0.5) * t * t;
  }
  return S(0);
}

// 27-tap quadratic B-spline read; BORDER yields 0 (sampling.hpp:268-366).
template <int C, class T, class S>
__device__ __forceinline__ void read_quadratic(const T* __restrict__ g, S px, S py, S pz, const Dims& d, int bm,
                                               S out[C]) {
#pragma unroll
  for (int c = 0; c < C; ++c) out[c] = S(0);
  if (bm == BORDER) return;
  const S p[3] = {px, py, pz};
  const int n[3] = {d.x, d.y, d.z};
  int idx[3][3];
  S w[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int ctr = to_int_rz(floor(add_rn(p[a], S(0.5))));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      int i = ctr - 1 + k;
      w[a][k] = bspline2(fabs(p[a] - S(ctr - 1 + k)));
      idx[a][k] = (bm == CLAMP) ? min(max(i, 0), n[a] - 1) : wrap_index(i, n[a]);
    }
  }
#pragma unroll
  for (int c = 0; c < C; ++c) {
    S acc_z = S(0);
#pragma unroll
    for (int kz = 0; kz < 3; ++kz) {
      S acc_y = S(0);
#pragma unroll
      for (int ky = 0; ky < 3; ++ky) {
        S acc_x = S(0);
#pragma unroll
        for (int kx = 0; kx < 3; ++kx)
          acc_x += w[0][kx] * S(ld(g + flat(idx[0][kx], idx[1][ky], idx[2][kz], d) * C + c));
        acc_y += w[1][ky] * acc_x;
      }
      acc_z += w[2][kz] * acc_y;
    }
    out[c] = acc_z;
  }
}

template <int C, class T, class S>
__device__ __forceinline__ void read_filtered(const T* __restrict__ g, S px, S py, S pz, const Dims& d, int fm, int bm,
                                              S out[C]) {
  if (fm == LINEAR) {
    read_linear<C>(g, px, py, pz, d, bm, out);
  } else if (fm == NEAREST) {
    read_nearest<C>(g, px, py, pz, d, bm, out);
  } else if (fm == QUADRATIC) {
    read_quadratic<C>(g, px, py, pz, d, bm, out);
  } else {
    int arg[C];
    int64_t ci[8];
    read_extremum<C>(g, px, py, pz, d, bm, fm == FMAX, out, arg, ci);
  }
}

// ------------------------------------------------------------- exact adjoints
// Adjoint of read_linear: value[k] * weight[k] added to the 8 corners.
template <int C, class S>
__device__ __forceinline__ void scatter_linear(S* __restrict__ grad, S px, S py, S pz, const Dims& d, int bm,
                                               const S g[C]) {
  const Tri<S> t = tri_setup(px, py, pz, d, bm);
  if (bm == BORDER && !t.inside) return;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    bool ok;
    const int64_t i = tri_corner(t, k, d, ok);
    if (!ok) continue;
    const S w = tri_weight(t, k);
#pragma unroll
    for (int c = 0; c < C; ++c) atomic_add(grad + i * C + c, mul_rn(g[c], w));
  }
}

// The reference's count-normalised scatter (resample_grid.cu.cc:1080-1131): BORDER
// scatters when -1 < p < dims, and every receiving corner counts one sample.
template <int C, class S>
__device__ __forceinline__ void scatter_linear_counted(S* __restrict__ grad, unsigned* __restrict__ count, S px, S py,
                                                       S pz, const Dims& d, int bm, const S g[C]) {
  if (bm == BORDER) {
    if (!(px > S(-1) && px < S(d.x) && py > S(-1) && py < S(d.y) && pz > S(-1) && pz < S(d.z))) return;
  }
  Tri<S> t;
  const S p[3] = {px, py, pz};
  const int n[3] = {d.x, d.y, d.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const S f = floor(p[a]);
    t.w[a] = sub_rn(p[a], f);
    int i0 = to_int_rz(f), i1 = to_int_rz(ceil(p[a]));
    bool ok0 = true, ok1 = true;
    if (bm == BORDER) {
      ok0 = i0 >= 0 && i0 < n[a];
      ok1 = i1 >= 0 && i1 < n[a];
    } else if (bm == CLAMP) {
      i0 = min(max(i0, 0), n[a] - 1);
      i1 = min(max(i1, 0), n[a] - 1);
    } else {
      i0 = wrap_index(i0, n[a]);
      i1 = wrap_index(i1, n[a]);
    }
    t.i0[a] = i0;
    t.i1[a] = i1;
    t.ok0[a] = ok0;
    t.ok1[a] = ok1;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    bool ok;
    const int64_t i = tri_corner(t, k, d, ok);
    if (!ok) continue;
    const S w = tri_weight(t, k);
#pragma unroll
    for (int c = 0; c < C; ++c) atomic_add(grad + i * C + c, mul_rn(g[c], w));
    atomicAdd(count + i, 1u);
  }
}

template <int C, class S>
__device__ __forceinline__ void scatter_nearest(S* __restrict__ grad, S px, S py, S pz, const Dims& d, int bm,
                                                const S g[C]) {
  int64_t i;
  if (!nearest_index(px, py, pz, d, bm, i)) return;
#pragma unroll
  for (int c = 0; c < C; ++c) atomic_add(grad + i * C + c, g[c]);
}

template <int C, class T, class S>
__device__ __forceinline__ void scatter_extremum(S* __restrict__ grad, const T* __restrict__ x, S px, S py, S pz,
                                                 const Dims& d, int bm, bool is_max, const S g[C]) {
  S v[C];
  int arg[C];
  int64_t ci[8];
  read_extremum<C>(x, px, py, pz, d, bm, is_max, v, arg, ci);
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (arg[c] >= 0) atomic_add(grad + ci[arg[c]] * C + c, g[c]);
}

template <int C, class S>
__device__ __forceinline__ void scatter_quadratic(S* __restrict__ grad, S px, S py, S pz, const Dims& d, int bm,
                                                  const S g[C]) {
  if (bm == BORDER) return;
  const S p[3] = {px, py, pz};
  const int n[3] = {d.x, d.y, d.z};
  int idx[3][3];
  S w[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int ctr = to_int_rz(floor(add_rn(p[a], S(0.5))));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int i = ctr - 1 + k;
      w[a][k] = bspline2(fabs(p[a] - S(i)));
      idx[a][k] = (bm == CLAMP) ? min(max(i, 0), n[a] - 1) : wrap_index(i, n[a]);
    }
  }
  for (int kz = 0; kz < 3; ++kz)
    for (int ky = 0; ky < 3; ++ky)
      for (int kx = 0; kx < 3; ++kx) {
        const S wt = w[0][kx] * w[1][ky] * w[2][kz];
        const int64_t i = flat(idx[0][kx], idx[1][ky], idx[2][kz], d);
#pragma unroll
        for (int c = 0; c < C; ++c) atomic_add(grad + i * C + c, g[c] * wt);
      }
}

// The reference's quadratic scatter (resample_grid.cu.cc:903-1078), with the
// out-of-range centre taps that the reference writes out of bounds dropped.
template <int C, class S>
__device__ __forceinline__ void scatter_quadratic_counted(S* __restrict__ grad, unsigned* __restrict__ count, S px,
                                                          S py, S pz, const Dims& d, int bm, const S g[C]) {
  const S p[3] = {px, py, pz};
  const int n[3] = {d.x, d.y, d.z};
  if (bm == BORDER && !(px > S(-1.5) && px < S(d.x) && py > S(-1.5) && py < S(d.y) && pz > S(-1.5) && pz < S(d.z)))
    return;
  int idx[3][3];
  S w[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int ctr = to_int_rz(floor(add_rn(p[a], S(0.5))));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int i = ctr - 1 + k;
      w[a][k] = bspline2(fabs(p[a] - S(i)));
      idx[a][k] = (bm == CLAMP) ? min(max(i, 0), n[a] - 1) : (bm == WRAP ? wrap_index(i, n[a]) : i);
    }
  }
  for (int kz = 0; kz < 3; ++kz)
    for (int ky = 0; ky < 3; ++ky)
      for (int kx = 0; kx < 3; ++kx) {
        if (bm == BORDER) {
          if (kx == 1 && ky == 1 && kz == 1) continue;
          const int ks[3] = {kx, ky, kz};
          bool ok = true;
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const int i = idx[a][ks[a]];
            ok = ok && i >= 0 && i < n[a];
          }
          if (!ok) continue;
        }
        const S wt = w[0][kx] * w[1][ky] * w[2][kz];
        const int64_t i = flat(idx[0][kx], idx[1][ky], idx[2][kz], d);
#pragma unroll
        for (int c = 0; c < C; ++c) atomic_add(grad + i * C + c, g[c] * wt);
        atomicAdd(count + i, 1u);
      }
}

// -------------------------------------------------------------- camera math
// Matrices enter as 16 floats read column-major (transformations.hpp:42-47).
// Per (batch, camera) the kernels need MV = V*M, its inverse and P, P^-1.
struct Cam {
  float mv[16], mvi[16], p[16], pi[16];  // row-major: m[r*4+c]
  float near_, far_;
};

// 3x3 determinant and signed 4x4 cofactor C_ij (row i, column j removed).
__device__ __forceinline__ double det3(double a, double b, double c, double d, double e, double f, double g,
                                       double h, double i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

__device__ __forceinline__ double cofactor4(const double* m, int i, int j) {
  const int r0 = i == 0 ? 1 : 0, r1 = i <= 1 ? 2 : 1, r2 = i <= 2 ? 3 : 2;
  const int c0 = j == 0 ? 1 : 0, c1 = j <= 1 ? 2 : 1, c2 = j <= 2 ? 3 : 2;
  const double d = det3(m[r0 * 4 + c0], m[r0 * 4 + c1], m[r0 * 4 + c2], m[r1 * 4 + c0], m[r1 * 4 + c1],
                        m[r1 * 4 + c2], m[r2 * 4 + c0], m[r2 * 4 + c1], m[r2 * 4 + c2]);
  return ((i + j) & 1) ? -d : d;
}

// Element (r, c) of the inverse by the adjugate: C_cr / det, det expanded along row 0.
__device__ __forceinline__ double inverse_element(const double* m, int r, int c) {
  const double det = m[0] * cofactor4(m, 0, 0) + m[1] * cofactor4(m, 0, 1) + m[2] * cofactor4(m, 0, 2) +
                     m[3] * cofactor4(m, 0, 3);
  return cofactor4(m, c, r) / det;
}

// Scratch of build_cam_warp: M, V, P, MV in double (row-major).
struct CamScratch {
  double M[16], V[16], P[16], MV[16];
};

// Forms ``cam`` cooperatively with the 32 lanes of the calling warp (every lane
// must call it): lanes 0-15 one element each of MV = V*M and of MV^-1, lanes
// 16-31 one element each of P^-1, in double and rounded to float.  M16 may be
// null (identity model matrix).  Inputs are column-major (the reference's
// setTransformations, transformations.hpp:48-68, reads them so); Cam holds
// row-major matrices.
__device__ inline void build_cam_warp(const float* M16, const float* V16, const float* P16, const float* F6,
                                      Cam& cam, CamScratch& sh) {
  const int lane = threadIdx.x & 31;
  const int e = lane & 15, r = e >> 2, c = e & 3;
  if (lane < 16) {
    sh.M[e] = M16 ? (double)M16[c * 4 + r] : (r == c ? 1.0 : 0.0);
    sh.V[e] = (double)V16[c * 4 + r];
  } else {
    sh.P[e] = (double)P16[c * 4 + r];
  }
  __syncwarp();
  if (lane < 16) {
    const double s = sh.V[r * 4 + 0] * sh.M[0 * 4 + c] + sh.V[r * 4 + 1] * sh.M[1 * 4 + c] +
                     sh.V[r * 4 + 2] * sh.M[2 * 4 + c] + sh.V[r * 4 + 3] * sh.M[3 * 4 + c];
    sh.MV[e] = s;
    cam.mv[e] = (float)s;
  } else {
    cam.p[e] = (float)sh.P[e];
  }
  __syncwarp();
  if (lane < 16)
    cam.mvi[e] = (float)inverse_element(sh.MV, r, c);
  else
    cam.pi[e] = (float)inverse_element(sh.P, r, c);
  if (lane == 0) {
    cam.near_ = F6[0];
    cam.far_ = F6[1];
  }
}

__device__ __forceinline__ void mat4_apply(const float* m, const float v[4], float o[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) o[r] = m[r * 4 + 0] * v[0] + m[r * 4 + 1] * v[1] + m[r * 4 + 2] * v[2] + m[r * 4 + 3] * v[3];
}

// IDXtoOS / IDXtoOSlinearDepth (transformations.hpp:124-149): frustum-grid index
// coordinates (already +0.5) to volume object-space coordinates.
__device__ __forceinline__ void idx_to_os(const Cam& cam, float ix, float iy, float iz, const float dinv[3],
                                          bool lin_depth, float os[3]) {
  float ndc[4] = {ix * dinv[0] * 2.0f - 1.0f, iy * dinv[1] * 2.0f - 1.0f, iz * dinv[2] * 2.0f - 1.0f, 1.0f};
  if (lin_depth) {
    const float t = iz * dinv[2];
    const float z = -(cam.near_ + (cam.far_ - cam.near_) * t);
    ndc[2] = -cam.p[2 * 4 + 2] - cam.p[2 * 4 + 3] / z;
  }
  float vs[4], o[4];
  mat4_apply(cam.pi, ndc, vs);
  const float iw = 1.0f / vs[3];
  vs[0] *= iw;
  vs[1] *= iw;
  vs[2] *= iw;
  vs[3] = 1.0f;
  mat4_apply(cam.mvi, vs, o);
  os[0] = o[0];
  os[1] = o[1];
  os[2] = o[2];
}

// OStoIDX / OStoIDXlinearDepth (transformations.hpp:106-121): volume object space
// to frustum-grid index coordinates of a grid with dimensions ``dims``.
__device__ __forceinline__ void os_to_idx(const Cam& cam, float x, float y, float z, const float dims[3], bool lin_depth,
                                          float idx[3]) {
  const float p4[4] = {x, y, z, 1.0f};
  float vs[4], nd[4];
  mat4_apply(cam.mv, p4, vs);
  mat4_apply(cam.p, vs, nd);
  const float iw = 1.0f / nd[3];
  const float n0 = nd[0] * iw, n1 = nd[1] * iw, n2 = nd[2] * iw;
  idx[0] = (n0 * 0.5f + 0.5f) * dims[0];
  idx[1] = (n1 * 0.5f + 0.5f) * dims[1];
  idx[2] = (n2 * 0.5f + 0.5f) * dims[2];
  if (lin_depth) {
    const float zv = -cam.p[2 * 4 + 3] / (n2 + cam.p[2 * 4 + 2]);
    const float t = -(zv + cam.near_) / (cam.far_ - cam.near_);
    idx[2] = t * dims[2];
  }
}

}  // namespace ngt
