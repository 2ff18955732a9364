// Padded (x, y)-quad layout of a one-channel grid for trilinear gathers and
// scatters: two 16-byte (float) or 8-byte (16-bit) accesses per sample instead
// of eight scattered 4-byte ones.
//
// Entry (xq, yq, zq) of a W x H x D grid, xq in [0, W], yq in [0, H], zq in
// [0, D + 1], holds the four cells (x0, y0), (x0 + 1, y0), (x0, y0 + 1),
// (x0 + 1, y0 + 1) of plane z with x0 = xq - 1, y0 = yq - 1, z = zq - 1, in the
// reference's corner order (x fastest, then y).  The boundary rule is applied
// to every corner when the quads are built: BORDER reads 0 outside the grid,
// CLAMP the clamped cell, WRAP the wrapped cell.  A trilinear sample with lower
// corner (x0, y0, z0) reads entry (x0 + 1, y0 + 1) of planes z0 + 1 and z0 + 2,
// after the lower corner is normalised per axis (BORDER: already in [-1, n-1]
// for a sample inside the grid; CLAMP: clamped to [-1, n-1]; WRAP: wrapped to
// [0, n-1]).  The interpolation weights and the lerp order are those of
// read_linear, and the upper corner there is ceil(p) where this layout uses
// floor(p) + 1; the two differ only when the weight of that corner is 0, so for
// finite data the samples are identical.
//
// The adjoint accumulates into a float4 quad grid of the same shape (one
// vector atomic per plane); k_quad_fold then sums, for every cell, the four
// quad components that hold it (plus, for CLAMP and WRAP, the padded entries
// whose corner maps onto it).
#pragma once

#include "ngt_common.cuh"

namespace ngt {

template <class T> struct QuadOf;
template <> struct QuadOf<float> { typedef float4 type; };
template <> struct QuadOf<__nv_bfloat16> { typedef uint2 type; };
template <> struct QuadOf<__half> { typedef uint2 type; };

struct QuadDims {
  int x, y, z;          // W + 1, H + 1, D + 2
  int64_t plane, count;  // entries per plane, per grid
  __device__ __host__ static QuadDims of(const Dims& d) {
    QuadDims q;
    q.x = d.x + 1;
    q.y = d.y + 1;
    q.z = d.z + 2;
    q.plane = int64_t(q.x) * q.y;
    q.count = q.plane * q.z;
    return q;
  }
};

__device__ __forceinline__ int quad_cell(int i, int n, int bm, bool& valid) {
  valid = true;
  if (bm == BORDER) {
    valid = i >= 0 && i < n;
    return valid ? i : 0;
  }
  if (bm == CLAMP) return min(max(i, 0), n - 1);
  return wrap_index(i, n);
}

template <class T>
__device__ __forceinline__ uint32_t raw16(T v) {
  return uint32_t(*reinterpret_cast<const uint16_t*>(&v));
}

// One thread per entry, launched as cell_launch over the padded W+1, H+1 and
// (D+2) * N planes (blockIdx.z = zq + (D+2) * b).
// With ``neg`` set it also raises *neg when scale * value < 0 for some cell (the
// extinction-sign check of the raymarch backward).
template <class T>
__device__ __forceinline__ void quad_build_at(const T* __restrict__ g, const Dims& d, int bm,
                                              typename QuadOf<T>::type* __restrict__ q, int* neg, float scale, int xq,
                                              int yq, int zq, int b) {
  const QuadDims qd = QuadDims::of(d);
  const int64_t e = (int64_t(zq) * qd.y + yq) * qd.x + xq;
  // the two columns, two rows and the plane of this entry, boundary rule applied once each
  bool vz, vx0, vx1, vy0, vy1;
  const int z = quad_cell(zq - 1, d.z, bm, vz);
  const int x0 = quad_cell(xq - 1, d.x, bm, vx0), x1 = quad_cell(xq, d.x, bm, vx1);
  const int y0 = quad_cell(yq - 1, d.y, bm, vy0), y1 = quad_cell(yq, d.y, bm, vy1);
  const T* plane = g + (int64_t(b) * d.z + z) * (int64_t(d.x) * d.y);
  const T* r0 = plane + int64_t(y0) * d.x;
  const T* r1 = plane + int64_t(y1) * d.x;
  const T zero = T(0.0f);
  T v[4];
  v[0] = (vz && vy0 && vx0) ? r0[x0] : zero;
  v[1] = (vz && vy0 && vx1) ? r0[x1] : zero;
  v[2] = (vz && vy1 && vx0) ? r1[x0] : zero;
  v[3] = (vz && vy1 && vx1) ? r1[x1] : zero;
  if (neg) {
    bool n = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) n = n || (scale * float(v[k]) < 0.0f);
    if (__any_sync(__activemask(), n) && n) atomicOr(neg, 1);
  }
  typename QuadOf<T>::type o;
  if constexpr (sizeof(T) == 4) {
    o = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    o.x = raw16(v[0]) | (raw16(v[1]) << 16);
    o.y = raw16(v[2]) | (raw16(v[3]) << 16);
  }
  q[int64_t(b) * qd.count + e] = o;
}

// Planes of entries one thread of k_quad_build fills (the (x, y) boundary
// mapping and the sign vote are then shared by those planes).
constexpr int kQuadPlanes = 8;

// One thread per (xq, yq) and kQuadPlanes consecutive planes of the N * (D + 2)
// planes (blockIdx.z = first plane / kQuadPlanes); quad_build_at's entries.
template <class T>
__global__ void k_quad_build(const T* __restrict__ g, Dims d, int bm, typename QuadOf<T>::type* __restrict__ q,
                             int* neg, float scale, int planes) {
  const QuadDims qd = QuadDims::of(d);
  const int xq = int(blockIdx.x * blockDim.x + threadIdx.x), yq = int(blockIdx.y * blockDim.y + threadIdx.y);
  const bool in = xq < qd.x && yq < qd.y;
  bool vx0 = false, vx1 = false, vy0 = false, vy1 = false;
  int x0 = 0, x1 = 0, y0 = 0, y1 = 0;
  if (in) {
    x0 = quad_cell(xq - 1, d.x, bm, vx0);
    x1 = quad_cell(xq, d.x, bm, vx1);
    y0 = quad_cell(yq - 1, d.y, bm, vy0);
    y1 = quad_cell(yq, d.y, bm, vy1);
  }
  const int64_t plane_cells = int64_t(d.x) * d.y;
  const T zero = T(0.0f);
  bool n = false;
  const int first = int(blockIdx.z) * kQuadPlanes;
#pragma unroll
  for (int k = 0; k < kQuadPlanes; ++k) {
    const int zz = first + k;
    if (!in || zz >= planes) break;
    const int b = zz / qd.z, zq = zz - b * qd.z;
    bool vz;
    const int z = quad_cell(zq - 1, d.z, bm, vz);
    const T* pl = g + (int64_t(b) * d.z + z) * plane_cells;
    const T* r0 = pl + int64_t(y0) * d.x;
    const T* r1 = pl + int64_t(y1) * d.x;
    T v[4];
    v[0] = (vz && vy0 && vx0) ? r0[x0] : zero;
    v[1] = (vz && vy0 && vx1) ? r0[x1] : zero;
    v[2] = (vz && vy1 && vx0) ? r1[x0] : zero;
    v[3] = (vz && vy1 && vx1) ? r1[x1] : zero;
    if (neg) {
#pragma unroll
      for (int c = 0; c < 4; ++c) n = n || (scale * float(v[c]) < 0.0f);
    }
    typename QuadOf<T>::type o;
    if constexpr (sizeof(T) == 4) {
      o = make_float4(v[0], v[1], v[2], v[3]);
    } else {
      o.x = raw16(v[0]) | (raw16(v[1]) << 16);
      o.y = raw16(v[2]) | (raw16(v[3]) << 16);
    }
    q[int64_t(b) * qd.count + (int64_t(zq) * qd.y + yq) * qd.x + xq] = o;
  }
  if (neg && __any_sync(0xffffffffu, n) && n) atomicOr(neg, 1);
}

template <class T>
__device__ __forceinline__ T from_raw16(uint32_t r) {
  const uint16_t h = uint16_t(r);
  return *reinterpret_cast<const T*>(&h);
}

__device__ __forceinline__ void quad_load(const float4* q, int64_t i, float v[4]) {
  const float4 a = __ldg(q + i);
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
  v[3] = a.w;
}

template <class T>
__device__ __forceinline__ void quad_load16(const uint2* q, int64_t i, float v[4]) {
  const uint2 a = __ldg(q + i);
  v[0] = float(from_raw16<T>(a.x & 0xffffu));
  v[1] = float(from_raw16<T>(a.x >> 16));
  v[2] = float(from_raw16<T>(a.y & 0xffffu));
  v[3] = float(from_raw16<T>(a.y >> 16));
}

template <class T>
__device__ __forceinline__ void quad_fetch(const typename QuadOf<T>::type* q, int64_t i, float v[4]) {
  if constexpr (sizeof(T) == 4)
    quad_load(q, i, v);
  else
    quad_load16<T>(q, i, v);
}

// Lower corner and weights of a trilinear sample (tri_setup's arithmetic);
// returns false when BORDER puts the sample outside the grid (it reads 0).
struct QuadPos {
  int64_t idx;  // entry of plane z0 + 1
  float w[3];
};

__device__ __forceinline__ bool quad_setup(float px, float py, float pz, const Dims& d, const QuadDims& qd, int bm,
                                           QuadPos& s) {
  const float p[3] = {px, py, pz};
  const int n[3] = {d.x, d.y, d.z};
  int i0[3];
  bool inside = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float f = floorf(p[a]);
    s.w[a] = sub_rn(p[a], f);
    int i = to_int_rz(f);
    if (bm == BORDER) {
      const float q = add_rn(p[a], 0.5f);
      inside = inside && (q >= 0.0f) && (q < float(n[a]));
    } else if (bm == CLAMP) {
      i = min(max(i, -1), n[a] - 1);
    } else {
      i = wrap_index(i, n[a]);
    }
    i0[a] = i;
  }
  if (!inside) return false;
  s.idx = (int64_t(i0[2] + 1) * qd.y + (i0[1] + 1)) * qd.x + (i0[0] + 1);
  return true;
}

// The raymarch's sample through the quad layout, without the explicit rounding
// of read_linear_quad: the lerps contract to FMAs (the raymarch matches the
// oracle to a tolerance, not bit for bit).  Returns false outside (BORDER).
template <class T>
__device__ __forceinline__ bool quad_sample_fma(const typename QuadOf<T>::type* __restrict__ q, float px, float py,
                                                float pz, const Dims& d, const QuadDims& qd, int bm, QuadPos& s,
                                                float& v) {
  if (!quad_setup(px, py, pz, d, qd, bm, s)) {
    v = 0.0f;
    return false;
  }
  float a[4], b[4];
  quad_fetch<T>(q, s.idx, a);
  quad_fetch<T>(q, s.idx + qd.plane, b);
  const float a0 = fmaf(s.w[0], a[1] - a[0], a[0]), a1 = fmaf(s.w[0], a[3] - a[2], a[2]);
  const float b0 = fmaf(s.w[0], b[1] - b[0], b[0]), b1 = fmaf(s.w[0], b[3] - b[2], b[2]);
  const float v0 = fmaf(s.w[1], a1 - a0, a0), v1 = fmaf(s.w[1], b1 - b0, b0);
  v = fmaf(s.w[2], v1 - v0, v0);
  return true;
}

// scatter_linear_quad for a position already set up by quad_sample_fma.
__device__ __forceinline__ void scatter_quad_at(float4* __restrict__ gq, const QuadPos& s, const QuadDims& qd,
                                                float g) {
  const float wx1 = s.w[0], wx0 = 1.0f - s.w[0];
  const float wy1 = s.w[1], wy0 = 1.0f - s.w[1];
  const float g0 = g * (1.0f - s.w[2]), g1 = g * s.w[2];
  const float a00 = wx0 * wy0, a10 = wx1 * wy0, a01 = wx0 * wy1, a11 = wx1 * wy1;
  atomicAdd(gq + s.idx, make_float4(g0 * a00, g0 * a10, g0 * a01, g0 * a11));
  atomicAdd(gq + s.idx + qd.plane, make_float4(g1 * a00, g1 * a10, g1 * a01, g1 * a11));
}

template <class T>
__device__ __forceinline__ float read_linear_quad(const typename QuadOf<T>::type* __restrict__ q, float px, float py,
                                                  float pz, const Dims& d, const QuadDims& qd, int bm) {
  QuadPos s;
  if (!quad_setup(px, py, pz, d, qd, bm, s)) return 0.0f;
  float a[4], b[4];
  quad_fetch<T>(q, s.idx, a);
  quad_fetch<T>(q, s.idx + qd.plane, b);
  const float v0 = lerp_rn(lerp_rn(a[0], a[1], s.w[0]), lerp_rn(a[2], a[3], s.w[0]), s.w[1]);
  const float v1 = lerp_rn(lerp_rn(b[0], b[1], s.w[0]), lerp_rn(b[2], b[3], s.w[0]), s.w[1]);
  return lerp_rn(v0, v1, s.w[2]);
}

// Adjoint of read_linear_quad: g times the eight corner weights (tri_weight's
// products) added to the quad gradient grid with two vector atomics.
__device__ __forceinline__ void scatter_linear_quad(float4* __restrict__ gq, float px, float py, float pz,
                                                    const Dims& d, const QuadDims& qd, int bm, float g) {
  QuadPos s;
  if (!quad_setup(px, py, pz, d, qd, bm, s)) return;
  const float wx1 = s.w[0], wx0 = sub_rn(1.0f, s.w[0]);
  const float wy1 = s.w[1], wy0 = sub_rn(1.0f, s.w[1]);
  const float wz1 = s.w[2], wz0 = sub_rn(1.0f, s.w[2]);
  const float a00 = mul_rn(wx0, wy0), a10 = mul_rn(wx1, wy0), a01 = mul_rn(wx0, wy1), a11 = mul_rn(wx1, wy1);
  atomicAdd(gq + s.idx, make_float4(mul_rn(g, mul_rn(a00, wz0)), mul_rn(g, mul_rn(a10, wz0)),
                                    mul_rn(g, mul_rn(a01, wz0)), mul_rn(g, mul_rn(a11, wz0))));
  atomicAdd(gq + s.idx + qd.plane, make_float4(mul_rn(g, mul_rn(a00, wz1)), mul_rn(g, mul_rn(a10, wz1)),
                                               mul_rn(g, mul_rn(a01, wz1)), mul_rn(g, mul_rn(a11, wz1))));
}

// Coordinates of an axis of n cells whose boundary rule maps onto cell i: i
// itself, plus the padding coordinates -1 / n that CLAMP or WRAP send to i.
// Returns the count (at most 3, for n == 1).
__device__ __forceinline__ int quad_sources(int i, int n, int bm, int src[3]) {
  int k = 0;
  src[k++] = i;
  if (bm == CLAMP) {
    if (i == 0) src[k++] = -1;
    if (i == n - 1) src[k++] = n;
  } else if (bm == WRAP) {
    if (i == 0) src[k++] = n;
    if (i == n - 1) src[k++] = -1;
  }
  return k;
}

// Cell gradients from the quad gradient grid, written (not added) to grad; one
// thread per cell, launched as cell_launch over W, H and D * N planes
// (blockIdx.z = z + D * b).  Component (kx, ky) of entry (xq, yq) is coordinate
// (xq - 1 + kx, yq - 1 + ky) of plane zq - 1.
__device__ __forceinline__ void quad_fold_at(const float4* __restrict__ gq, const Dims& d, int bm,
                                             float* __restrict__ grad, int x, int y, int z, int b,
                                             bool accumulate = false) {
  const QuadDims qd = QuadDims::of(d);
  const int64_t i = (int64_t(z) * d.y + y) * d.x + x;
  const float4* q = gq + int64_t(b) * qd.count;
  int sx[3], sy[3], sz[3];
  const int nx = quad_sources(x, d.x, bm, sx), ny = quad_sources(y, d.y, bm, sy), nz = quad_sources(z, d.z, bm, sz);
  float acc = 0.0f;
  for (int kz = 0; kz < nz; ++kz) {
    const int64_t pz = int64_t(sz[kz] + 1) * qd.plane;
    for (int ky = 0; ky < ny; ++ky) {
      const int cy = sy[ky];
      for (int kx = 0; kx < nx; ++kx) {
        const int cx = sx[kx];
        // (cx, cy) is component (0,0) of entry (cx+1, cy+1), (1,0) of (cx, cy+1),
        // (0,1) of (cx+1, cy), (1,1) of (cx, cy); entries outside [0,W]x[0,H] do not exist
        if (cx + 1 <= d.x && cy + 1 <= d.y) acc += q[pz + int64_t(cy + 1) * qd.x + (cx + 1)].x;
        if (cx >= 0 && cy + 1 <= d.y) acc += q[pz + int64_t(cy + 1) * qd.x + cx].y;
        if (cx + 1 <= d.x && cy >= 0) acc += q[pz + int64_t(cy) * qd.x + (cx + 1)].z;
        if (cx >= 0 && cy >= 0) acc += q[pz + int64_t(cy) * qd.x + cx].w;
      }
    }
  }
  float* out = grad + int64_t(b) * d.count() + i;
  *out = accumulate ? *out + acc : acc;
}

static __global__ void k_quad_fold(const float4* __restrict__ gq, Dims d, int bm, float* __restrict__ grad,
                                   int accumulate) {
  const int x = int(blockIdx.x * blockDim.x + threadIdx.x), y = int(blockIdx.y * blockDim.y + threadIdx.y);
  if (x >= d.x || y >= d.y) return;
  const int b = int(blockIdx.z) / d.z, z = int(blockIdx.z) - b * d.z;
  quad_fold_at(gq, d, bm, grad, x, y, z, b, accumulate != 0);
}

}  // namespace ngt
