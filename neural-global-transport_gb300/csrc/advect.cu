// Fused semi-Lagrangian / MacCormack advection of a cell-centred grid by a
// MAC-staggered velocity, and its gradient.
//
// The reference composes this in TensorFlow (VelocityGrid.warp,
// data_structures.py:1690-1737): centred velocity (:1634-1654), lookup
// ``-u*dt`` (:1684-1688), SampleGridLut forward and back, correction
// ``fwd + 0.5*(data - back)``, MIN / MAX lookups and the MC_SMOOTH revert
// clamp -- four resample launches and about six elementwise passes over HBM.
// Here it is two kernels forward and three backward:
//
//   forward 1: u_c from the faces, trilinear lookup  -> fwd field
//   forward 2: back-trace of fwd, correction, extrema of the forward lookup's
//              corners, revert clamp                    -> output
//   backward 1: recompute state, route the gradient of the correction; scatter
//               into the fwd-field gradient; lookup gradient of the back-trace
//   backward 2: scatter the fwd-field gradient into the data gradient; lookup
//               gradient of the forward trace
//   backward 3: centred-velocity gradient back to the faces (a gather, no atomics)
//
// Arithmetic of positions, interpolation and correction is explicitly rounded
// in the composition's order, so float32 results equal an op-by-op evaluation
// of the reference's formula and the clamp mask is reproduced exactly.
#include "ngt_common.cuh"
#include "ngt_host.cuh"

namespace ngt {
namespace {

constexpr int kBlock = 256;

template <class T>
struct AdvParams {
  const T* data;
  const T* vx;
  const T* vy;
  const T* vz;
  T* out;
  typename Compute<T>::type* fwd;  // fwd field (compute type)
  const typename Compute<T>::type* gout;
  typename Compute<T>::type* gdata;
  typename Compute<T>::type* gvx;
  typename Compute<T>::type* gvy;
  typename Compute<T>::type* gvz;
  typename Compute<T>::type* gfwd;  // workspace: gradient w.r.t. the fwd field
  typename Compute<T>::type* guc;   // workspace: gradient w.r.t. the centred velocity (3 per cell)
  typename Compute<T>::type* buf;   // reference mode: unnormalised scatter
  unsigned* cnt;                    // reference mode: sample counts
  Dims d;
  float dt;
  int order, clamp, bm, reference;
};

__device__ __forceinline__ void cell_of(int64_t i, const Dims& d, int& x, int& y, int& z) {
  x = int(i % d.x);
  y = int((i / d.x) % d.y);
  z = int(i / (int64_t(d.x) * d.y));
}

// lookup = centred(u) * (-dt) (data_structures.py:1634-1654, 1684-1688)
template <class T, class S>
__device__ __forceinline__ void lookup(const AdvParams<T>& p, int x, int y, int z, S lut[3]) {
  const Dims& d = p.d;
  const S h = S(0.5);
  const S ux0 = S(ld(p.vx + (int64_t(z) * d.y + y) * (d.x + 1) + x));
  const S ux1 = S(ld(p.vx + (int64_t(z) * d.y + y) * (d.x + 1) + x + 1));
  const S uy0 = S(ld(p.vy + (int64_t(z) * (d.y + 1) + y) * d.x + x));
  const S uy1 = S(ld(p.vy + (int64_t(z) * (d.y + 1) + y + 1) * d.x + x));
  const S uz0 = S(ld(p.vz + (int64_t(z) * d.y + y) * d.x + x));
  const S uz1 = S(ld(p.vz + (int64_t(z + 1) * d.y + y) * d.x + x));
  const S ndt = S(-p.dt);
  lut[0] = mul_rn(mul_rn(add_rn(ux1, ux0), h), ndt);
  lut[1] = mul_rn(mul_rn(add_rn(uy1, uy0), h), ndt);
  lut[2] = mul_rn(mul_rn(add_rn(uz1, uz0), h), ndt);
}

template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_adv_fwd1(AdvParams<T> p) {
  typedef typename Compute<T>::type S;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= p.d.count()) return;
  int x, y, z;
  cell_of(i, p.d, x, y, z);
  S lut[3];
  lookup<T, S>(p, x, y, z, lut);
  S v[C];
  read_linear<C>(p.data, add_rn(lut[0], S(x)), add_rn(lut[1], S(y)), add_rn(lut[2], S(z)), p.d, p.bm, v);
  if (p.order == 1) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const S o = (p.clamp == NGT_CLAMP_NEGATIVE) ? fmax(v[c], S(0)) : v[c];
      p.out[i * C + c] = from_compute<T>(o);
    }
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) p.fwd[i * C + c] = v[c];
  }
}

// MacCormack state of one cell: fwd, back, correction, clamp mask and result
template <int C, class S>
struct McState {
  S fwd[C], back[C], corr[C], res[C];
  bool mask[C];
};

template <int C, class T, class S>
__device__ __forceinline__ void mc_state(const AdvParams<T>& p, int64_t i, int x, int y, int z, const S lut[3],
                                         McState<C, S>& s, S vb[8][C], Tri<S>& tb) {
  const S p2x = add_rn(-lut[0], S(x)), p2y = add_rn(-lut[1], S(y)), p2z = add_rn(-lut[2], S(z));
  tb = tri_setup(p2x, p2y, p2z, p.d, p.bm);
  if (p.bm == BORDER && !tb.inside) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
      for (int c = 0; c < C; ++c) vb[k][c] = S(0);
#pragma unroll
    for (int c = 0; c < C; ++c) s.back[c] = S(0);
  } else {
    tri_fetch<C>(p.fwd, tb, p.d, vb);
    tri_combine<C>(vb, tb, s.back);
  }
  S mn[C], mx[C];
  if (p.clamp == NGT_CLAMP_MC_SMOOTH) {
    const S p1x = add_rn(lut[0], S(x)), p1y = add_rn(lut[1], S(y)), p1z = add_rn(lut[2], S(z));
    int arg[C];
    int64_t ci[8];
    read_extremum<C>(p.data, p1x, p1y, p1z, p.d, p.bm, false, mn, arg, ci);
    read_extremum<C>(p.data, p1x, p1y, p1z, p.d, p.bm, true, mx, arg, ci);
  }
#pragma unroll
  for (int c = 0; c < C; ++c) {
    s.fwd[c] = p.fwd[i * C + c];
    const S rho = S(ld(p.data + i * C + c));
    s.corr[c] = add_rn(s.fwd[c], mul_rn(S(0.5), sub_rn(rho, s.back[c])));
    s.mask[c] = (p.clamp == NGT_CLAMP_MC_SMOOTH) && (s.corr[c] < mn[c] || s.corr[c] > mx[c]);
    s.res[c] = s.mask[c] ? s.fwd[c] : s.corr[c];
  }
}

template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_adv_fwd2(AdvParams<T> p) {
  typedef typename Compute<T>::type S;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= p.d.count()) return;
  int x, y, z;
  cell_of(i, p.d, x, y, z);
  S lut[3];
  lookup<T, S>(p, x, y, z, lut);
  McState<C, S> s;
  S vb[8][C];
  Tri<S> tb;
  mc_state<C>(p, i, x, y, z, lut, s, vb, tb);
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const S o = (p.clamp == NGT_CLAMP_NEGATIVE) ? fmax(s.res[c], S(0)) : s.res[c];
    p.out[i * C + c] = from_compute<T>(o);
  }
}

// backward 1: gradient of the correction; back-trace adjoint into gfwd
template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_adv_bwd1(AdvParams<T> p) {
  typedef typename Compute<T>::type S;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= p.d.count()) return;
  int x, y, z;
  cell_of(i, p.d, x, y, z);
  S lut[3];
  lookup<T, S>(p, x, y, z, lut);
  S g[C];
  S duc[3] = {S(0), S(0), S(0)};
  if (p.order == 1) {
    S v[C];
    if (p.clamp == NGT_CLAMP_NEGATIVE)
      read_linear<C>(p.data, add_rn(lut[0], S(x)), add_rn(lut[1], S(y)), add_rn(lut[2], S(z)), p.d, p.bm, v);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      g[c] = p.gout[i * C + c];
      if (p.clamp == NGT_CLAMP_NEGATIVE && !(v[c] >= S(0))) g[c] = S(0);
      p.gfwd[i * C + c] = g[c];
      p.gdata[i * C + c] = S(0);
    }
  } else {
    McState<C, S> s;
    S vb[8][C];
    Tri<S> tb;
    mc_state<C>(p, i, x, y, z, lut, s, vb, tb);
    S gback[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      g[c] = p.gout[i * C + c];
      if (p.clamp == NGT_CLAMP_NEGATIVE && !(s.res[c] >= S(0))) g[c] = S(0);
      const S gc = s.mask[c] ? S(0) : g[c];
      gback[c] = -(S(0.5) * gc);
      p.gdata[i * C + c] = S(0.5) * gc;  // direct term of the correction
    }
    if (p.reference) {
#pragma unroll
      for (int c = 0; c < C; ++c) p.gfwd[i * C + c] = g[c];
      scatter_linear_counted<C>(p.buf, p.cnt, add_rn(-lut[0], S(x)), add_rn(-lut[1], S(y)), add_rn(-lut[2], S(z)),
                                p.d, p.bm, gback);
    } else {
#pragma unroll
      for (int c = 0; c < C; ++c) atomic_add(p.gfwd + i * C + c, g[c]);
      scatter_linear<C>(p.gfwd, add_rn(-lut[0], S(x)), add_rn(-lut[1], S(y)), add_rn(-lut[2], S(z)), p.d, p.bm,
                        gback);
    }
    if (!(p.bm == BORDER && !tb.inside)) {
      S dx[C], dy[C], dz[C];
      tri_gradient<C>(vb, tb, dx, dy, dz);
      // d pos2 / d u_c = +dt
#pragma unroll
      for (int c = 0; c < C; ++c) {
        duc[0] += S(p.dt) * gback[c] * dx[c];
        duc[1] += S(p.dt) * gback[c] * dy[c];
        duc[2] += S(p.dt) * gback[c] * dz[c];
      }
    }
  }
  p.guc[i * 3 + 0] = duc[0];
  p.guc[i * 3 + 1] = duc[1];
  p.guc[i * 3 + 2] = duc[2];
}

// add normalised buffered scatter (reference mode) and clear the buffer
template <int C, class S>
__global__ void k_adv_norm(S* __restrict__ target, S* __restrict__ buf, unsigned* __restrict__ cnt, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned k = cnt[i];
  if (k > 0) {
    const S w = S(1) / S(k);
#pragma unroll
    for (int c = 0; c < C; ++c) target[i * C + c] += buf[i * C + c] * w;
  }
#pragma unroll
  for (int c = 0; c < C; ++c) buf[i * C + c] = S(0);
  cnt[i] = 0u;
}

// backward 2: forward-trace adjoint into the data gradient
template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_adv_bwd2(AdvParams<T> p) {
  typedef typename Compute<T>::type S;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= p.d.count()) return;
  int x, y, z;
  cell_of(i, p.d, x, y, z);
  S lut[3];
  lookup<T, S>(p, x, y, z, lut);
  const S p1x = add_rn(lut[0], S(x)), p1y = add_rn(lut[1], S(y)), p1z = add_rn(lut[2], S(z));
  S g[C];
#pragma unroll
  for (int c = 0; c < C; ++c) g[c] = p.gfwd[i * C + c];
  if (p.reference) scatter_linear_counted<C>(p.buf, p.cnt, p1x, p1y, p1z, p.d, p.bm, g);
  else scatter_linear<C>(p.gdata, p1x, p1y, p1z, p.d, p.bm, g);
  const Tri<S> t = tri_setup(p1x, p1y, p1z, p.d, p.bm);
  S duc[3] = {p.guc[i * 3 + 0], p.guc[i * 3 + 1], p.guc[i * 3 + 2]};
  if (!(p.bm == BORDER && !t.inside)) {
    S v[8][C], dx[C], dy[C], dz[C];
    tri_fetch<C>(p.data, t, p.d, v);
    tri_gradient<C>(v, t, dx, dy, dz);
    // d pos1 / d u_c = -dt
#pragma unroll
    for (int c = 0; c < C; ++c) {
      duc[0] -= S(p.dt) * g[c] * dx[c];
      duc[1] -= S(p.dt) * g[c] * dy[c];
      duc[2] -= S(p.dt) * g[c] * dz[c];
    }
  }
  p.guc[i * 3 + 0] = duc[0];
  p.guc[i * 3 + 1] = duc[1];
  p.guc[i * 3 + 2] = duc[2];
}

// backward 3: faces receive half of each adjacent cell's centred-velocity gradient
template <class S>
__global__ void __launch_bounds__(kBlock) k_adv_faces(const S* __restrict__ guc, S* __restrict__ gx, S* __restrict__ gy,
                                                      S* __restrict__ gz, Dims d) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nx = int64_t(d.x + 1) * d.y * d.z;
  const int64_t ny = int64_t(d.x) * (d.y + 1) * d.z;
  const int64_t nz = int64_t(d.x) * d.y * (d.z + 1);
  const S h = S(0.5);
  if (i < nx) {
    const int x = int(i % (d.x + 1)), y = int((i / (d.x + 1)) % d.y), z = int(i / (int64_t(d.x + 1) * d.y));
    S s = S(0);
    if (x > 0) s += guc[flat(x - 1, y, z, d) * 3 + 0] * h;
    if (x < d.x) s += guc[flat(x, y, z, d) * 3 + 0] * h;
    gx[i] = s;
  } else if (i < nx + ny) {
    const int64_t j = i - nx;
    const int x = int(j % d.x), y = int((j / d.x) % (d.y + 1)), z = int(j / (int64_t(d.x) * (d.y + 1)));
    S s = S(0);
    if (y > 0) s += guc[flat(x, y - 1, z, d) * 3 + 1] * h;
    if (y < d.y) s += guc[flat(x, y, z, d) * 3 + 1] * h;
    gy[j] = s;
  } else if (i < nx + ny + nz) {
    const int64_t j = i - nx - ny;
    const int x = int(j % d.x), y = int((j / d.x) % d.y), z = int(j / (int64_t(d.x) * d.y));
    S s = S(0);
    if (z > 0) s += guc[flat(x, y, z - 1, d) * 3 + 2] * h;
    if (z < d.z) s += guc[flat(x, y, z, d) * 3 + 2] * h;
    gz[j] = s;
  }
}

int validate(const ngt_advect_args* a) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: null arguments");
  if (!positive_shape(a->grid_dhw, 3)) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: shapes must be positive");
  if (!valid_channels(a->channels)) return fail(NGT_ERR_INVALID_ARGUMENT, "Only 1,2 and 4 Channel supported.");
  if (a->grid_dhw[0] * a->grid_dhw[1] * a->grid_dhw[2] >= (int64_t(1) << 31))
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect: grid too large");
  if (a->order != 1 && a->order != 2) return fail(NGT_ERR_INVALID_ARGUMENT, "Unsupported warp order '%d'", a->order);
  if (a->clamp < NGT_CLAMP_NONE || a->clamp > NGT_CLAMP_NEGATIVE) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: invalid clamp");
  if (a->clamp == NGT_CLAMP_MC_SMOOTH && a->order != 2)
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect: MC_SMOOTH needs order 2");
  if (a->boundary < NGT_BORDER || a->boundary > NGT_WRAP) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: invalid boundary");
  if (a->dtype < NGT_F32 || a->dtype > NGT_F16) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: invalid dtype");
  if (!a->data || !a->vel_x || !a->vel_y || !a->vel_z) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: null pointer");
  if (a->order == 2 && !a->fwd_field) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: MacCormack needs fwd_field");
  return NGT_OK;
}

size_t compute_size(int dtype) { return dtype == NGT_F64 ? 8 : 4; }

template <class T>
AdvParams<T> params(const ngt_advect_args* a) {
  typedef typename Compute<T>::type S;
  AdvParams<T> p = {};
  p.data = static_cast<const T*>(a->data);
  p.vx = static_cast<const T*>(a->vel_x);
  p.vy = static_cast<const T*>(a->vel_y);
  p.vz = static_cast<const T*>(a->vel_z);
  p.out = static_cast<T*>(a->output);
  p.fwd = static_cast<S*>(a->fwd_field);
  p.d = Dims{int(a->grid_dhw[2]), int(a->grid_dhw[1]), int(a->grid_dhw[0])};
  p.dt = a->dt;
  p.order = a->order;
  p.clamp = a->clamp;
  p.bm = a->boundary;
  return p;
}

template <int C, class T>
int fwd_typed(const ngt_advect_args* a, cudaStream_t st) {
  AdvParams<T> p = params<T>(a);
  const unsigned nb = ceil_div_u(p.d.count(), kBlock);
  k_adv_fwd1<C, T><<<nb, kBlock, 0, st>>>(p);
  if (p.order == 2) k_adv_fwd2<C, T><<<nb, kBlock, 0, st>>>(p);
  return check_launch("ngt_advect_maccormack_fwd");
}

template <int C, class T>
int bwd_typed(const ngt_advect_grad_args* g, cudaStream_t st) {
  typedef typename Compute<T>::type S;
  AdvParams<T> p = params<T>(&g->fwd);
  const int64_t n = p.d.count();
  p.gout = static_cast<const S*>(g->output_grad);
  p.gdata = static_cast<S*>(g->data_grad);
  p.gvx = static_cast<S*>(g->vel_x_grad);
  p.gvy = static_cast<S*>(g->vel_y_grad);
  p.gvz = static_cast<S*>(g->vel_z_grad);
  p.reference = g->grad_mode == NGT_GRAD_REFERENCE;
  char* w = static_cast<char*>(g->workspace);
  p.gfwd = reinterpret_cast<S*>(w);
  w += size_t(n) * C * sizeof(S);
  p.guc = reinterpret_cast<S*>(w);
  w += size_t(n) * 3 * sizeof(S);
  if (p.reference) {
    p.buf = reinterpret_cast<S*>(w);
    w += size_t(n) * C * sizeof(S);
    p.cnt = reinterpret_cast<unsigned*>(w);
    if (cudaMemsetAsync(p.buf, 0, size_t(n) * (C * sizeof(S) + sizeof(unsigned)), st) != cudaSuccess)
      return check_launch("advect_bwd memset");
  }
  if (!p.reference && cudaMemsetAsync(p.gfwd, 0, size_t(n) * C * sizeof(S), st) != cudaSuccess)
    return check_launch("advect_bwd memset");
  const unsigned nb = ceil_div_u(n, kBlock);
  k_adv_bwd1<C, T><<<nb, kBlock, 0, st>>>(p);
  if (p.reference && p.order == 2) k_adv_norm<C, S><<<nb, kBlock, 0, st>>>(p.gfwd, p.buf, p.cnt, n);
  k_adv_bwd2<C, T><<<nb, kBlock, 0, st>>>(p);
  if (p.reference) k_adv_norm<C, S><<<nb, kBlock, 0, st>>>(p.gdata, p.buf, p.cnt, n);
  if (p.gvx && p.gvy && p.gvz) {
    const int64_t nf = int64_t(p.d.x + 1) * p.d.y * p.d.z + int64_t(p.d.x) * (p.d.y + 1) * p.d.z +
                       int64_t(p.d.x) * p.d.y * (p.d.z + 1);
    k_adv_faces<S><<<ceil_div_u(nf, kBlock), kBlock, 0, st>>>(p.guc, p.gvx, p.gvy, p.gvz, p.d);
  }
  return check_launch("ngt_advect_maccormack_bwd");
}

template <class T>
int fwd_c(const ngt_advect_args* a, cudaStream_t st) {
  switch (a->channels) {
    case 1: return fwd_typed<1, T>(a, st);
    case 2: return fwd_typed<2, T>(a, st);
    default: return fwd_typed<4, T>(a, st);
  }
}

template <class T>
int bwd_c(const ngt_advect_grad_args* g, cudaStream_t st) {
  switch (g->fwd.channels) {
    case 1: return bwd_typed<1, T>(g, st);
    case 2: return bwd_typed<2, T>(g, st);
    default: return bwd_typed<4, T>(g, st);
  }
}

}  // namespace
}  // namespace ngt

using namespace ngt;

extern "C" int ngt_advect_maccormack_fwd(const ngt_advect_args* a, void* stream) {
  int rc = validate(a);
  if (rc) return rc;
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: null output");
  cudaStream_t st = as_stream(stream);
  switch (a->dtype) {
    case NGT_F32: return fwd_c<float>(a, st);
    case NGT_F64: return fwd_c<double>(a, st);
    case NGT_BF16: return fwd_c<__nv_bfloat16>(a, st);
    default: return fwd_c<__half>(a, st);
  }
}

extern "C" size_t ngt_advect_maccormack_bwd_workspace_bytes(const ngt_advect_grad_args* g) {
  if (!g) return 0;
  const int64_t n = g->fwd.grid_dhw[0] * g->fwd.grid_dhw[1] * g->fwd.grid_dhw[2];
  const int64_t C = g->fwd.channels;
  const size_t cs = compute_size(g->fwd.dtype);
  size_t bytes = size_t(n) * size_t(C + 3) * cs;
  if (g->grad_mode == NGT_GRAD_REFERENCE) bytes += size_t(n) * (size_t(C) * cs + sizeof(unsigned));
  return bytes;
}

extern "C" int ngt_advect_maccormack_bwd(const ngt_advect_grad_args* g, void* stream) {
  if (!g) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_bwd: null arguments");
  int rc = validate(&g->fwd);
  if (rc) return rc;
  if (!g->output_grad || !g->data_grad) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_bwd: null pointer");
  if (g->grad_mode != NGT_GRAD_EXACT && g->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect_bwd: invalid grad_mode");
  const size_t need = ngt_advect_maccormack_bwd_workspace_bytes(g);
  if (!g->workspace || g->workspace_bytes < need)
    return fail(NGT_ERR_WORKSPACE, "advect_bwd needs %zu workspace bytes", need);
  cudaStream_t st = as_stream(stream);
  switch (g->fwd.dtype) {
    case NGT_F32: return bwd_c<float>(g, st);
    case NGT_F64: return bwd_c<double>(g, st);
    case NGT_BF16: return bwd_c<__nv_bfloat16>(g, st);
    default: return bwd_c<__half>(g, st);
  }
}
