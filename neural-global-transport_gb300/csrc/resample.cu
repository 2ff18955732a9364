// Grid resampling: lookup-table (LUT) resample and camera / grid transform
// resample, their gradients, the mip pyramid and the LoD lookup table.
//
// Semantics follow the reference kernels kSampleGrid3DLuT
// (resample_grid.cu.cc:604-623), kScatterLuT3DGradients (:1420-1450),
// kSample3D (:255-267), kScatter3DGradients (:1160-1190), kGenerateMip3D
// (:58-84) and kComputeLoD3D (:1702-1717).  One thread per output voxel;
// blockIdx.y enumerates (batch, camera) output slots, so all cameras of a batch
// run in one launch with no per-camera host round trip.
#include "ngt_common.cuh"
#include "ngt_gather.cuh"
#include "ngt_host.cuh"

namespace ngt {
namespace {

constexpr int kMaxMip = 15;
constexpr int kBlock = 256;

template <class T>
struct Mips {
  const T* base[kMaxMip + 1];   // level pointers for batch 0
  int64_t bstride[kMaxMip + 1];  // elements between batch entries per level
  Dims dims[kMaxMip + 1];
  int levels;                    // number of coarser levels (0: no mipmapping)
};

template <class S>
__device__ __forceinline__ S fract_(S v) { return v - floor(v); }

// sample3D with mipmapping (sampling.hpp:991-1010): level l reads dims>>l at
// position/2^l minus the cell-centre offset.
template <int C, class T>
__device__ __forceinline__ void sample_mip(const Mips<T>& m, int b, T px, T py, T pz, T lodw, T cco, int fm, int bm,
                                           int mipmode, float bias, T out[C]) {
  if (mipmode == NGT_MIP_NONE || m.levels == 0) {
    read_filtered<C>(m.base[0] + b * m.bstride[0], sub_rn(px, cco), sub_rn(py, cco), sub_rn(pz, cco), m.dims[0], fm,
                     bm, out);
    return;
  }
  T lod = lodw + T(bias);
  lod = fmin(fmax(lod, T(0)), T(m.levels));
  auto level_read = [&](int l, T o[C]) {
    const T sc = T(1 << l);
    read_filtered<C>(m.base[l] + b * m.bstride[l], px / sc - cco, py / sc - cco, pz / sc - cco, m.dims[l], fm, bm, o);
  };
  if (mipmode == NGT_MIP_NEAREST) {
    const int l = min(to_int_rz(lod + T(0.5)), m.levels);
    level_read(l, out);
    return;
  }
  const int lf = min(to_int_rz(lod), m.levels);
  const int lc = min(to_int_rz(ceil(lod)), m.levels);
  level_read(lf, out);
  if (lc > lf) {
    T hi[C];
    level_read(lc, hi);
    const T t = fract_(lod);
#pragma unroll
    for (int c = 0; c < C; ++c) out[c] = out[c] + t * (hi[c] - out[c]);
  }
}

// ------------------------------------------------------------------ LUT
template <class T>
struct LutParams {
  const T* lut;
  T* out;
  const T* out_grad;
  T* in_grad;
  T* lut_grad;
  unsigned* count;
  Mips<T> mips;
  Dims din, dout;
  int N, V, sep;
  int fm, bm, mipmode;
  float bias;
  T cco;
  int relative, normalized;
  int slot0;
};

template <class T>
__device__ __forceinline__ void lut_position(const LutParams<T>& p, int cam, int64_t i, T& x, T& y, T& z, T& w) {
  const int64_t osz = p.dout.count();
  const T* l = p.lut + (int64_t(cam) * osz + i) * 4;
  x = l[0];
  y = l[1];
  z = l[2];
  w = l[3];
  if (p.normalized) {
    x = mul_rn(x, T(p.dout.x));
    y = mul_rn(y, T(p.dout.y));
    z = mul_rn(z, T(p.dout.z));
  }
  if (p.relative) {
    const int ix = int(i % p.dout.x);
    const int iy = int((i / p.dout.x) % p.dout.y);
    const int iz = int(i / (int64_t(p.dout.x) * p.dout.y));
    x = add_rn(x, T(ix));
    y = add_rn(y, T(iy));
    z = add_rn(z, T(iz));
  }
}

template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_lut_fwd(LutParams<T> p) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t osz = p.dout.count();
  if (i >= osz) return;
  const int slot = p.slot0 + blockIdx.y;
  const int b = p.sep ? slot / p.V : slot;
  const int cam = p.sep ? slot % p.V : slot;
  T x, y, z, w;
  lut_position(p, cam, i, x, y, z, w);
  T v[C];
  sample_mip<C>(p.mips, b, x, y, z, w, p.cco, p.fm, p.bm, p.mipmode, p.bias, v);
  T* o = p.out + (int64_t(slot) * osz + i) * C;
#pragma unroll
  for (int c = 0; c < C; ++c) o[c] = v[c];
}

// One thread per (camera, output voxel); the batches reading that camera's
// lookup are looped inside, so the lookup gradient is written once.
template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_lut_bwd(LutParams<T> p, int reference, int skip_scatter) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t osz = p.dout.count();
  if (i >= osz) return;
  const int cam = blockIdx.y;
  T x, y, z, w;
  lut_position(p, cam, i, x, y, z, w);
  const T px = sub_rn(x, p.cco), py = sub_rn(y, p.cco), pz = sub_rn(z, p.cco);
  const int b0 = p.sep ? 0 : cam, b1 = p.sep ? p.N : cam + 1;
  T lg[3] = {T(0), T(0), T(0)};
  const int64_t vsz = p.din.count();
  for (int b = b0; b < b1; ++b) {
    const int slot = p.sep ? b * p.V + cam : b;
    T g[C];
#pragma unroll
    for (int c = 0; c < C; ++c) g[c] = p.out_grad[(int64_t(slot) * osz + i) * C + c];
    const T* in = p.mips.base[0] + b * p.mips.bstride[0];
    T* ig = p.in_grad + int64_t(b) * vsz * C;
    if (p.fm == LINEAR && p.lut_grad) {
      const Tri<T> t = tri_setup(px, py, pz, p.din, p.bm);
      T cur[3] = {T(0), T(0), T(0)};
      if (!(p.bm == BORDER && !t.inside)) {
        T v[8][C], dx[C], dy[C], dz[C];
        tri_fetch<C>(in, t, p.din, v);
        tri_gradient<C>(v, t, dx, dy, dz);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          cur[0] = add_rn(cur[0], mul_rn(g[c], dx[c]));
          cur[1] = add_rn(cur[1], mul_rn(g[c], dy[c]));
          cur[2] = add_rn(cur[2], mul_rn(g[c], dz[c]));
        }
      }
      if (reference) {  // each batch overwrites (resample_grid.cu.cc:1437-1443)
        lg[0] = cur[0];
        lg[1] = cur[1];
        lg[2] = cur[2];
      } else {
        lg[0] += cur[0];
        lg[1] += cur[1];
        lg[2] += cur[2];
      }
    }
    if (skip_scatter) {
    } else if (reference) {
      scatter_linear_counted<C>(ig, p.count + int64_t(b) * vsz, px, py, pz, p.din, p.bm, g);
    } else if (p.fm == LINEAR) {
      scatter_linear<C>(ig, px, py, pz, p.din, p.bm, g);
    } else if (p.fm == NEAREST) {
      scatter_nearest<C>(ig, px, py, pz, p.din, p.bm, g);
    } else {
      scatter_extremum<C>(ig, in, px, py, pz, p.din, p.bm, p.fm == FMAX, g);
    }
  }
  if (p.lut_grad) {
    T* o = p.lut_grad + (int64_t(cam) * osz + i) * 4;
    if (!reference && p.normalized) {
      lg[0] *= T(p.dout.x);
      lg[1] *= T(p.dout.y);
      lg[2] *= T(p.dout.z);
    }
    o[0] = lg[0];
    o[1] = lg[1];
    o[2] = lg[2];
    o[3] = T(0);
  }
}

// Samples of batch b for the deterministic input gradient: every (camera, output
// voxel) pair that reads batch b, at its lookup position.
template <int C, class T>
struct LutSource {
  LutParams<T> p;
  int b;
  __device__ __forceinline__ bool operator()(int64_t s, T pos[3], T g[C]) const {
    const int64_t osz = p.dout.count();
    const int cam = p.sep ? int(s / osz) : b;
    const int64_t i = p.sep ? s % osz : s;
    const int slot = p.sep ? b * p.V + cam : b;
    T x, y, z, w;
    lut_position(p, cam, i, x, y, z, w);
    pos[0] = sub_rn(x, p.cco);
    pos[1] = sub_rn(y, p.cco);
    pos[2] = sub_rn(z, p.cco);
#pragma unroll
    for (int c = 0; c < C; ++c) g[c] = p.out_grad[(int64_t(slot) * osz + i) * C + c];
    return true;
  }
};

// kNormalize3DGradients (resample_grid.cu.cc:1133-1151): divide by the per-voxel
// sample count where it is non-zero.
template <int C, class T>
__global__ void k_normalize_count(T* __restrict__ grad, const unsigned* __restrict__ count, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned k = count[i];
  if (k > 0) {
    const T w = T(1) / T(k);
#pragma unroll
    for (int c = 0; c < C; ++c) grad[i * C + c] = grad[i * C + c] * w;
  }
}

// ------------------------------------------------------------- transform
template <class T>
struct XfParams {
  T* out;
  const T* out_grad;
  T* in_grad;
  unsigned* count;
  Mips<T> mips;
  const float *M, *V, *P, *F;
  Dims din, dout;
  int N, ncam, sep;
  int fm, bm, mipmode, cm;
  float bias;
  T cco;
  int slot0;
};

__device__ __forceinline__ bool reverse_mode(int cm) {
  return cm == NGT_TRANSFORM_LINDEPTH_REVERSE || cm == NGT_TRANSFORM_REVERSE;
}
__device__ __forceinline__ bool lindepth_mode(int cm) {
  return cm == NGT_TRANSFORM_LINDEPTH || cm == NGT_TRANSFORM_LINDEPTH_REVERSE;
}

// samplePos3D<CM,false> (sampling.hpp:154-228)
__device__ __forceinline__ void xf_position(const Cam& cam, int cm, float ix, float iy, float iz, const Dims& dout,
                                            const Dims& din, float pos[3]) {
  if (reverse_mode(cm)) {
    const float dims[3] = {float(din.x), float(din.y), float(din.z)};
    os_to_idx(cam, ix, iy, iz, dims, lindepth_mode(cm), pos);
  } else {
    const float dinv[3] = {1.0f / float(dout.x), 1.0f / float(dout.y), 1.0f / float(dout.z)};
    idx_to_os(cam, ix, iy, iz, dinv, lindepth_mode(cm), pos);
  }
}

// level of detail of samplePos3D<CM,true>: forward differences over one output cell
__device__ __forceinline__ float xf_lod(const Cam& cam, int cm, float ix, float iy, float iz, const Dims& dout,
                                        const Dims& din, const float p0[3]) {
  float d[3][3];
  for (int a = 0; a < 3; ++a) {
    float q[3];
    xf_position(cam, cm, ix + (a == 0), iy + (a == 1), iz + (a == 2), dout, din, q);
    for (int k = 0; k < 3; ++k) d[a][k] = p0[k] - q[k];
  }
  float px, py, pz;
  if (reverse_mode(cm)) {
    px = sqrtf(d[0][0] * d[0][0] + d[0][1] * d[0][1] + d[0][2] * d[0][2]);
    py = sqrtf(d[1][0] * d[1][0] + d[1][1] * d[1][1] + d[1][2] * d[1][2]);
    pz = sqrtf(d[2][0] * d[2][0] + d[2][1] * d[2][1] + d[2][2] * d[2][2]);
  } else {
    px = sqrtf(d[0][0] * d[0][0] + d[1][0] * d[1][0] + d[2][0] * d[2][0]);
    py = sqrtf(d[0][1] * d[0][1] + d[1][1] * d[1][1] + d[2][1] * d[2][1]);
    pz = sqrtf(d[0][2] * d[0][2] + d[1][2] * d[1][2] + d[2][2] * d[2][2]);
  }
  return fmaxf(0.0f, log2f(fmaxf(px, fmaxf(py, pz))));
}

template <class T>
__device__ __forceinline__ void xf_slot(const XfParams<T>& p, int slot, int& b, int& cam) {
  b = p.sep ? slot / p.ncam : slot;
  cam = p.sep ? slot % p.ncam : slot;
}

template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_xf_fwd(XfParams<T> p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  const int slot = p.slot0 + blockIdx.y;
  int b, c;
  xf_slot(p, slot, b, c);
  if (threadIdx.x < 32) build_cam_warp(p.M + 16 * b, p.V + 16 * c, p.P + 16 * c, p.F + 6 * c, cam, cam_sh);
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t osz = p.dout.count();
  if (i >= osz) return;
  const int x = int(i % p.dout.x), y = int((i / p.dout.x) % p.dout.y), z = int(i / (int64_t(p.dout.x) * p.dout.y));
  float pos[3];
  xf_position(cam, p.cm, x + 0.5f, y + 0.5f, z + 0.5f, p.dout, p.din, pos);
  const float lod = (p.mipmode != NGT_MIP_NONE) ? xf_lod(cam, p.cm, x + 0.5f, y + 0.5f, z + 0.5f, p.dout, p.din, pos)
                                                 : 0.0f;
  T v[C];
  sample_mip<C>(p.mips, b, T(pos[0]), T(pos[1]), T(pos[2]), T(lod), p.cco, p.fm, p.bm, p.mipmode, p.bias, v);
  T* o = p.out + (int64_t(slot) * osz + i) * C;
#pragma unroll
  for (int k = 0; k < C; ++k) o[k] = v[k];
}

template <int C, class T>
__global__ void __launch_bounds__(kBlock) k_xf_bwd(XfParams<T> p, int reference) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  const int slot = p.slot0 + blockIdx.y;
  int b, c;
  xf_slot(p, slot, b, c);
  if (threadIdx.x < 32) build_cam_warp(p.M + 16 * b, p.V + 16 * c, p.P + 16 * c, p.F + 6 * c, cam, cam_sh);
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t osz = p.dout.count();
  if (i >= osz) return;
  const int x = int(i % p.dout.x), y = int((i / p.dout.x) % p.dout.y), z = int(i / (int64_t(p.dout.x) * p.dout.y));
  float pos[3];
  xf_position(cam, p.cm, x + 0.5f, y + 0.5f, z + 0.5f, p.dout, p.din, pos);
  const T px = T(pos[0]) - p.cco, py = T(pos[1]) - p.cco, pz = T(pos[2]) - p.cco;
  T g[C];
#pragma unroll
  for (int k = 0; k < C; ++k) g[k] = p.out_grad[(int64_t(slot) * osz + i) * C + k];
  const int64_t vsz = p.din.count();
  T* ig = p.in_grad + int64_t(b) * vsz * C;
  if (reference) {
    unsigned* cnt = p.count + int64_t(b) * vsz;
    if (p.fm == QUADRATIC) scatter_quadratic_counted<C>(ig, cnt, px, py, pz, p.din, p.bm, g);
    else scatter_linear_counted<C>(ig, cnt, px, py, pz, p.din, p.bm, g);
  } else if (p.fm == LINEAR) {
    scatter_linear<C>(ig, px, py, pz, p.din, p.bm, g);
  } else if (p.fm == NEAREST) {
    scatter_nearest<C>(ig, px, py, pz, p.din, p.bm, g);
  } else {
    scatter_quadratic<C>(ig, px, py, pz, p.din, p.bm, g);
  }
}

// Every slot's camera transform, one warp per slot, for the deterministic
// adjoint's sample source.
template <class T>
__global__ void k_xf_cams(XfParams<T> p, Cam* __restrict__ cams) {
  __shared__ Cam cam;
  __shared__ CamScratch sh;
  int b, c;
  xf_slot(p, int(blockIdx.x), b, c);
  build_cam_warp(p.M + 16 * b, p.V + 16 * c, p.P + 16 * c, p.F + 6 * c, cam, sh);
  __syncwarp();
  const float* src = reinterpret_cast<const float*>(&cam);
  float* dst = reinterpret_cast<float*>(cams + blockIdx.x);
  for (int i = threadIdx.x; i < int(sizeof(Cam) / sizeof(float)); i += 32) dst[i] = src[i];
}

// Samples of batch b for the deterministic input gradient: every (camera, output
// voxel) of a slot that reads batch b, at the position k_xf_bwd scatters from.
template <int C, class T>
struct XfSource {
  XfParams<T> p;
  const Cam* cams;
  int b;
  __device__ __forceinline__ bool operator()(int64_t s, T pos[3], T g[C]) const {
    const int64_t osz = p.dout.count();
    const int slot = p.sep ? b * p.ncam + int(s / osz) : b;
    const int64_t i = p.sep ? s % osz : s;
    const int x = int(i % p.dout.x), y = int((i / p.dout.x) % p.dout.y), z = int(i / (int64_t(p.dout.x) * p.dout.y));
    float q[3];
    xf_position(cams[slot], p.cm, x + 0.5f, y + 0.5f, z + 0.5f, p.dout, p.din, q);
    pos[0] = T(q[0]) - p.cco;
    pos[1] = T(q[1]) - p.cco;
    pos[2] = T(q[2]) - p.cco;
#pragma unroll
    for (int k = 0; k < C; ++k) g[k] = p.out_grad[(int64_t(slot) * osz + i) * C + k];
    return true;
  }
};

// ------------------------------------------------------------------- mips
// One 2x2x2 level (kGenerateMip3D): pairs averaged along z, then y, then x.
template <int C, class T>
__global__ void k_mip_down(const T* __restrict__ in, T* __restrict__ out, Dims din, Dims dout, int64_t in_bs,
                           int64_t out_bs) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= dout.count()) return;
  const int b = blockIdx.y;
  const int x = int(i % dout.x), y = int((i / dout.x) % dout.y), z = int(i / (int64_t(dout.x) * dout.y));
  const T* src = in + b * in_bs;
  const T h = T(0.5);
#pragma unroll
  for (int c = 0; c < C; ++c) {
    T sy[2];
    for (int ox = 0; ox < 2; ++ox) {
      T sz[2];
      for (int oy = 0; oy < 2; ++oy) {
        const T a0 = src[flat(2 * x + ox, 2 * y + oy, 2 * z, din) * C + c];
        const T a1 = src[flat(2 * x + ox, 2 * y + oy, 2 * z + 1, din) * C + c];
        sz[oy] = mul_rn(add_rn(a0, a1), h);
      }
      sy[ox] = mul_rn(add_rn(sz[0], sz[1]), h);
    }
    out[b * out_bs + i * C + c] = mul_rn(add_rn(sy[0], sy[1]), h);
  }
}

// --------------------------------------------------------------------- LoD
__global__ void k_lod(const float* MV, const float* P, const float* F, Dims din, Dims dout, int cm, int relative,
                      float* out) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  const int v = blockIdx.y;
  if (threadIdx.x < 32) build_cam_warp(nullptr, MV + 16 * v, P + 16 * v, F + 6 * v, cam, cam_sh);
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t osz = dout.count();
  if (i >= osz) return;
  const int x = int(i % dout.x), y = int((i / dout.x) % dout.y), z = int(i / (int64_t(dout.x) * dout.y));
  const float ix = x + 0.5f, iy = y + 0.5f, iz = z + 0.5f;
  float pos[3];
  xf_position(cam, cm, ix, iy, iz, dout, din, pos);
  // calcLoD<CM> (sampling.hpp:74-148): central differences, footprint per axis
  float d[3][3];
  for (int a = 0; a < 3; ++a) {
    float qm[3], qp[3];
    xf_position(cam, cm, ix - (a == 0), iy - (a == 1), iz - (a == 2), dout, din, qm);
    xf_position(cam, cm, ix + (a == 0), iy + (a == 1), iz + (a == 2), dout, din, qp);
    for (int k = 0; k < 3; ++k) d[a][k] = (qm[k] - qp[k]) * 0.5f;
  }
  const float px = sqrtf(d[0][0] * d[0][0] + d[1][0] * d[1][0] + d[2][0] * d[2][0]);
  const float py = sqrtf(d[0][1] * d[0][1] + d[1][1] * d[1][1] + d[2][1] * d[2][1]);
  const float pz = sqrtf(d[0][2] * d[0][2] + d[1][2] * d[1][2] + d[2][2] * d[2][2]);
  const float lod = fmaxf(0.0f, log2f(fmaxf(px, fmaxf(py, pz))));
  float* o = out + (int64_t(v) * osz + i) * 4;
  o[0] = pos[0] - (relative ? float(x) : 0.0f);
  o[1] = pos[1] - (relative ? float(y) : 0.0f);
  o[2] = pos[2] - (relative ? float(z) : 0.0f);
  o[3] = lod;
}

// ------------------------------------------------------------ host helpers
size_t elem_size(int dtype) { return dtype == NGT_F64 ? 8 : 4; }

Dims dims_of(const int64_t* s5) { return Dims{int(s5[3]), int(s5[2]), int(s5[1])}; }

size_t level_bytes(const int64_t s[5], int l, size_t es) {
  const int64_t d = s[1] >> l, h = s[2] >> l, w = s[3] >> l;
  const size_t raw = size_t(s[0] * d * h * w * s[4]) * es;
  return (raw + 255) & ~size_t(255);
}

size_t mip_bytes(int dtype, const int64_t s[5], int levels) {
  size_t total = 0;
  for (int l = 1; l <= levels; ++l) total += level_bytes(s, l, elem_size(dtype));
  return total;
}

template <class T>
int build_mips(const int64_t s[5], const T* input, int levels, void* pyramid, size_t bytes, cudaStream_t st,
               Mips<T>& m) {
  const int C = int(s[4]);
  m.levels = levels;
  m.base[0] = input;
  m.dims[0] = dims_of(s);
  m.bstride[0] = m.dims[0].count() * C;
  char* ptr = static_cast<char*>(pyramid);
  if (levels > 0 && (!pyramid || bytes < mip_bytes(sizeof(T) == 8 ? NGT_F64 : NGT_F32, s, levels)))
    return fail(NGT_ERR_WORKSPACE, "mip pyramid needs %zu bytes", mip_bytes(sizeof(T) == 8 ? NGT_F64 : NGT_F32, s, levels));
  for (int l = 1; l <= levels; ++l) {
    m.dims[l] = Dims{int(s[3] >> l), int(s[2] >> l), int(s[1] >> l)};
    m.bstride[l] = m.dims[l].count() * C;
    m.base[l] = reinterpret_cast<const T*>(ptr);
    if (m.dims[l].count() > 0) {
      const dim3 grid(ceil_div_u(m.dims[l].count(), kBlock), unsigned(s[0]));
      T* out = reinterpret_cast<T*>(ptr);
      const T* in = m.base[l - 1];
      if (C == 1) k_mip_down<1, T><<<grid, kBlock, 0, st>>>(in, out, m.dims[l - 1], m.dims[l], m.bstride[l - 1], m.bstride[l]);
      else if (C == 2) k_mip_down<2, T><<<grid, kBlock, 0, st>>>(in, out, m.dims[l - 1], m.dims[l], m.bstride[l - 1], m.bstride[l]);
      else k_mip_down<4, T><<<grid, kBlock, 0, st>>>(in, out, m.dims[l - 1], m.dims[l], m.bstride[l - 1], m.bstride[l]);
    }
    ptr += level_bytes(s, l, sizeof(T));
  }
  return check_launch("mip build");
}

// every mip level must keep at least one cell per axis
bool mip_levels_ok(const int64_t s[5], int levels) {
  return levels >= 0 && levels <= kMaxMip && (s[1] >> levels) >= 1 && (s[2] >> levels) >= 1 && (s[3] >> levels) >= 1;
}

int validate_grid(const int64_t s[5], const char* op) {
  if (!positive_shape(s, 5)) return fail(NGT_ERR_INVALID_ARGUMENT, "%s: shapes must be positive", op);
  if (!valid_channels(s[4])) return fail(NGT_ERR_INVALID_ARGUMENT, "Only 1,2 and 4 Channel supported.");
  if (s[1] * s[2] * s[3] >= (int64_t(1) << 31)) return fail(NGT_ERR_INVALID_ARGUMENT, "%s: grid too large", op);
  return NGT_OK;
}

int validate_lut(const ngt_sample_lut_args* a) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut: null arguments");
  int rc = validate_grid(a->input_shape, "sample_lut");
  if (rc) return rc;
  if (!positive_shape(a->lookup_shape, 4) || a->lookup_shape[4] != 4)
    return fail(NGT_ERR_INVALID_ARGUMENT, "Invalid lut shape (NDHWC) with C=4");
  if (a->dtype != NGT_F32 && a->dtype != NGT_F64) return fail(NGT_ERR_UNSUPPORTED, "sample_lut: dtype must be F32 or F64");
  if (!a->separate_camera_batch && a->lookup_shape[0] != a->input_shape[0])
    return fail(NGT_ERR_INVALID_ARGUMENT, "camera batch must match data batch when not using global sampling.");
  if (a->interpolation < NGT_NEAREST || a->interpolation > NGT_MAX)
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut: invalid interpolation");
  if (a->boundary < NGT_BORDER || a->boundary > NGT_WRAP) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut: invalid boundary");
  if (a->mipmapping < NGT_MIP_NONE || a->mipmapping > NGT_MIP_LINEAR)
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut: invalid mipmapping");
  if (a->mipmapping != NGT_MIP_NONE && !mip_levels_ok(a->input_shape, a->num_mipmaps))
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut: num_mipmaps out of range for the grid size");
  if (a->normalized_coords && a->cell_center_offset != 0.5f)
    return fail(NGT_ERR_INVALID_ARGUMENT, "Invalid cell center offset must be 0.5 when using normalized coordinates.");
  if (!a->input || !a->lookup) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut: null pointer");
  if ((rc = check_aligned("sample_lut", elem_size(a->dtype),
                          {{"input", a->input}, {"lookup", a->lookup}, {"output", a->output}})))
    return rc;
  return check_aligned("sample_lut", kScratchAlign, {{"workspace", a->workspace}});
}

template <class T>
LutParams<T> lut_params(const ngt_sample_lut_args* a) {
  LutParams<T> p = {};
  p.lut = static_cast<const T*>(a->lookup);
  p.din = dims_of(a->input_shape);
  p.dout = dims_of(a->lookup_shape);
  p.N = int(a->input_shape[0]);
  p.V = int(a->lookup_shape[0]);
  p.sep = a->separate_camera_batch ? 1 : 0;
  p.fm = a->interpolation;
  p.bm = a->boundary;
  p.mipmode = a->mipmapping;
  p.bias = a->mip_bias;
  p.cco = T(a->cell_center_offset);
  p.relative = a->relative_coords;
  p.normalized = a->normalized_coords;
  return p;
}

template <class T>
int lut_fwd_typed(const ngt_sample_lut_args* a, cudaStream_t st) {
  LutParams<T> p = lut_params<T>(a);
  p.out = static_cast<T*>(a->output);
  const int levels = a->mipmapping != NGT_MIP_NONE ? a->num_mipmaps : 0;
  int rc = build_mips<T>(a->input_shape, static_cast<const T*>(a->input), levels, a->workspace, a->workspace_bytes, st,
                         p.mips);
  if (rc) return rc;
  const int slots = p.sep ? p.N * p.V : p.N;
  const int C = int(a->input_shape[4]);
  for (int s0 = 0; s0 < slots; s0 += 65535) {
    p.slot0 = s0;
    const dim3 grid(ceil_div_u(p.dout.count(), kBlock), min(65535, slots - s0));
    if (C == 1) k_lut_fwd<1, T><<<grid, kBlock, 0, st>>>(p);
    else if (C == 2) k_lut_fwd<2, T><<<grid, kBlock, 0, st>>>(p);
    else k_lut_fwd<4, T><<<grid, kBlock, 0, st>>>(p);
  }
  return check_launch("ngt_sample_lut_fwd");
}

size_t lut_gather_bytes(const ngt_sample_lut_grad_args* a) {
  const int64_t osz = a->fwd.lookup_shape[1] * a->fwd.lookup_shape[2] * a->fwd.lookup_shape[3];
  const int64_t ns = (a->fwd.separate_camera_batch ? a->fwd.lookup_shape[0] : 1) * osz;
  return gather_bytes(ns, dims_of(a->fwd.input_shape), a->fwd.boundary);
}

template <class T>
int lut_bwd_typed(const ngt_sample_lut_grad_args* a, cudaStream_t st) {
  LutParams<T> p = lut_params<T>(&a->fwd);
  p.out_grad = static_cast<const T*>(a->output_grad);
  p.in_grad = static_cast<T*>(a->input_grad);
  p.lut_grad = static_cast<T*>(a->lookup_grad);
  build_mips<T>(a->fwd.input_shape, static_cast<const T*>(a->fwd.input), 0, nullptr, 0, st, p.mips);
  const int C = int(a->fwd.input_shape[4]);
  const int64_t vsz = p.din.count();
  if (cudaMemsetAsync(p.in_grad, 0, size_t(p.N * vsz * C) * sizeof(T), st) != cudaSuccess)
    return check_launch("sample_lut_bwd memset");
  const int reference = a->grad_mode == NGT_GRAD_REFERENCE;
  if (reference) {
    const size_t need = size_t(p.N * vsz) * sizeof(unsigned);
    if (!a->workspace || a->workspace_bytes < need)
      return fail(NGT_ERR_WORKSPACE, "sample_lut_bwd: reference mode needs %zu workspace bytes", need);
    p.count = static_cast<unsigned*>(a->workspace);
    if (cudaMemsetAsync(p.count, 0, need, st) != cudaSuccess) return check_launch("sample_lut_bwd memset");
  }
  const int det = !reference && a->deterministic;
  if (det) {
    const size_t need = lut_gather_bytes(a);
    if (!a->workspace || a->workspace_bytes < need)
      return fail(NGT_ERR_WORKSPACE, "sample_lut_bwd: deterministic mode needs %zu workspace bytes", need);
  }
  const dim3 grid(ceil_div_u(p.dout.count(), kBlock), unsigned(p.V));
  if (C == 1) k_lut_bwd<1, T><<<grid, kBlock, 0, st>>>(p, reference, det);
  else if (C == 2) k_lut_bwd<2, T><<<grid, kBlock, 0, st>>>(p, reference, det);
  else k_lut_bwd<4, T><<<grid, kBlock, 0, st>>>(p, reference, det);
  if (det) {
    const int64_t ns = (p.sep ? int64_t(p.V) : 1) * p.dout.count();
    for (int b = 0; b < p.N; ++b) {
      T* ig = p.in_grad + int64_t(b) * vsz * C;
      cudaError_t e;
      if (C == 1) e = gather_adjoint<1, T>(LutSource<1, T>{p, b}, ns, p.din, p.bm, a->workspace, ig, 0, st);
      else if (C == 2) e = gather_adjoint<2, T>(LutSource<2, T>{p, b}, ns, p.din, p.bm, a->workspace, ig, 0, st);
      else e = gather_adjoint<4, T>(LutSource<4, T>{p, b}, ns, p.din, p.bm, a->workspace, ig, 0, st);
      if (e != cudaSuccess) return check_launch("sample_lut_bwd memset");
    }
  }
  if (reference) {
    const int64_t n = p.N * vsz;
    const unsigned nb = ceil_div_u(n, kBlock);
    if (C == 1) k_normalize_count<1, T><<<nb, kBlock, 0, st>>>(p.in_grad, p.count, n);
    else if (C == 2) k_normalize_count<2, T><<<nb, kBlock, 0, st>>>(p.in_grad, p.count, n);
    else k_normalize_count<4, T><<<nb, kBlock, 0, st>>>(p.in_grad, p.count, n);
  }
  return check_launch("ngt_sample_lut_bwd");
}

int validate_xf(const ngt_sample_transform_args* a) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: null arguments");
  int rc = validate_grid(a->input_shape, "sample_transform");
  if (rc) return rc;
  if (!positive_shape(a->output_dhw, 3)) return fail(NGT_ERR_INVALID_ARGUMENT, "Invalid output_shape");
  if (a->dtype != NGT_F32 && a->dtype != NGT_F64)
    return fail(NGT_ERR_UNSUPPORTED, "sample_transform: dtype must be F32 or F64");
  if (a->num_cameras <= 0) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: num_cameras must be positive");
  if (!a->separate_camera_batch && a->num_cameras != a->input_shape[0])
    return fail(NGT_ERR_INVALID_ARGUMENT, "camera batch must match data batch when not using global sampling.");
  if (!(a->interpolation == NGT_NEAREST || a->interpolation == NGT_LINEAR || a->interpolation == NGT_QUADRATIC))
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: invalid interpolation");
  if (a->boundary != NGT_BORDER && a->boundary != NGT_CLAMP)
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: invalid boundary");
  if (!(a->coordinate_mode == NGT_TRANSFORM_LINDEPTH || a->coordinate_mode == NGT_TRANSFORM_LINDEPTH_REVERSE ||
        a->coordinate_mode == NGT_TRANSFORM || a->coordinate_mode == NGT_TRANSFORM_REVERSE))
    return fail(NGT_ERR_INVALID_ARGUMENT, "invalid coordinate_mode.");
  if (a->mipmapping < NGT_MIP_NONE || a->mipmapping > NGT_MIP_LINEAR)
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: invalid mipmapping");
  if (a->mipmapping != NGT_MIP_NONE && !mip_levels_ok(a->input_shape, a->num_mipmaps))
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: num_mipmaps out of range for the grid size");
  if (!a->input || !a->matrix_m || !a->matrix_v || !a->matrix_p || !a->frustum)
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: null pointer");
  if ((rc = check_aligned("sample_transform", elem_size(a->dtype), {{"input", a->input}, {"output", a->output}})) ||
      (rc = check_aligned("sample_transform", sizeof(float), {{"matrix_m", a->matrix_m}, {"matrix_v", a->matrix_v},
                                                              {"matrix_p", a->matrix_p}, {"frustum", a->frustum}})))
    return rc;
  return check_aligned("sample_transform", kScratchAlign, {{"workspace", a->workspace}});
}

template <class T>
XfParams<T> xf_params(const ngt_sample_transform_args* a) {
  XfParams<T> p = {};
  p.M = a->matrix_m;
  p.V = a->matrix_v;
  p.P = a->matrix_p;
  p.F = a->frustum;
  p.din = dims_of(a->input_shape);
  p.dout = Dims{int(a->output_dhw[2]), int(a->output_dhw[1]), int(a->output_dhw[0])};
  p.N = int(a->input_shape[0]);
  p.ncam = a->num_cameras;
  p.sep = a->separate_camera_batch ? 1 : 0;
  p.fm = a->interpolation;
  p.bm = a->boundary;
  p.mipmode = a->mipmapping;
  p.cm = a->coordinate_mode;
  p.bias = a->mip_bias;
  p.cco = T(a->cell_center_offset);
  return p;
}

template <class T>
int xf_fwd_typed(const ngt_sample_transform_args* a, cudaStream_t st) {
  XfParams<T> p = xf_params<T>(a);
  p.out = static_cast<T*>(a->output);
  const int levels = a->mipmapping != NGT_MIP_NONE ? a->num_mipmaps : 0;
  int rc = build_mips<T>(a->input_shape, static_cast<const T*>(a->input), levels, a->workspace, a->workspace_bytes, st,
                         p.mips);
  if (rc) return rc;
  const int slots = p.sep ? p.N * p.ncam : p.N;
  const int C = int(a->input_shape[4]);
  for (int s0 = 0; s0 < slots; s0 += 65535) {
    p.slot0 = s0;
    const dim3 grid(ceil_div_u(p.dout.count(), kBlock), min(65535, slots - s0));
    if (C == 1) k_xf_fwd<1, T><<<grid, kBlock, 0, st>>>(p);
    else if (C == 2) k_xf_fwd<2, T><<<grid, kBlock, 0, st>>>(p);
    else k_xf_fwd<4, T><<<grid, kBlock, 0, st>>>(p);
  }
  return check_launch("ngt_sample_transform_fwd");
}

// Deterministic transform adjoint workspace: [per-slot cameras][gather buckets].
size_t xf_cams_bytes(const ngt_sample_transform_args* a) {
  const int64_t slots = a->separate_camera_batch ? a->input_shape[0] * a->num_cameras : a->input_shape[0];
  return (size_t(slots) * sizeof(Cam) + 255) & ~size_t(255);
}

int64_t xf_det_samples(const ngt_sample_transform_args* a) {
  return (a->separate_camera_batch ? int64_t(a->num_cameras) : 1) * a->output_dhw[0] * a->output_dhw[1] *
         a->output_dhw[2];
}

size_t xf_det_bytes(const ngt_sample_transform_grad_args* a) {
  return xf_cams_bytes(&a->fwd) + gather_bytes(xf_det_samples(&a->fwd), dims_of(a->fwd.input_shape), a->fwd.boundary);
}

template <class T>
int xf_bwd_typed(const ngt_sample_transform_grad_args* a, cudaStream_t st) {
  XfParams<T> p = xf_params<T>(&a->fwd);
  p.out_grad = static_cast<const T*>(a->output_grad);
  p.in_grad = static_cast<T*>(a->input_grad);
  const int C = int(a->fwd.input_shape[4]);
  const int64_t vsz = p.din.count();
  if (cudaMemsetAsync(p.in_grad, 0, size_t(p.N * vsz * C) * sizeof(T), st) != cudaSuccess)
    return check_launch("sample_transform_bwd memset");
  const int reference = a->grad_mode == NGT_GRAD_REFERENCE;
  if (reference) {
    const size_t need = size_t(p.N * vsz) * sizeof(unsigned);
    if (!a->workspace || a->workspace_bytes < need)
      return fail(NGT_ERR_WORKSPACE, "sample_transform_bwd: reference mode needs %zu workspace bytes", need);
    p.count = static_cast<unsigned*>(a->workspace);
    if (cudaMemsetAsync(p.count, 0, need, st) != cudaSuccess) return check_launch("sample_transform_bwd memset");
  }
  const int slots = p.sep ? p.N * p.ncam : p.N;
  if (!reference && a->deterministic) {
    // gather form: each batch entry's samples bucketed by cell, summed per voxel in a fixed order
    const size_t need = xf_det_bytes(a);
    if (!a->workspace || a->workspace_bytes < need)
      return fail(NGT_ERR_WORKSPACE, "sample_transform_bwd: deterministic mode needs %zu workspace bytes", need);
    Cam* cams = static_cast<Cam*>(a->workspace);
    k_xf_cams<T><<<unsigned(slots), 32, 0, st>>>(p, cams);
    char* gw = static_cast<char*>(a->workspace) + xf_cams_bytes(&a->fwd);
    const int64_t ns = xf_det_samples(&a->fwd);
    for (int b = 0; b < p.N; ++b) {
      T* ig = p.in_grad + int64_t(b) * vsz * C;
      cudaError_t e;
      if (C == 1) e = gather_adjoint<1, T>(XfSource<1, T>{p, cams, b}, ns, p.din, p.bm, gw, ig, 0, st);
      else if (C == 2) e = gather_adjoint<2, T>(XfSource<2, T>{p, cams, b}, ns, p.din, p.bm, gw, ig, 0, st);
      else e = gather_adjoint<4, T>(XfSource<4, T>{p, cams, b}, ns, p.din, p.bm, gw, ig, 0, st);
      if (e != cudaSuccess) return check_launch("sample_transform_bwd memset");
    }
    return check_launch("ngt_sample_transform_bwd");
  }
  for (int s0 = 0; s0 < slots; s0 += 65535) {
    p.slot0 = s0;
    const dim3 grid(ceil_div_u(p.dout.count(), kBlock), min(65535, slots - s0));
    if (C == 1) k_xf_bwd<1, T><<<grid, kBlock, 0, st>>>(p, reference);
    else if (C == 2) k_xf_bwd<2, T><<<grid, kBlock, 0, st>>>(p, reference);
    else k_xf_bwd<4, T><<<grid, kBlock, 0, st>>>(p, reference);
  }
  if (reference) {
    const int64_t n = p.N * vsz;
    const unsigned nb = ceil_div_u(n, kBlock);
    if (C == 1) k_normalize_count<1, T><<<nb, kBlock, 0, st>>>(p.in_grad, p.count, n);
    else if (C == 2) k_normalize_count<2, T><<<nb, kBlock, 0, st>>>(p.in_grad, p.count, n);
    else k_normalize_count<4, T><<<nb, kBlock, 0, st>>>(p.in_grad, p.count, n);
  }
  return check_launch("ngt_sample_transform_bwd");
}

}  // namespace
}  // namespace ngt

using namespace ngt;

extern "C" size_t ngt_mip_bytes(int32_t dtype, const int64_t input_shape[5], int32_t levels) {
  if (!input_shape || levels <= 0) return 0;
  return mip_bytes(dtype, input_shape, levels);
}

extern "C" int ngt_mip_build(int32_t dtype, const int64_t input_shape[5], const void* input, int32_t levels,
                             void* pyramid, size_t pyramid_bytes, void* stream) {
  if (!input_shape || !input) return fail(NGT_ERR_INVALID_ARGUMENT, "mip_build: null pointer");
  int rc = validate_grid(input_shape, "mip_build");
  if (rc) return rc;
  if (!mip_levels_ok(input_shape, levels)) return fail(NGT_ERR_INVALID_ARGUMENT, "mip_build: levels out of range");
  if ((dtype == NGT_F32 || dtype == NGT_F64) &&
      ((rc = check_aligned("mip_build", elem_size(dtype), {{"input", input}})) ||
       (rc = check_aligned("mip_build", kScratchAlign, {{"pyramid", pyramid}}))))
    return rc;
  if (dtype == NGT_F32) {
    Mips<float> m;
    return build_mips<float>(input_shape, static_cast<const float*>(input), levels, pyramid, pyramid_bytes,
                             as_stream(stream), m);
  }
  if (dtype == NGT_F64) {
    Mips<double> m;
    return build_mips<double>(input_shape, static_cast<const double*>(input), levels, pyramid, pyramid_bytes,
                              as_stream(stream), m);
  }
  return fail(NGT_ERR_UNSUPPORTED, "mip_build: dtype must be F32 or F64");
}

extern "C" size_t ngt_sample_lut_fwd_workspace_bytes(const ngt_sample_lut_args* a) {
  if (!a || a->mipmapping == NGT_MIP_NONE) return 0;
  return mip_bytes(a->dtype, a->input_shape, a->num_mipmaps);
}

extern "C" int ngt_sample_lut_fwd(const ngt_sample_lut_args* a, void* stream) {
  int rc = validate_lut(a);
  if (rc) return rc;
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut: null output");
  if (a->dtype == NGT_F64) return lut_fwd_typed<double>(a, as_stream(stream));
  return lut_fwd_typed<float>(a, as_stream(stream));
}

extern "C" size_t ngt_sample_lut_bwd_workspace_bytes(const ngt_sample_lut_grad_args* a) {
  if (!a) return 0;
  if (a->grad_mode == NGT_GRAD_EXACT && a->deterministic) return lut_gather_bytes(a);
  if (a->grad_mode != NGT_GRAD_REFERENCE) return 0;
  const int64_t* s = a->fwd.input_shape;
  return size_t(s[0] * s[1] * s[2] * s[3]) * sizeof(unsigned);
}

extern "C" int ngt_sample_lut_bwd(const ngt_sample_lut_grad_args* a, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut_bwd: null arguments");
  int rc = validate_lut(&a->fwd);
  if (rc) return rc;
  if (a->fwd.mipmapping != NGT_MIP_NONE) return fail(NGT_ERR_UNSUPPORTED, "gradients of mipmapped sampling are not supported");
  if (!a->output_grad || !a->input_grad) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut_bwd: null pointer");
  if ((rc = check_aligned("sample_lut_bwd", elem_size(a->fwd.dtype),
                          {{"output_grad", a->output_grad}, {"input_grad", a->input_grad},
                           {"lookup_grad", a->lookup_grad}})) ||
      (rc = check_aligned("sample_lut_bwd", kScratchAlign, {{"workspace", a->workspace}})))
    return rc;
  if (a->grad_mode != NGT_GRAD_EXACT && a->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_lut_bwd: invalid grad_mode");
  if (a->deterministic && a->grad_mode == NGT_GRAD_EXACT && a->fwd.interpolation != NGT_LINEAR)
    return fail(NGT_ERR_UNSUPPORTED, "sample_lut_bwd: the deterministic gather form is for LINEAR interpolation");
  if (a->fwd.dtype == NGT_F64) return lut_bwd_typed<double>(a, as_stream(stream));
  return lut_bwd_typed<float>(a, as_stream(stream));
}

extern "C" size_t ngt_sample_transform_fwd_workspace_bytes(const ngt_sample_transform_args* a) {
  if (!a || a->mipmapping == NGT_MIP_NONE) return 0;
  return mip_bytes(a->dtype, a->input_shape, a->num_mipmaps);
}

extern "C" int ngt_sample_transform_fwd(const ngt_sample_transform_args* a, void* stream) {
  int rc = validate_xf(a);
  if (rc) return rc;
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform: null output");
  if (a->dtype == NGT_F64) return xf_fwd_typed<double>(a, as_stream(stream));
  return xf_fwd_typed<float>(a, as_stream(stream));
}

extern "C" size_t ngt_sample_transform_bwd_workspace_bytes(const ngt_sample_transform_grad_args* a) {
  if (!a) return 0;
  if (a->grad_mode == NGT_GRAD_EXACT && a->deterministic) return xf_det_bytes(a);
  if (a->grad_mode != NGT_GRAD_REFERENCE) return 0;
  const int64_t* s = a->fwd.input_shape;
  return size_t(s[0] * s[1] * s[2] * s[3]) * sizeof(unsigned);
}

extern "C" int ngt_sample_transform_bwd(const ngt_sample_transform_grad_args* a, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform_bwd: null arguments");
  int rc = validate_xf(&a->fwd);
  if (rc) return rc;
  if (a->fwd.mipmapping != NGT_MIP_NONE) return fail(NGT_ERR_UNSUPPORTED, "gradients of mipmapped sampling are not supported");
  if (!a->output_grad || !a->input_grad) return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform_bwd: null pointer");
  if ((rc = check_aligned("sample_transform_bwd", elem_size(a->fwd.dtype),
                          {{"output_grad", a->output_grad}, {"input_grad", a->input_grad}})) ||
      (rc = check_aligned("sample_transform_bwd", kScratchAlign, {{"workspace", a->workspace}})))
    return rc;
  if (a->grad_mode != NGT_GRAD_EXACT && a->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "sample_transform_bwd: invalid grad_mode");
  if (a->deterministic && a->grad_mode == NGT_GRAD_EXACT) {
    if (a->fwd.interpolation != NGT_LINEAR)
      return fail(NGT_ERR_UNSUPPORTED, "sample_transform_bwd: the deterministic gather form is for LINEAR interpolation");
    if (xf_det_samples(&a->fwd) >= (int64_t(1) << 31))
      return fail(NGT_ERR_UNSUPPORTED, "sample_transform_bwd: the deterministic gather form takes < 2^31 samples per batch entry");
  }
  if (a->fwd.dtype == NGT_F64) return xf_bwd_typed<double>(a, as_stream(stream));
  return xf_bwd_typed<float>(a, as_stream(stream));
}

extern "C" int ngt_lod_transform(const ngt_lod_args* a, void* stream) {
  if (!a || !a->matrix_mv || !a->matrix_p || !a->frustum || !a->output)
    return fail(NGT_ERR_INVALID_ARGUMENT, "lod_transform: null pointer");
  if (!positive_shape(a->input_dhw, 3) || !positive_shape(a->output_dhw, 3) || a->num_cameras <= 0)
    return fail(NGT_ERR_INVALID_ARGUMENT, "lod_transform: shapes must be positive");
  const int ra = check_aligned("lod_transform", sizeof(float), {{"matrix_mv", a->matrix_mv}, {"matrix_p", a->matrix_p},
                                                                {"frustum", a->frustum}, {"output", a->output}});
  if (ra) return ra;
  int cm;
  if (a->linearize_depth) cm = a->inverse_transform ? NGT_TRANSFORM_LINDEPTH_REVERSE : NGT_TRANSFORM_LINDEPTH;
  else cm = a->inverse_transform ? NGT_TRANSFORM_REVERSE : NGT_TRANSFORM;
  const Dims din{int(a->input_dhw[2]), int(a->input_dhw[1]), int(a->input_dhw[0])};
  const Dims dout{int(a->output_dhw[2]), int(a->output_dhw[1]), int(a->output_dhw[0])};
  const dim3 grid(ceil_div_u(dout.count(), kBlock), unsigned(a->num_cameras));
  k_lod<<<grid, kBlock, 0, as_stream(stream)>>>(a->matrix_mv, a->matrix_p, a->frustum, din, dout, cm,
                                               a->relative_coords, a->output);
  return check_launch("ngt_lod_transform");
}
