// Fused frustum raymarch: per-pixel ray through the volume, sample + blend
// front to back (forward), and its gradients.
//
// Semantics follow the reference kernels kRaymarchGridTransformLindepth
// (raymarch_grid.cu.cc:202-252) and kRaymarchGridTransformLindepthGrad
// (:482-521): rays run from frustum-grid index z = 0.5 to z = max(D'-1,1)+0.5 in
// object space (getRaymarchStep, :173-200); with BORDER they are clipped to the
// box through the outer cell centres (RayGridIntersectionDistances, :109-165)
// with one step of margin; sample positions accumulate ``pos += step``.
//
// GB300 layout: one thread per ray, a 16x8-pixel tile per 128-thread block
// (each warp an 8x4 sub-tile, so the 32 rays of a warp gather from nearby
// cells and hit L1); blockIdx.y enumerates (batch, camera) slots and the
// block's camera matrices are formed once in shared memory.
//
// Host entry points (device code in raymarch_kernels.cuh, instantiated per
// storage type in raymarch_<type>.cu) and the small set-up kernels: cameras,
// ray tables, quad layouts and folds of batches, fixed-point conversion.
#include "raymarch_kernels.cuh"

#include <algorithm>
#include <mutex>

namespace ngt {
namespace {
using namespace rm;

// The largest number of (slot, tile) items a ray table orders (one block sorts them).
constexpr int kMaxOrdered = 4096;

// A slot's inverse projection and inverse model-view in double, formed by the
// 32 lanes of a warp (lanes 0-15 one element of MV^-1, 16-31 one of P^-1).
struct CamD {
  double mvi[16], pi[16];
};

__device__ inline void build_cam_double(const float* M16, const float* V16, const float* P16, CamD& cd,
                                        CamScratch& sh) {
  const int lane = threadIdx.x & 31;
  const int e = lane & 15, r = e >> 2, c = e & 3;
  if (lane < 16) {
    sh.M[e] = (double)M16[c * 4 + r];
    sh.V[e] = (double)V16[c * 4 + r];
  } else {
    sh.P[e] = (double)P16[c * 4 + r];
  }
  __syncwarp();
  if (lane < 16)
    sh.MV[e] = sh.V[r * 4 + 0] * sh.M[0 * 4 + c] + sh.V[r * 4 + 1] * sh.M[1 * 4 + c] +
               sh.V[r * 4 + 2] * sh.M[2 * 4 + c] + sh.V[r * 4 + 3] * sh.M[3 * 4 + c];
  __syncwarp();
  if (lane < 16)
    cd.mvi[e] = inverse_element(sh.MV, r, c);
  else
    cd.pi[e] = inverse_element(sh.P, r, c);
}

// IDXtoOS (transformations.hpp:124-138) in double: index -> NDC -> view space
// (homogeneous divide) -> object space.
__device__ inline void idx_to_os_f64(const CamD& cd, double ix, double iy, double iz, const double dinv[3],
                                     double os[3]) {
  const double ndc[4] = {ix * dinv[0] * 2.0 - 1.0, iy * dinv[1] * 2.0 - 1.0, iz * dinv[2] * 2.0 - 1.0, 1.0};
  double vs[4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
    vs[r] = cd.pi[r * 4 + 0] * ndc[0] + cd.pi[r * 4 + 1] * ndc[1] + cd.pi[r * 4 + 2] * ndc[2] + cd.pi[r * 4 + 3] * ndc[3];
  const double v[4] = {vs[0] / vs[3], vs[1] / vs[3], vs[2] / vs[3], 1.0};
#pragma unroll
  for (int r = 0; r < 3; ++r)
    os[r] = cd.mvi[r * 4 + 0] * v[0] + cd.mvi[r * 4 + 1] * v[1] + cd.mvi[r * 4 + 2] * v[2] + cd.mvi[r * 4 + 3] * v[3];
}

// The ray set-up of ray_setup (getRaymarchStep / RayGridIntersectionDistances,
// raymarch_grid.cu.cc:109-200) carried out in double and rounded once to the
// float start and step the march accumulates, so every ray starts at the float
// nearest its exact start; written as two float4 (start, sample count as int
// bits) and (step, hit).
__global__ void k_build_rays(const __grid_constant__ RayParams p, float4* __restrict__ rays) {
  __shared__ CamD cd;
  __shared__ CamScratch sh;
  int b, c, oslot;
  const int slot = p.slot0 + blockIdx.y;
  slot_to_bc(p, slot, b, c, oslot);
  if (threadIdx.x < 32) build_cam_double(p.M + 16 * b, p.V + 16 * c, p.P + 16 * c, cd, sh);
  __syncthreads();
  int px, py;
  pixel_of_thread(px, py);
  const int tiles_x = (p.W + kTileX - 1) / kTileX;
  px += (blockIdx.x % tiles_x) * kTileX;
  py += (blockIdx.x / tiles_x) * kTileY;
  if (px >= p.W || py >= p.H) return;
  const double dinv[3] = {1.0 / double(p.W), 1.0 / double(p.H), 1.0 / double(p.D)};
  const double zmax = double(max(p.D - 1, 1));
  double s[3], e[3], st[3];
  idx_to_os_f64(cd, px + 0.5, py + 0.5, 0.5, dinv, s);
  idx_to_os_f64(cd, px + 0.5, py + 0.5, zmax + 0.5, dinv, e);
#pragma unroll
  for (int a = 0; a < 3; ++a) st[a] = (e[a] - s[a]) / zmax;
  int steps = p.D;
  bool hit = true;
  if (p.bm == BORDER) {
    const double v[3] = {e[0] - s[0], e[1] - s[1], e[2] - s[2]};
    const double len = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double dir[3] = {v[0] / len, v[1] / len, v[2] / len};
    const double bmax[3] = {double(p.din.x), double(p.din.y), double(p.din.z)};
    double tmin = -INFINITY, tmax = INFINITY;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double half = bmax[a] * 0.5 - 0.5;
      const double co = s[a] - bmax[a] * 0.5;
      const double inv = 1.0 / dir[a];
      const double n = inv * co;
      const double k = fabs(inv) * half;
      tmin = fmax(tmin, -n - k);  // fmax / fmin skip the NaN of an axis-parallel ray's inf * 0
      tmax = fmin(tmax, k - n);
    }
    hit = !(tmin > tmax || tmax < 0.0);
    if (hit) {
      const double t0 = fmax(tmin - 1.0, 0.0);
      double e2[3], s2[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        e2[a] = s[a] + dir[a] * (tmax + 1.0);
        s2[a] = s[a] + dir[a] * t0;
      }
      const double ss = sqrt(st[0] * st[0] + st[1] * st[1] + st[2] * st[2]);
      const double d0 = s2[0] - e2[0], d1 = s2[1] - e2[1], d2 = s2[2] - e2[2];
      const double q = sqrt(d0 * d0 + d1 * d1 + d2 * d2) / ss;
      steps = q < double(kMaxSteps) ? int(q) + 2 : kMaxSteps;
#pragma unroll
      for (int a = 0; a < 3; ++a) s[a] = s2[a];
    } else {
      steps = 0;
      s[0] = s[1] = s[2] = 0.0;
    }
  }
  float4* o = rays + 2 * ((int64_t(slot) * p.H + py) * p.W + px);
  o[0] = make_float4(float(s[0]), float(s[1]), float(s[2]), __int_as_float(steps));
  o[1] = make_float4(float(st[0]), float(st[1]), float(st[2]), hit ? 1.0f : 0.0f);
}

// The summed sample counts of the rays of every (slot, tile) item, one block each.
__global__ void k_tile_cost(const __grid_constant__ RayParams p, const float4* __restrict__ rays, int tiles,
                            int* __restrict__ cost) {
  const int item = int(blockIdx.x);
  const int slot = item / tiles, tile = item - slot * tiles;
  int px, py;
  pixel_of_thread(px, py);
  const int tiles_x = (p.W + kTileX - 1) / kTileX;
  px += (tile % tiles_x) * kTileX;
  py += (tile / tiles_x) * kTileY;
  int n = 0;
  if (px < p.W && py < p.H) {
    const float4* q = rays + 2 * ((int64_t(slot) * p.H + py) * p.W + px);
    n = q[1].w != 0.0f ? __float_as_int(q[0].w) : 0;
  }
  __shared__ int part[kThreads / 32];
  int v = n;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kThreads / 32; ++w) t += part[w];
    cost[item] = t;
  }
}

// ``order`` = the n <= kMaxOrdered items by descending cost (ties by item), one
// block sorting (cost, item) keys bitonically in shared memory.
__global__ void __launch_bounds__(1024) k_tile_order(const int* __restrict__ cost, int n, int* __restrict__ order) {
  __shared__ unsigned long long key[kMaxOrdered];
  for (int i = threadIdx.x; i < kMaxOrdered; i += blockDim.x)
    key[i] = i < n ? ((unsigned long long)(0x7fffffff - cost[i]) << 32) | unsigned(i) : ~0ull;
  __syncthreads();
  for (int k = 2; k <= kMaxOrdered; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < kMaxOrdered; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = key[i], b = key[l];
          if ((a > b) == ((i & k) == 0)) {
            key[i] = b;
            key[l] = a;
          }
        }
      }
      __syncthreads();
    }
  for (int i = threadIdx.x; i < n; i += blockDim.x) order[i] = int(key[i] & 0xffffffffu);
}

// Every (batch, camera) slot's camera, one warp per slot, formed once per call
// into ``cams`` for the raymarch blocks to copy.
__global__ void k_build_cams(RayParams p, Cam* __restrict__ cams) {
  __shared__ Cam cam;
  __shared__ CamScratch sh;
  int b, c, oslot;
  slot_to_bc(p, blockIdx.x, b, c, oslot);
  build_cam_warp(p.M + 16 * b, p.V + 16 * c, p.P + 16 * c, p.F + 6 * c, cam, sh);
  __syncwarp();
  const float* src = reinterpret_cast<const float*>(&cam);
  float* dst = reinterpret_cast<float*>(cams + blockIdx.x);
  for (int i = threadIdx.x; i < int(sizeof(Cam) / sizeof(float)); i += 32) dst[i] = src[i];
}

// grad (+)= fixed-point sums times 2^-E, in the compute type.
template <class S>
__global__ void k_fix_convert(const unsigned long long* __restrict__ fix, const FixStats* fst, int64_t rays,
                              S* __restrict__ grad, int64_t n, int accumulate) {
  const int e = fix_exponent(fst, rays);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    S v;
    fixed_value((long long)fix[i], e, v);  // in the compute type: float data never goes through double
    grad[i] = accumulate ? grad[i] + v : v;
  }
}

// kNormalize3DGradients<T,SetZero,AddGrad> (raymarch_grid.cu.cc:458-480): add the
// camera's buffered gradient divided by the summed weights, then clear both.
template <int C, class S>
__global__ void k_normalize_add(S* __restrict__ grad, S* __restrict__ buf, S* __restrict__ wsum, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const S w = wsum[i];
  if (w > S(0)) {
    const S inv = S(1) / w;
#pragma unroll
    for (int c = 0; c < C; ++c) grad[i * C + c] += buf[i * C + c] * inv;
  }
#pragma unroll
  for (int c = 0; c < C; ++c) buf[i * C + c] = S(0);
  wsum[i] = S(0);
}

// ------------------------------------------------------------- host side
int validate(const ngt_raymarch_args* a, int& cin, int& cb) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: null arguments");
  if (!positive_shape(a->input_shape, 5) || !positive_shape(a->output_dhw, 3))
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: shapes must be positive");
  cin = int(a->input_shape[4]);
  if (!valid_channels(cin)) return fail(NGT_ERR_INVALID_ARGUMENT, "Only 1,2 and 4 Channel supported.");
  cb = cin;
  if (a->emission_channels) {
    if (cin != 1 || !(a->emission_channels == 2 || a->emission_channels == 4))
      return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: emission expansion needs a 1-channel input and 2 or 4 channels");
    cb = a->emission_channels;
  }
  if (!a->input || !a->matrix_m || !a->matrix_v || !a->matrix_p || !a->frustum)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: null pointer");
  if (a->num_cameras <= 0) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: num_cameras must be positive");
  if (!a->separate_camera_batch && a->num_cameras != a->input_shape[0])
    return fail(NGT_ERR_INVALID_ARGUMENT, "camera batch must match data batch when not using global sampling.");
  if (a->interpolation < NGT_NEAREST || a->interpolation > NGT_MAX)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: invalid interpolation");
  if (a->boundary < NGT_BORDER || a->boundary > NGT_WRAP) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: invalid boundary");
  if (!(a->blending_mode == NGT_BEER_LAMBERT || a->blending_mode == NGT_ALPHA ||
        a->blending_mode == NGT_ALPHA_ADDITIVE || a->blending_mode == NGT_ADDITIVE))
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: invalid blending_mode");
  if (a->dtype < NGT_F32 || a->dtype > NGT_F16) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: invalid dtype");
  if (a->input_shape[1] > (1 << 30) || a->output_dhw[1] * a->output_dhw[2] > (int64_t(1) << 31))
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: shape too large");
  int rc;
  if ((rc = check_aligned("raymarch", storage_bytes(a->dtype), {{"input", a->input}})) ||
      (rc = check_aligned("raymarch", arith_bytes(a->dtype), {{"output", a->output}})) ||
      (rc = check_aligned("raymarch", sizeof(float), {{"matrix_m", a->matrix_m}, {"matrix_v", a->matrix_v},
                                                      {"matrix_p", a->matrix_p}, {"frustum", a->frustum}})) ||
      (rc = check_aligned("raymarch", kScratchAlign,
                          {{"cameras", a->cameras}, {"workspace", a->workspace}, {"rays", a->rays}})) ||
      (rc = check_aligned("raymarch", 256, {{"quad", a->quad}})))
    return rc;
  return NGT_OK;
}

RayParams make_params(const ngt_raymarch_args* a) {
  RayParams p = {};
  p.input = a->input;
  p.output = a->output;
  p.M = a->matrix_m;
  p.V = a->matrix_v;
  p.P = a->matrix_p;
  p.F = a->frustum;
  p.din = Dims{int(a->input_shape[3]), int(a->input_shape[2]), int(a->input_shape[1])};
  p.D = int(a->output_dhw[0]);
  p.H = int(a->output_dhw[1]);
  p.W = int(a->output_dhw[2]);
  p.N = int(a->input_shape[0]);
  p.ncam = a->num_cameras;
  p.sep = a->separate_camera_batch ? 1 : 0;
  p.fm = a->interpolation;
  p.bm = a->boundary;
  p.blend = a->blending_mode;
  for (int i = 0; i < 4; ++i) p.scale[i] = a->emission_scale[i];
  p.rays = static_cast<const float4*>(a->rays);
  p.order = nullptr;
  return p;
}

int num_slots(const RayParams& p) { return p.sep ? p.N * p.ncam : p.N; }

int launch_dtype(int dtype, int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p) {
  switch (dtype) {
    case NGT_F32: return launch_f32(which, cin, cb, grid, st, p);
    case NGT_F64: return launch_f64(which, cin, cb, grid, st, p);
    case NGT_BF16: return launch_bf16(which, cin, cb, grid, st, p);
    case NGT_F16: return launch_f16(which, cin, cb, grid, st, p);
  }
  return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: invalid dtype");
}

// Scene, plane and in-plane position of this thread of a 1-D launch over the
// scenes' 32x8 blocks (block_end / nbx / nby); false for padding threads.
__device__ __forceinline__ bool batch_block(const int* block_end, const int* nbx, const int* nby, int count, int dx,
                                            int dy, int& it, int& x, int& y, int& z) {
  const int w = int(blockIdx.x);
  it = 0;
  while (it < count - 1 && block_end[it] <= w) ++it;
  const int local = w - (it ? block_end[it - 1] : 0);
  const int per_plane = nbx[it] * nby[it];
  z = local / per_plane;
  const int r = local - z * per_plane;
  const int by = r / nbx[it], bx = r - by * nbx[it];
  x = bx * 32 + int(threadIdx.x);
  y = by * 8 + int(threadIdx.y);
  return true;
}

// Quad layouts of every scene (blockIdx.z over the concatenated padded planes);
// with flags, also each scene's extinction-sign check.
template <class T>
__global__ void k_quad_build_batch(const __grid_constant__ RayBatch bp, int with_flags, int cb) {
  int it, xq, yq, zl;
  batch_block(bp.qblock_end, bp.qnbx, bp.qnby, bp.count, 32, 8, it, xq, yq, zl);
  const RayParams& p = bp.item[it];
  if (xq >= p.qd.x || yq >= p.qd.y) return;
  const int b = zl / p.qd.z, zq = zl - b * p.qd.z;
  quad_build_at<T>(static_cast<const T*>(p.input), p.din, p.bm,
                   static_cast<typename QuadOf<T>::type*>(const_cast<void*>(p.quad)),
                   with_flags ? bp.flags + it : nullptr, cb > 1 ? p.scale[cb - 1] : 1.0f, xq, yq, zq, b);
}

// Cell gradients of every scene from its quad gradient (blockIdx.z over all planes).
__global__ void k_quad_fold_batch(const __grid_constant__ RayBatch bp) {
  int it, x, y, zl;
  batch_block(bp.cblock_end, bp.cnbx, bp.cnby, bp.count, 32, 8, it, x, y, zl);
  const RayParams& p = bp.item[it];
  if (x >= p.din.x || y >= p.din.y) return;
  const int b = zl / p.din.z, z = zl - b * p.din.z;
  quad_fold_at(p.gquad, p.din, p.bm, static_cast<float*>(p.in_grad), x, y, z, b);
}

// Cameras of every scene's slots (blockIdx.y = scene, blockIdx.x = slot).
__global__ void k_build_cams_batch(const __grid_constant__ RayBatch bp) {
  __shared__ Cam cam;
  __shared__ CamScratch sh;
  const RayParams& p = bp.item[blockIdx.y];
  if (int(blockIdx.x) >= num_slots_dev(p)) return;
  int b, c, oslot;
  slot_to_bc(p, blockIdx.x, b, c, oslot);
  build_cam_warp(p.M + 16 * b, p.V + 16 * c, p.P + 16 * c, p.F + 6 * c, cam, sh);
  __syncwarp();
  const float* src = reinterpret_cast<const float*>(&cam);
  float* dst = reinterpret_cast<float*>(const_cast<Cam*>(p.cams) + blockIdx.x);
  for (int i = threadIdx.x; i < int(sizeof(Cam) / sizeof(float)); i += 32) dst[i] = src[i];
}

int launch_batch_dtype(int dtype, int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp) {
  switch (dtype) {
    case NGT_F32: return launch_batch_f32(which, cin, cb, blocks, st, bp);
    case NGT_BF16: return launch_batch_bf16(which, cin, cb, blocks, st, bp);
    case NGT_F16: return launch_batch_f16(which, cin, cb, blocks, st, bp);
  }
  return fail(NGT_ERR_UNSUPPORTED, "raymarch batch: float or 16-bit storage");
}

size_t compute_size(int dtype) { return dtype == NGT_F64 ? 8 : 4; }

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

Dims in_dims(const ngt_raymarch_args* a) {
  return Dims{int(a->input_shape[3]), int(a->input_shape[2]), int(a->input_shape[1])};
}

int64_t slots_of(const ngt_raymarch_args* a) {
  return a->separate_camera_batch ? a->input_shape[0] * a->num_cameras : a->input_shape[0];
}

// One-channel LINEAR float / 16-bit inputs are gathered through the quad layout.
bool quad_case(const ngt_raymarch_args* a) {
  return a->input_shape[4] == 1 && a->interpolation == NGT_LINEAR && a->dtype != NGT_F64 &&
         a->input_shape[0] * (a->input_shape[1] + 2) <= 65535;
}

size_t quad_bytes(const ngt_raymarch_args* a) {
  const QuadDims q = QuadDims::of(in_dims(a));
  return align256(size_t(a->input_shape[0] * q.count) * (a->dtype == NGT_F32 ? 16 : 8));
}

size_t gquad_bytes(const ngt_raymarch_args* a) {
  return align256(size_t(a->input_shape[0] * QuadDims::of(in_dims(a)).count) * 16);
}

size_t cams_bytes(const ngt_raymarch_args* a) { return align256(size_t(slots_of(a)) * sizeof(Cam)); }

// Exact Beer-Lambert backward needs the extinction-sign flag.
bool needs_sign_flag(const ngt_raymarch_grad_args* a) {
  const int cin = int(a->fwd.input_shape[4]);
  const int cb = a->fwd.emission_channels ? a->fwd.emission_channels : cin;
  return a->grad_mode == NGT_GRAD_EXACT && a->fwd.blending_mode == NGT_BEER_LAMBERT && cb > 1;
}

// A prepared quad layout: [header, 256 bytes: extinction-sign word at 0, sample
// tag at 8][quad input][cached samples, with sample_cache].
constexpr size_t kQuadHeader = 256;
constexpr size_t kSampleTagOffset = 8;

// Cached samples of a prepared quad layout: every (slot, tile) item's 4 warps
// hold D x 32 floats (sample_slot).
size_t samples_bytes(const ngt_raymarch_args* a) {
  if (!a->sample_cache) return 0;
  const int64_t tiles = int64_t(ceil_div_u(a->output_dhw[2], kTileX)) * ceil_div_u(a->output_dhw[1], kTileY);
  return align256(size_t(slots_of(a) * tiles * kThreads * a->output_dhw[0]) * sizeof(float));
}

// SplitMix64's finaliser (a published 64-bit mixing function).
uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Points p at the sample cache of the prepared layout ``a->quad`` when this
// call can keep or use it: one-channel Beer-Lambert with emission through a
// prepared layout sized with sample_cache, and a ray table.  The tag mixes the
// table's address with the render's depth, image and slot counts (the cache's
// layout), so a forward of other rays overwrites it and a call of other sizes
// does not match it; it is odd, never the cleared 0.
void use_sample_cache(const ngt_raymarch_args* a, int cb, RayParams& p) {
  if (!a->quad || !a->sample_cache || !a->rays || !quad_case(a) || a->blending_mode != NGT_BEER_LAMBERT || cb < 2)
    return;
  char* q = const_cast<char*>(static_cast<const char*>(a->quad));
  p.samples = reinterpret_cast<float*>(q + kQuadHeader + quad_bytes(a));
  p.sample_word = reinterpret_cast<unsigned long long*>(q + kSampleTagOffset);
  uint64_t t = mix64(uint64_t(reinterpret_cast<uintptr_t>(a->rays)));
  for (const int64_t v : {a->output_dhw[0], a->output_dhw[1], a->output_dhw[2], slots_of(a)})
    t = mix64(t ^ uint64_t(v));
  p.sample_tag = static_cast<unsigned long long>(t | 1ull);
}

int check_prepared_quad(const ngt_raymarch_args* a) {
  if (a->quad && !quad_case(a))
    return fail(NGT_ERR_INVALID_ARGUMENT,
                "raymarch: a prepared quad layout serves one-channel LINEAR inputs in float or 16-bit storage");
  return NGT_OK;
}

// Workspace layouts (offsets in bytes, 256-aligned).
//   forward:            [cameras][quad input]
//   backward, exact:    [sign flag 256][cameras][quad input][quad gradient]
//   backward, reference:[cameras][gradient buffer][weight sums]
//   backward, exact deterministic: [sign flag 256][pass statistics 256][cameras][fixed-point sums]
struct Layout {
  size_t flag, cams, quad, gquad, buf, wsum, fst, fix, total;
};

Layout fwd_layout(const ngt_raymarch_args* a) {
  Layout l = {};
  l.cams = 0;
  l.quad = cams_bytes(a);
  l.total = l.quad + (quad_case(a) && !a->quad ? quad_bytes(a) : 0);
  return l;
}

Layout bwd_layout(const ngt_raymarch_grad_args* g) {
  const ngt_raymarch_args* a = &g->fwd;
  Layout l = {};
  if (g->grad_mode == NGT_GRAD_REFERENCE) {
    const int64_t vox = a->input_shape[1] * a->input_shape[2] * a->input_shape[3];
    l.cams = 0;
    l.buf = cams_bytes(a);
    l.wsum = l.buf + align256(size_t(vox * a->input_shape[4]) * compute_size(a->dtype));
    l.total = l.wsum + align256(size_t(vox) * compute_size(a->dtype));
    return l;
  }
  if (g->deterministic) {
    const int64_t vox = a->input_shape[1] * a->input_shape[2] * a->input_shape[3];
    l.flag = 0;
    l.fst = 256;
    l.cams = 512;
    l.fix = l.cams + cams_bytes(a);
    l.total = l.fix + align256(size_t(a->input_shape[0] * vox * a->input_shape[4]) * sizeof(unsigned long long));
    return l;
  }
  l.flag = 0;
  l.cams = 256;
  l.quad = l.cams + cams_bytes(a);
  l.gquad = l.quad + (quad_case(a) && !a->quad ? quad_bytes(a) : 0);
  l.total = l.gquad + (quad_case(a) ? gquad_bytes(a) : 0);
  return l;
}

int build_quad(const ngt_raymarch_args* a, void* q, cudaStream_t st, int* neg = nullptr, float scale = 1.0f) {
  const Dims d = in_dims(a);
  const QuadDims qd = QuadDims::of(d);
  CellLaunch l = cell_launch(Dims{qd.x, qd.y, qd.z});
  const int planes = int(qd.z * a->input_shape[0]);
  l.grid.z = unsigned((planes + kQuadPlanes - 1) / kQuadPlanes);
  const dim3 grid = l.grid, blk = l.block;
  switch (a->dtype) {
    case NGT_F32:
      k_quad_build<float><<<grid, blk, 0, st>>>(static_cast<const float*>(a->input), d, a->boundary,
                                                 static_cast<float4*>(q), neg, scale, planes);
      break;
    case NGT_BF16:
      k_quad_build<__nv_bfloat16><<<grid, blk, 0, st>>>(static_cast<const __nv_bfloat16*>(a->input), d,
                                                         a->boundary, static_cast<uint2*>(q), neg, scale, planes);
      break;
    case NGT_F16:
      k_quad_build<__half><<<grid, blk, 0, st>>>(static_cast<const __half*>(a->input), d, a->boundary,
                                                  static_cast<uint2*>(q), neg, scale, planes);
      break;
    default:
      return fail(NGT_ERR_UNSUPPORTED, "raymarch: quad layout needs float or 16-bit storage");
  }
  return NGT_OK;
}

// The call's cameras: the caller's prepared block, else formed into ``at``.
void build_cams(RayParams& p, const ngt_raymarch_args* a, void* at, cudaStream_t st) {
  if (a->cameras) {
    p.cams = static_cast<const Cam*>(a->cameras);
    return;
  }
  Cam* cams = static_cast<Cam*>(at);
  k_build_cams<<<unsigned(num_slots(p)), 32, 0, st>>>(p, cams);
  p.cams = cams;
}

size_t rays_table_bytes(const ngt_raymarch_args* a) {
  return align256(size_t(slots_of(a) * a->output_dhw[1] * a->output_dhw[2]) * 2 * sizeof(float4));
}

int64_t ray_items(const ngt_raymarch_args* a) {
  return slots_of(a) * int64_t(ceil_div_u(a->output_dhw[2], kTileX)) * ceil_div_u(a->output_dhw[1], kTileY);
}

// The item order behind a prepared ray table (ngt_raymarch_rays), or null when
// there are too many items to order.
const int* ray_order(const ngt_raymarch_args* a) {
  if (!a->rays || ray_items(a) > kMaxOrdered) return nullptr;
  return reinterpret_cast<const int*>(static_cast<const char*>(a->rays) + rays_table_bytes(a));
}

int launch_slots(int dtype, int which, int cin, int cb, int tiles, cudaStream_t st, RayParams& p) {
  const int slots = num_slots(p);
  const int* order = p.order;
  p.order = nullptr;
  if (order && (which == FWD || which == BWD_BL || which == FWD_L2_BWD)) {
    // the prepared order: the items with the longest rays dispatched first
    p.order = order;
    p.tiles = tiles;
    p.slot0 = 0;
    const int rc = launch_dtype(dtype, which, cin, cb, dim3(unsigned(tiles * slots)), st, p);
    p.order = order;
    return rc;
  }
  for (int s0 = 0; s0 < slots; s0 += 65535) {
    p.slot0 = s0;
    const int rc = launch_dtype(dtype, which, cin, cb, dim3(tiles, min(65535, slots - s0)), st, p);
    if (rc) {
      p.order = order;
      return rc;
    }
  }
  p.order = order;
  return NGT_OK;
}

}  // namespace
}  // namespace ngt

using namespace ngt;

extern "C" size_t ngt_raymarch_cameras_bytes(const ngt_raymarch_args* a) { return a ? cams_bytes(a) : 0; }

extern "C" int ngt_raymarch_cameras(const ngt_raymarch_args* a, void* cameras, void* stream) {
  int cin, cb;
  const int rc = validate(a, cin, cb);
  if (rc) return rc;
  if (!cameras) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_cameras: null output");
  RayParams p = make_params(a);
  k_build_cams<<<unsigned(num_slots(p)), 32, 0, as_stream(stream)>>>(p, static_cast<Cam*>(cameras));
  return check_launch("ngt_raymarch_cameras");
}

extern "C" size_t ngt_raymarch_rays_bytes(const ngt_raymarch_args* a) {
  if (!a) return 0;
  const size_t n = size_t(ray_items(a));
  // [ray table][item order][item costs]
  return rays_table_bytes(a) + (n <= size_t(kMaxOrdered) ? 2 * align256(n * sizeof(int)) : 0);
}

extern "C" int ngt_raymarch_rays(const ngt_raymarch_args* a, void* rays, void* stream) {
  int cin, cb;
  const int rc = validate(a, cin, cb);
  if (rc) return rc;
  if (!rays || (reinterpret_cast<uintptr_t>(rays) & 15))
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_rays: null or not 16-byte aligned output");
  RayParams p = make_params(a);
  const int tiles = ceil_div_u(p.W, kTileX) * ceil_div_u(p.H, kTileY);
  const int slots = num_slots(p);
  for (int s0 = 0; s0 < slots; s0 += 65535) {
    p.slot0 = s0;
    k_build_rays<<<dim3(tiles, min(65535, slots - s0)), kThreads, 0, as_stream(stream)>>>(p, static_cast<float4*>(rays));
  }
  const int64_t n = ray_items(a);
  if (n <= kMaxOrdered) {
    int* order = reinterpret_cast<int*>(static_cast<char*>(rays) + rays_table_bytes(a));
    int* cost = reinterpret_cast<int*>(reinterpret_cast<char*>(order) + align256(size_t(n) * sizeof(int)));
    k_tile_cost<<<unsigned(n), kThreads, 0, as_stream(stream)>>>(p, static_cast<const float4*>(rays), tiles, cost);
    k_tile_order<<<1, 1024, 0, as_stream(stream)>>>(cost, int(n), order);
  }
  return check_launch("ngt_raymarch_rays");
}

extern "C" size_t ngt_raymarch_quad_bytes(const ngt_raymarch_args* a) {
  return a && quad_case(a) ? kQuadHeader + quad_bytes(a) + samples_bytes(a) : 0;
}

extern "C" int ngt_raymarch_quad(const ngt_raymarch_args* a, void* quad, void* stream) {
  int cin, cb;
  const int rc = validate(a, cin, cb);
  if (rc) return rc;
  if (!quad_case(a))
    return fail(NGT_ERR_UNSUPPORTED,
                "raymarch_quad: the quad layout serves one-channel LINEAR inputs in float or 16-bit storage");
  if (!quad || (reinterpret_cast<uintptr_t>(quad) & 255))
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_quad: null or not 256-byte aligned output");
  cudaStream_t st = as_stream(stream);
  char* q = static_cast<char*>(quad);
  // the sign word and the sample tag
  if (cudaMemsetAsync(q, 0, kSampleTagOffset + sizeof(unsigned long long), st) != cudaSuccess)
    return check_launch("raymarch_quad memset");
  const float scale = cb > 1 ? a->emission_scale[cb - 1] : 1.0f;
  const int r = build_quad(a, q + kQuadHeader, st, reinterpret_cast<int*>(q), scale);
  if (r) return r;
  return check_launch("ngt_raymarch_quad");
}

extern "C" size_t ngt_raymarch_fwd_workspace_bytes(const ngt_raymarch_args* a) {
  return a ? fwd_layout(a).total : 0;
}

namespace {
// The forward of ngt_raymarch_fwd / ngt_raymarch_fwd_l2.  With a workspace the
// cameras are formed once per call and a one-channel LINEAR input is gathered
// through the quad layout; without one every block forms its camera and gathers
// directly (same results).
int raymarch_fwd(const ngt_raymarch_args* a, const void* l2_target, int l2_lc, void* l2_grad, void* l2_loss,
                 const void* l2_bkg, void* stream, const char* name) {
  int cin, cb;
  int rc = validate(a, cin, cb);
  if (rc) return rc;
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: null output");
  RayParams p = make_params(a);
  p.order = ray_order(a);
  if ((rc = check_prepared_quad(a))) return rc;
  p.l2_target = l2_target;
  p.l2_lc = l2_lc;
  p.l2_grad = l2_grad;
  p.l2_loss = l2_loss;
  p.l2_bkg = l2_bkg;
  cudaStream_t st = as_stream(stream);
  if (a->cameras) p.cams = static_cast<const Cam*>(a->cameras);
  if (a->quad) {
    p.quad = static_cast<const char*>(a->quad) + kQuadHeader;
    p.qd = QuadDims::of(p.din);
    use_sample_cache(a, cb, p);
  }
  if (a->workspace) {
    const Layout l = fwd_layout(a);
    if (a->workspace_bytes < l.total)
      return fail(NGT_ERR_WORKSPACE, "raymarch: the forward workspace needs %zu bytes", l.total);
    char* w = static_cast<char*>(a->workspace);
    build_cams(p, a, w + l.cams, st);
    if (quad_case(a) && !a->quad) {
      rc = build_quad(a, w + l.quad, st);
      if (rc) return rc;
      p.quad = w + l.quad;
      p.qd = QuadDims::of(p.din);
    }
  }
  const int tiles = ceil_div_u(p.W, kTileX) * ceil_div_u(p.H, kTileY);
  rc = launch_slots(a->dtype, FWD, cin, cb, tiles, st, p);
  if (rc) return rc;
  return check_launch(name);
}
}  // namespace

extern "C" int ngt_raymarch_fwd(const ngt_raymarch_args* a, void* stream) {
  return raymarch_fwd(a, nullptr, 0, nullptr, nullptr, nullptr, stream, "ngt_raymarch_fwd");
}

extern "C" int ngt_raymarch_fwd_l2(const ngt_raymarch_args* a, const void* target, int32_t loss_channels,
                                   void* image_grad, void* loss, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: null arguments");
  if (!target || !image_grad || !loss) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2: null pointer");
  const int ra = check_aligned("raymarch_fwd_l2", arith_bytes(a->dtype),
                               {{"target", target}, {"image_grad", image_grad}, {"loss", loss}});
  if (ra) return ra;
  const int cb = a->emission_channels ? a->emission_channels : int(a->input_shape[4]);
  if (loss_channels <= 0 || loss_channels > cb)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2: loss_channels must be in 1..%d", cb);
  return raymarch_fwd(a, target, loss_channels, image_grad, loss, nullptr, stream, "ngt_raymarch_fwd_l2");
}

extern "C" int ngt_raymarch_fwd_l2_background(const ngt_raymarch_args* a, const void* background, const void* target,
                                              int32_t loss_channels, void* image_grad, void* loss, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: null arguments");
  if (!background || !target || !image_grad || !loss)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2_background: null pointer");
  const int ra = check_aligned("raymarch_fwd_l2_background", arith_bytes(a->dtype),
                               {{"background", background}, {"target", target}, {"image_grad", image_grad},
                                {"loss", loss}});
  if (ra) return ra;
  const int cb = a->emission_channels ? a->emission_channels : int(a->input_shape[4]);
  if (cb < 2)
    return fail(NGT_ERR_INVALID_ARGUMENT,
                "raymarch_fwd_l2_background: the background needs light channels and an optical depth channel");
  if (a->blending_mode != NGT_BEER_LAMBERT)
    return fail(NGT_ERR_UNSUPPORTED, "raymarch_fwd_l2_background: the transmittance exp(-d) is Beer-Lambert's");
  if (loss_channels <= 0 || loss_channels > cb - 1)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2_background: loss_channels must be in 1..%d", cb - 1);
  return raymarch_fwd(a, target, loss_channels, image_grad, loss, background, stream,
                      "ngt_raymarch_fwd_l2_background");
}

extern "C" size_t ngt_raymarch_bwd_workspace_bytes(const ngt_raymarch_grad_args* a) {
  return a ? bwd_layout(a).total : 0;
}

namespace {
// The image L2 loss of a render fused with its forward and backward
// (ngt_raymarch_fwd_l2_bwd); null for a plain backward.
struct FusedLoss {
  const void* target;
  int lc;
  void* loss;
  const void* background;
};

// Whether the fused call runs as one launch (k_raymarch_fwd_bwd): the exact,
// float-atomic Beer-Lambert adjoint with emission through the quad layout.
bool fused_launch(const ngt_raymarch_grad_args* a) {
  return a->grad_mode == NGT_GRAD_EXACT && !a->deterministic && quad_case(&a->fwd) && needs_sign_flag(a);
}

// ``check_only``: validate the arguments and return before any launch.
int raymarch_bwd_impl(const ngt_raymarch_grad_args* a, const FusedLoss* fl, void* stream, bool check_only = false);
}  // namespace

extern "C" int ngt_raymarch_bwd(const ngt_raymarch_grad_args* a, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd: null arguments");
  return raymarch_bwd_impl(a, nullptr, stream);
}

extern "C" int ngt_raymarch_fwd_l2_bwd(const ngt_raymarch_grad_args* a, const void* background, const void* target,
                                       int32_t loss_channels, void* loss, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2_bwd: null arguments");
  if (!target || !loss || !a->output || !a->output_grad)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2_bwd: null pointer");
  int cin, cb;
  int rc = validate(&a->fwd, cin, cb);
  if (rc) return rc;
  if ((rc = check_aligned("raymarch_fwd_l2_bwd", arith_bytes(a->fwd.dtype),
                          {{"target", target}, {"loss", loss}, {"background", background}})))
    return rc;
  if (background) {
    if (cb < 2)
      return fail(NGT_ERR_INVALID_ARGUMENT,
                  "raymarch_fwd_l2_bwd: the background needs light channels and an optical depth channel");
    if (a->fwd.blending_mode != NGT_BEER_LAMBERT)
      return fail(NGT_ERR_UNSUPPORTED, "raymarch_fwd_l2_bwd: the transmittance exp(-d) is Beer-Lambert's");
  }
  const int top = background ? cb - 1 : cb;
  if (loss_channels <= 0 || loss_channels > top)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2_bwd: loss_channels must be in 1..%d", top);
  const FusedLoss fl = {target, int(loss_channels), loss, background};
  if (!fused_launch(a)) {
    // the two passes: the forward with its loss, then the backward (whose arguments
    // are checked first, so that a rejected call launches nothing)
    if ((rc = raymarch_bwd_impl(a, nullptr, stream, true))) return rc;
    ngt_raymarch_args f = a->fwd;
    f.output = const_cast<void*>(a->output);
    void* ig = const_cast<void*>(a->output_grad);
    rc = background ? ngt_raymarch_fwd_l2_background(&f, background, target, loss_channels, ig, loss, stream)
                    : ngt_raymarch_fwd_l2(&f, target, loss_channels, ig, loss, stream);
    if (rc) return rc;
    return raymarch_bwd_impl(a, nullptr, stream);
  }
  return raymarch_bwd_impl(a, &fl, stream);
}

namespace {
int raymarch_bwd_impl(const ngt_raymarch_grad_args* a, const FusedLoss* fl, void* stream, bool check_only) {
  int cin, cb;
  int rc = validate(&a->fwd, cin, cb);
  if (rc) return rc;
  if (a->fwd.interpolation != NGT_LINEAR)
    return fail(NGT_ERR_UNSUPPORTED, "raymarch gradients support LINEAR interpolation only");
  if (!a->output_grad || !a->input_grad) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd: null pointer");
  if (a->grad_mode != NGT_GRAD_EXACT && a->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd: invalid grad_mode");
  if (a->accumulate && a->grad_mode != NGT_GRAD_EXACT)
    return fail(NGT_ERR_UNSUPPORTED, "raymarch_bwd: accumulate needs the exact gradient");
  if (a->deterministic && a->grad_mode != NGT_GRAD_EXACT)
    return fail(NGT_ERR_UNSUPPORTED, "raymarch_bwd: the deterministic mode computes the exact gradient");
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd: the forward output is required");
  if ((rc = check_aligned("raymarch_bwd", arith_bytes(a->fwd.dtype),
                          {{"output", a->output}, {"output_grad", a->output_grad}, {"input_grad", a->input_grad}})))
    return rc;
  if ((rc = check_prepared_quad(&a->fwd))) return rc;
  const Layout l = bwd_layout(a);
  if (!a->workspace || a->workspace_bytes < l.total)
    return fail(NGT_ERR_WORKSPACE, "raymarch_bwd: needs %zu workspace bytes", l.total);
  if (check_only) return NGT_OK;
  RayParams p = make_params(&a->fwd);
  p.order = ray_order(&a->fwd);
  p.out_fwd = a->output;
  p.out_grad = a->output_grad;
  p.in_grad = a->input_grad;
  cudaStream_t st = as_stream(stream);
  char* w = static_cast<char*>(a->workspace);
  const int64_t vox = p.din.count();
  const size_t cs = compute_size(a->fwd.dtype);
  const int tiles = ceil_div_u(p.W, kTileX) * ceil_div_u(p.H, kTileY);
  build_cams(p, &a->fwd, w + l.cams, st);

  if (a->grad_mode == NGT_GRAD_EXACT && a->deterministic) {
    // statistics pass, fixed-point scatter pass, conversion; the samples are read
    // through the caller's prepared quad layout when there is one (the same values
    // as the direct gathers, two vector loads instead of eight), else directly
    const bool bl = needs_sign_flag(a);
    if (quad_case(&a->fwd) && a->fwd.quad) {
      p.quad = static_cast<const char*>(a->fwd.quad) + kQuadHeader;
      p.qd = QuadDims::of(p.din);
    }
    p.fst = reinterpret_cast<FixStats*>(w + l.fst);
    p.fix = reinterpret_cast<unsigned long long*>(w + l.fix);
    p.nrays = int64_t(num_slots(p)) * p.H * p.W;
    const int64_t n = int64_t(p.N) * vox * cin;
    if (cudaMemsetAsync(w, 0, l.cams, st) != cudaSuccess ||
        cudaMemsetAsync(p.fix, 0, size_t(n) * sizeof(unsigned long long), st) != cudaSuccess)
      return check_launch("raymarch_bwd memset");
    if (bl) {
      p.flag = reinterpret_cast<const int*>(w + l.flag);
      if ((rc = launch_dtype(a->fwd.dtype, SIGN, cin, cb, dim3(1), st, p))) return rc;
    }
    if ((rc = launch_slots(a->fwd.dtype, bl ? BWD_BL_MAX : BWD_EXACT_MAX, cin, cb, tiles, st, p))) return rc;
    if ((rc = launch_slots(a->fwd.dtype, bl ? BWD_BL_FIX : BWD_EXACT_FIX, cin, cb, tiles, st, p))) return rc;
    const unsigned nb = unsigned(std::min<int64_t>((n + 255) / 256, 152 * 16));
    if (a->fwd.dtype == NGT_F64)
      k_fix_convert<double><<<nb, 256, 0, st>>>(p.fix, p.fst, p.nrays, static_cast<double*>(a->input_grad), n,
                                                a->accumulate);
    else
      k_fix_convert<float><<<nb, 256, 0, st>>>(p.fix, p.fst, p.nrays, static_cast<float*>(a->input_grad), n,
                                               a->accumulate);
    return check_launch("ngt_raymarch_bwd");
  }

  if (a->grad_mode == NGT_GRAD_EXACT) {
    const bool quad = quad_case(&a->fwd);
    const bool bl = needs_sign_flag(a);
    const bool prepared = quad && a->fwd.quad;
    if (bl) {
      if (prepared) {
        p.flag = static_cast<const int*>(a->fwd.quad);  // the prepared layout's sign word
      } else {
        p.flag = reinterpret_cast<const int*>(w + l.flag);
        if (cudaMemsetAsync(w + l.flag, 0, sizeof(int), st) != cudaSuccess)
          return check_launch("raymarch_bwd memset");
      }
    }
    if (quad) {
      if (prepared) {
        p.quad = static_cast<const char*>(a->fwd.quad) + kQuadHeader;
        if (bl) use_sample_cache(&a->fwd, cb, p);
      } else {
        // one channel: the quad build also checks the sign of scale * density
        rc = build_quad(&a->fwd, w + l.quad, st, bl ? reinterpret_cast<int*>(w + l.flag) : nullptr,
                        cb > 1 ? p.scale[cb - 1] : 1.0f);
        if (rc) return rc;
        p.quad = w + l.quad;
      }
      p.gquad = reinterpret_cast<float4*>(w + l.gquad);
      p.qd = QuadDims::of(p.din);
      if (cudaMemsetAsync(p.gquad, 0, gquad_bytes(&a->fwd), st) != cudaSuccess)
        return check_launch("raymarch_bwd memset");
    } else if (!a->accumulate && cudaMemsetAsync(a->input_grad, 0, size_t(p.N) * vox * cin * cs, st) != cudaSuccess) {
      return check_launch("raymarch_bwd memset");
    }
    if (bl) {
      if (!quad) {
        rc = launch_dtype(a->fwd.dtype, SIGN, cin, cb, dim3(1), st, p);
        if (rc) return rc;
      }
      if (fl) {
        // forward, loss and backward in one launch (fused_launch): the image and its
        // loss gradient are written to output and output_grad
        p.output = const_cast<void*>(a->output);
        p.l2_target = fl->target;
        p.l2_lc = fl->lc;
        p.l2_grad = const_cast<void*>(a->output_grad);
        p.l2_loss = fl->loss;
        p.l2_bkg = fl->background;
        rc = launch_slots(a->fwd.dtype, FWD_L2_BWD, cin, cb, tiles, st, p);
      } else {
        rc = launch_slots(a->fwd.dtype, BWD_BL, cin, cb, tiles, st, p);  // one-pass, or checkpointed on the flag
      }
      if (rc) return rc;
    } else {
      rc = launch_slots(a->fwd.dtype, BWD_EXACT, cin, cb, tiles, st, p);
      if (rc) return rc;
    }
    if (quad) {
      CellLaunch fl = cell_launch(p.din);
      fl.grid.z = unsigned(p.din.z * p.N);
      k_quad_fold<<<fl.grid, fl.block, 0, st>>>(p.gquad, p.din, p.bm, static_cast<float*>(a->input_grad),
                                                a->accumulate);
    }
    return check_launch("ngt_raymarch_bwd");
  }

  // reference: one (batch, camera) at a time, normalised by summed weights per camera
  if (cudaMemsetAsync(a->input_grad, 0, size_t(p.N) * vox * cin * cs, st) != cudaSuccess)
    return check_launch("raymarch_bwd memset");
  p.wbuf = w + l.buf;
  p.wsum = w + l.wsum;
  if (cudaMemsetAsync(w + l.buf, 0, l.total - l.buf, st) != cudaSuccess) return check_launch("raymarch_bwd memset");
  const int slots = num_slots(p);
  for (int s = 0; s < slots; ++s) {
    p.slot0 = s;
    const int b = p.sep ? s / p.ncam : s;
    rc = launch_dtype(a->fwd.dtype, BWD_REF, cin, cb, dim3(tiles, 1), st, p);
    if (rc) return rc;
    const unsigned nb = ceil_div_u(vox, 256);
    if (a->fwd.dtype == NGT_F64) {
      double* gr = static_cast<double*>(a->input_grad) + int64_t(b) * vox * cin;
      if (cin == 1) k_normalize_add<1, double><<<nb, 256, 0, st>>>(gr, (double*)p.wbuf, (double*)p.wsum, vox);
      else if (cin == 2) k_normalize_add<2, double><<<nb, 256, 0, st>>>(gr, (double*)p.wbuf, (double*)p.wsum, vox);
      else k_normalize_add<4, double><<<nb, 256, 0, st>>>(gr, (double*)p.wbuf, (double*)p.wsum, vox);
    } else {
      float* gr = static_cast<float*>(a->input_grad) + int64_t(b) * vox * cin;
      if (cin == 1) k_normalize_add<1, float><<<nb, 256, 0, st>>>(gr, (float*)p.wbuf, (float*)p.wsum, vox);
      else if (cin == 2) k_normalize_add<2, float><<<nb, 256, 0, st>>>(gr, (float*)p.wbuf, (float*)p.wsum, vox);
      else k_normalize_add<4, float><<<nb, 256, 0, st>>>(gr, (float*)p.wbuf, (float*)p.wsum, vox);
    }
  }
  return check_launch("ngt_raymarch_bwd");
}
}  // namespace

// ------------------------------------------------------------ batched calls
namespace ngt {
namespace {

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

// Scenes that all take the quad layout (one channel, LINEAR, float / 16-bit).
bool batch_quad(const ngt_raymarch_args* const* items, int count) {
  for (int i = 0; i < count; ++i)
    if (!quad_case(items[i])) return false;
  return true;
}

// Workspace of a batch: [work counters and per-scene flags, 256 bytes][cameras of
// each scene][quad layout of each scene][quad gradient of each scene].
size_t batch_bytes(const ngt_raymarch_args* const* items, int count) {
  size_t n = 256;
  const bool quad = batch_quad(items, count);
  for (int i = 0; i < count; ++i) {
    n += cams_bytes(items[i]);
    if (quad) n += quad_bytes(items[i]) + gquad_bytes(items[i]);
  }
  return n;
}

// Validates the scenes and fills bp (scenes ordered by descending work); cameras
// that the caller did not prepare are formed into the workspace.
int make_batch(const ngt_raymarch_args* const* items, int count, char* ws, size_t ws_bytes, RayBatch& bp, int& cin,
               int& cb, int order[kMaxBatch], cudaStream_t st) {
  if (count < 1 || count > kMaxBatch) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: 1 to %d scenes", kMaxBatch);
  int64_t work[kMaxBatch];
  for (int i = 0; i < count; ++i) {
    int ci, cbi;
    const int rc = validate(items[i], ci, cbi);
    if (rc) return rc;
    if (i == 0) {
      cin = ci;
      cb = cbi;
    } else if (ci != cin || cbi != cb || items[i]->dtype != items[0]->dtype) {
      return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: scenes must share dtype and channels");
    }
    if (items[i]->dtype == NGT_F64) return fail(NGT_ERR_UNSUPPORTED, "raymarch batch: float or 16-bit storage");
    order[i] = i;
    work[i] = slots_of(items[i]) * items[i]->output_dhw[0] * items[i]->output_dhw[1] * items[i]->output_dhw[2];
  }
  for (int i = 1; i < count; ++i)  // descending work: large scenes first
    for (int j = i; j > 0 && work[order[j]] > work[order[j - 1]]; --j) {
      const int t = order[j];
      order[j] = order[j - 1];
      order[j - 1] = t;
    }
  if (!ws) return fail(NGT_ERR_WORKSPACE, "raymarch batch: null workspace");
  const int ra = check_aligned("raymarch batch", kScratchAlign, {{"workspace", ws}});
  if (ra) return ra;
  const size_t need = batch_bytes(items, count);
  if (ws_bytes < need) return fail(NGT_ERR_WORKSPACE, "raymarch batch: needs %zu workspace bytes", need);
  bp = RayBatch{};
  bp.count = count;
  bp.counter = reinterpret_cast<int*>(ws);
  bp.flags = reinterpret_cast<int*>(ws) + 2;
  const bool quad = batch_quad(items, count);
  size_t off = 256, qoff = 256, goff = 256;
  for (int k = 0; k < count; ++k) qoff += cams_bytes(items[k]);
  goff = qoff;
  if (quad)
    for (int k = 0; k < count; ++k) goff += quad_bytes(items[k]);
  int total = 0, max_slots = 0, qz = 0, cz = 0;  // block counts of the quad and cell launches
  bool build = false;
  for (int k = 0; k < count; ++k) {
    const ngt_raymarch_args* a = items[order[k]];
    RayParams p = make_params(a);
    if (a->cameras) {
      p.cams = static_cast<const Cam*>(a->cameras);
    } else {
      p.cams = reinterpret_cast<const Cam*>(ws + off);
      build = true;
    }
    off += cams_bytes(a);
    if (quad) {
      p.quad = ws + qoff;
      p.gquad = reinterpret_cast<float4*>(ws + goff);
      p.qd = QuadDims::of(p.din);
      qoff += quad_bytes(a);
      goff += gquad_bytes(a);
      bp.qnbx[k] = (p.qd.x + 31) / 32;
      bp.qnby[k] = (p.qd.y + 7) / 8;
      bp.cnbx[k] = (p.din.x + 31) / 32;
      bp.cnby[k] = (p.din.y + 7) / 8;
      const int64_t qb = int64_t(bp.qnbx[k]) * bp.qnby[k] * p.N * p.qd.z;
      const int64_t cbk = int64_t(bp.cnbx[k]) * bp.cnby[k] * p.N * p.din.z;
      if (int64_t(qz) + qb >= (int64_t(1) << 31) || int64_t(cz) + cbk >= (int64_t(1) << 31))
        return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: grids too large");
      qz += int(qb);
      cz += int(cbk);
      bp.qblock_end[k] = qz;
      bp.cblock_end[k] = cz;
    }
    const int tiles = ceil_div_u(p.W, kTileX) * ceil_div_u(p.H, kTileY);
    const int slots = num_slots(p);
    if (int64_t(total) + int64_t(tiles) * slots >= (int64_t(1) << 31))
      return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: too many tiles");
    total += tiles * slots;
    max_slots = slots > max_slots ? slots : max_slots;
    bp.item[k] = p;
    bp.tiles_per_slot[k] = tiles;
    bp.tile_end[k] = total;
  }
  bp.total = total;
  if (build) {
    if (max_slots > 65535 * 32) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: too many cameras");
    k_build_cams_batch<<<dim3(unsigned(max_slots), unsigned(count)), 32, 0, st>>>(bp);
  }
  return NGT_OK;
}

unsigned persistent_blocks(int blocks_per_sm, int total) {
  const int per = blocks_per_sm > 0 ? blocks_per_sm : kMinBlocks;
  const int64_t n = int64_t(per) * sm_count();
  return unsigned(n < total ? n : (total > 0 ? total : 1));
}

}  // namespace
}  // namespace ngt

namespace ngt {
namespace {

// Quad layouts of a batch (every scene's layout, and with flags the sign check).
int build_quads_batch(int dtype, const RayBatch& bp, int with_flags, int cb, cudaStream_t st) {
  const dim3 grid(unsigned(bp.qblock_end[bp.count - 1])), block(32, 8);
  switch (dtype) {
    case NGT_F32: k_quad_build_batch<float><<<grid, block, 0, st>>>(bp, with_flags, cb); break;
    case NGT_BF16: k_quad_build_batch<__nv_bfloat16><<<grid, block, 0, st>>>(bp, with_flags, cb); break;
    case NGT_F16: k_quad_build_batch<__half><<<grid, block, 0, st>>>(bp, with_flags, cb); break;
    default: return fail(NGT_ERR_UNSUPPORTED, "raymarch batch: quad layout needs float or 16-bit storage");
  }
  return NGT_OK;
}

}  // namespace
}  // namespace ngt

extern "C" size_t ngt_raymarch_batch_workspace_bytes(const ngt_raymarch_args* items, int32_t count) {
  if (!items || count < 1 || count > kMaxBatch) return 0;
  const ngt_raymarch_args* ptrs[kMaxBatch];
  for (int i = 0; i < count; ++i) ptrs[i] = items + i;
  return batch_bytes(ptrs, count);
}

extern "C" int ngt_raymarch_fwd_batch(const ngt_raymarch_args* items, int32_t count, int32_t blocks_per_sm,
                                      void* workspace, size_t workspace_bytes, void* stream) {
  if (!items) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: null scenes");
  const ngt_raymarch_args* ptrs[kMaxBatch];
  if (count < 1 || count > kMaxBatch) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: 1 to %d scenes", kMaxBatch);
  for (int i = 0; i < count; ++i) {
    ptrs[i] = items + i;
    if (!items[i].output) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: null output");
    if (items[i].quad) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: builds its own quad layouts");
  }
  cudaStream_t st = as_stream(stream);
  RayBatch bp;
  int cin = 0, cb = 0, order[kMaxBatch];
  int rc = make_batch(ptrs, count, static_cast<char*>(workspace), workspace_bytes, bp, cin, cb, order, st);
  if (rc) return rc;
  if (cudaMemsetAsync(workspace, 0, 256, st) != cudaSuccess) return check_launch("raymarch batch memset");
  if (bp.item[0].quad) {
    // with the extinction-sign words, for ngt_raymarch_bwd_batch_after_fwd
    rc = build_quads_batch(items[0].dtype, bp, 1, cb, st);
    if (rc) return rc;
  }
  rc = launch_batch_dtype(items[0].dtype, FWD, cin, cb, persistent_blocks(blocks_per_sm, bp.total), st, bp);
  if (rc) return rc;
  return check_launch("ngt_raymarch_fwd_batch");
}

namespace {
// The fused batch's image L2 loss (ngt_raymarch_fwd_l2_bwd_batch); null for a plain backward.
struct FusedLossBatch {
  const void* const* targets;
  int lc;
  void* loss;
};

int raymarch_bwd_batch(const ngt_raymarch_grad_args* items, int32_t count, int32_t blocks_per_sm, void* workspace,
                       size_t workspace_bytes, void* stream, bool reuse, const FusedLossBatch* fl = nullptr) {
  if (!items) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: null scenes");
  if (count < 1 || count > kMaxBatch) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: 1 to %d scenes", kMaxBatch);
  const ngt_raymarch_args* ptrs[kMaxBatch];
  for (int i = 0; i < count; ++i) {
    const ngt_raymarch_grad_args& g = items[i];
    if (!g.output || !g.output_grad || !g.input_grad) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: null pointer");
    const int ra = check_aligned("raymarch batch", arith_bytes(g.fwd.dtype),
                                 {{"output", g.output}, {"output_grad", g.output_grad}, {"input_grad", g.input_grad}});
    if (ra) return ra;
    if (g.fwd.quad) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: builds its own quad layouts");
    if (g.grad_mode != NGT_GRAD_EXACT || g.fwd.blending_mode != NGT_BEER_LAMBERT || g.fwd.interpolation != NGT_LINEAR ||
        g.accumulate)
      return fail(NGT_ERR_UNSUPPORTED, "raymarch batch backward: exact Beer-Lambert gradients of LINEAR sampling, "
                                       "written");
    if (fl) {
      // (checked before make_batch launches anything)
      const int cbi = g.fwd.emission_channels ? g.fwd.emission_channels : int(g.fwd.input_shape[4]);
      if (cbi < 2)
        return fail(NGT_ERR_UNSUPPORTED, "raymarch_fwd_l2_bwd_batch: Beer-Lambert with emission channels");
      if (fl->lc <= 0 || fl->lc > cbi)
        return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2_bwd_batch: loss_channels must be in 1..%d", cbi);
      if (!fl->targets[i]) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: null target");
      const int rt = check_aligned("raymarch batch", arith_bytes(g.fwd.dtype), {{"target", fl->targets[i]}});
      if (rt) return rt;
      if (!quad_case(&g.fwd))
        return fail(NGT_ERR_UNSUPPORTED, "raymarch_fwd_l2_bwd_batch: one-channel LINEAR scenes in float or 16-bit "
                                         "storage (the quad layout); the others take the three batch calls");
    }
    ptrs[i] = &g.fwd;
  }
  cudaStream_t st = as_stream(stream);
  RayBatch bp;
  int cin = 0, cb = 0, order[kMaxBatch];
  int rc = make_batch(ptrs, count, static_cast<char*>(workspace), workspace_bytes, bp, cin, cb, order, st);
  if (rc) return rc;
  if (cb < 2) return fail(NGT_ERR_UNSUPPORTED, "raymarch batch backward: Beer-Lambert needs 2 or 4 blend channels");
  const bool quad = bp.item[0].quad != nullptr;
  for (int k = 0; k < count; ++k) {
    RayParams& p = bp.item[k];
    p.out_fwd = items[order[k]].output;
    p.out_grad = items[order[k]].output_grad;
    p.in_grad = items[order[k]].input_grad;
    if (fl) {  // the forward writes the image and its loss gradient that the backward reads
      p.output = const_cast<void*>(items[order[k]].output);
      p.l2_target = fl->targets[order[k]];
      p.l2_lc = fl->lc;
      p.l2_grad = const_cast<void*>(items[order[k]].output_grad);
      p.l2_loss = fl->loss;
    }
    // the quad path writes every cell gradient in its fold; the direct path adds
    if (!quad && cudaMemsetAsync(p.in_grad, 0, size_t(p.N) * p.din.count() * cin * sizeof(float), st) != cudaSuccess)
      return check_launch("raymarch batch memset");
  }
  // the work counter; the sign words too unless the forward's are reused
  if (cudaMemsetAsync(workspace, 0, (reuse && quad) ? sizeof(int) : 256, st) != cudaSuccess)
    return check_launch("raymarch batch memset");
  const int dtype = items[0].fwd.dtype;
  if (quad) {
    // quad gradients are contiguous: from the first scene's to the end of the workspace layout
    char* g0 = reinterpret_cast<char*>(bp.item[0].gquad);
    for (int k = 1; k < count; ++k) g0 = std::min(g0, reinterpret_cast<char*>(bp.item[k].gquad));
    const size_t gbytes = batch_bytes(ptrs, count) - size_t(g0 - static_cast<char*>(workspace));
    if (cudaMemsetAsync(g0, 0, gbytes, st) != cudaSuccess) return check_launch("raymarch batch memset");
    rc = reuse ? NGT_OK : build_quads_batch(dtype, bp, 1, cb, st);
  } else {
    rc = launch_batch_dtype(dtype, SIGN, cin, cb, unsigned(sm_count() * 2), st, bp);
  }
  if (rc) return rc;
  const unsigned blocks = persistent_blocks(blocks_per_sm, bp.total);
  rc = launch_batch_dtype(dtype, fl ? FWD_L2_BWD : BWD_BL, cin, cb, blocks, st, bp);
  if (rc) return rc;
  if (quad) k_quad_fold_batch<<<unsigned(bp.cblock_end[count - 1]), dim3(32, 8), 0, st>>>(bp);
  return check_launch(fl ? "ngt_raymarch_fwd_l2_bwd_batch"
                         : reuse ? "ngt_raymarch_bwd_batch_after_fwd" : "ngt_raymarch_bwd_batch");
}
}  // namespace

extern "C" int ngt_raymarch_fwd_l2_bwd_batch(const ngt_raymarch_grad_args* items, const void* const* targets,
                                             int32_t count, int32_t loss_channels, void* loss, int32_t blocks_per_sm,
                                             void* workspace, size_t workspace_bytes, void* stream) {
  if (!targets || !loss) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_fwd_l2_bwd_batch: null pointer");
  if (!items) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch batch: null scenes");
  const int ra = check_aligned("raymarch_fwd_l2_bwd_batch", arith_bytes(items[0].fwd.dtype), {{"loss", loss}});
  if (ra) return ra;
  const FusedLossBatch fl = {targets, int(loss_channels), loss};
  return raymarch_bwd_batch(items, count, blocks_per_sm, workspace, workspace_bytes, stream, false, &fl);
}

extern "C" int ngt_raymarch_bwd_batch(const ngt_raymarch_grad_args* items, int32_t count, int32_t blocks_per_sm,
                                      void* workspace, size_t workspace_bytes, void* stream) {
  return raymarch_bwd_batch(items, count, blocks_per_sm, workspace, workspace_bytes, stream, false);
}

extern "C" int ngt_raymarch_bwd_batch_after_fwd(const ngt_raymarch_grad_args* items, int32_t count,
                                                int32_t blocks_per_sm, void* workspace, size_t workspace_bytes,
                                                void* stream) {
  return raymarch_bwd_batch(items, count, blocks_per_sm, workspace, workspace_bytes, stream, true);
}

// ------------------------------------------ backward without caller memory
// Some callers cannot allocate device memory: a host program whose own pool
// owns the whole device, or a loop that may not allocate once it is running.
// ngt_raymarch_bwd_static serves them with the backward's scratch (sign flag,
// cameras, quad layout and quad gradient) in one file-scope device array of
// kStaticScratchBytes, which every GPU that loads the library holds until the
// process exits.  Every call shares the array and finds the previous call's
// contents in it; what must start at zero (the sign flag, the quad gradient,
// the reference-mode buffers) is cleared inside each call by ngt_raymarch_bwd's
// own stream-ordered memsets.  Calls whose work overlaps on the GPU (other
// streams, other host threads) race on the array.  In host code the array's
// name is only a stand-in: its device address in the calling thread's current
// context is looked up with cudaGetSymbolAddress by every call made outside a
// stream capture (so a device reset or another context of the same device
// gets its own address); a call made while its stream is being captured uses
// the address the last uncaptured call on that device found, so the first
// call on a device (and the first after a device reset) comes before any
// capture.
constexpr size_t kStaticScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_raymarch_scratch[kStaticScratchBytes];

namespace ngt {
namespace {

constexpr int kMaxDevices = 64;

std::mutex g_scratch_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// The array's device address on the current device: looked up afresh outside
// stream capture, the last looked-up address during a capture of ``st``.
int scratch_address(cudaStream_t st, void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("raymarch_bwd_static: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(NGT_ERR_UNSUPPORTED, "raymarch_bwd_static: device %d", dev);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return check_launch("raymarch_bwd_static: cudaStreamIsCapturing");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_raymarch_scratch);
    if (e != cudaSuccess)
      return fail(NGT_ERR_CUDA, "raymarch_bwd_static: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  } else if (!g_scratch_ptr[dev]) {
    return fail(NGT_ERR_UNSUPPORTED,
                "raymarch_bwd_static: the first call on device %d must come before any stream capture", dev);
  }
  *out = g_scratch_ptr[dev];
  return NGT_OK;
}

}  // namespace
}  // namespace ngt

extern "C" int ngt_raymarch_bwd_static(const ngt_raymarch_grad_args* a, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd_static: null arguments");
  int cin, cb;
  // the same argument checks as ngt_raymarch_bwd before the scratch size is formed from the shapes
  int rc = validate(&a->fwd, cin, cb);
  if (rc) return rc;
  if (a->grad_mode != NGT_GRAD_EXACT && a->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd: invalid grad_mode");
  const size_t need = bwd_layout(a).total;
  if (need > kStaticScratchBytes)
    return fail(NGT_ERR_WORKSPACE, "raymarch_bwd_static: this call needs %zu scratch bytes, above the %zu-byte static scratch",
                need, kStaticScratchBytes);
  void* scratch = nullptr;
  rc = scratch_address(as_stream(stream), &scratch);
  if (rc) return rc;
  ngt_raymarch_grad_args b = *a;
  b.workspace = scratch;
  b.workspace_bytes = kStaticScratchBytes;
  return ngt_raymarch_bwd(&b, stream);
}
