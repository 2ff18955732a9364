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
#include "ngt_common.cuh"
#include "ngt_host.cuh"
#include "ngt_blend.cuh"
#include "ngt_quad.cuh"

#include <algorithm>
#include <mutex>

namespace ngt {
namespace {

constexpr int kTileX = 16, kTileY = 8, kThreads = kTileX * kTileY;
constexpr int kSeg = 16;       // exact backward: steps recomputed per segment buffer
constexpr int kMaxCkpt = 64;   // exact backward: checkpoints per ray
constexpr int kMaxSteps = 1 << 20;
constexpr int kMinBlocks = 10;  // forward and one-pass backward: 48 registers, 40 warps per SM

struct RayParams {
  const void* input;
  void* output;
  const void* out_fwd;   // backward: forward output
  const void* out_grad;  // backward: output gradient
  void* in_grad;         // backward: input gradient (compute type)
  void* wbuf;            // reference backward: weighted gradient buffer
  void* wsum;            // reference backward: per-voxel weight sums
  const float *M, *V, *P, *F;
  Dims din;
  int D, H, W;           // depth samples, image height, width
  int N, ncam, sep;
  int fm, bm, blend;
  float scale[4];
  int slot0;             // first (batch, camera) slot of this launch
  const int* flag;       // exact Beer-Lambert backward: nonzero if an extinction sample can be negative
  const Cam* cams;       // per-slot cameras formed by k_build_cams, or null (each block forms its own)
  const void* quad;      // quad layout of the input (one channel, LINEAR) or null
  float4* gquad;         // quad gradient accumulator (exact backward) or null
  QuadDims qd;
  // forward with the image L2 loss fused: per-pixel target (l2_lc channels),
  // image gradient (CB channels) and the loss accumulator, or null
  const void* l2_target;
  void* l2_grad;
  void* l2_loss;
  int l2_lc;
  // with the fused loss: per-camera background images (cameras, H, W, CB - 1)
  // composited behind the light channels before the loss, or null
  const void* l2_bkg;
};

// One-channel float / 16-bit grids sampled LINEAR go through the quad layout.
template <int CIN, class T>
constexpr bool quad_able() {
  return CIN == 1 && !std::is_same<T, double>::value;
}

template <int CIN, class T>
__device__ __forceinline__ const void* quad_of(const RayParams& p, int b) {
  if constexpr (quad_able<CIN, T>())
    return p.quad ? static_cast<const void*>(static_cast<const typename QuadOf<T>::type*>(p.quad) + int64_t(b) * p.qd.count)
                  : nullptr;
  return nullptr;
}

__device__ __forceinline__ float4* gquad_of(const RayParams& p, int b) {
  return p.gquad ? p.gquad + int64_t(b) * p.qd.count : nullptr;
}

__device__ __forceinline__ void slot_to_bc(const RayParams& p, int slot, int& b, int& c, int& oslot) {
  if (p.sep) {
    b = slot / p.ncam;
    c = slot % p.ncam;
  } else {
    b = slot;
    c = slot;
  }
  oslot = slot;
}

__host__ __device__ __forceinline__ int num_slots_dev(const RayParams& p) { return p.sep ? p.N * p.ncam : p.N; }

// This thread's pixel within its 16x8 tile: each warp covers 8x4 pixels (rays
// that stay close in the grid, so a warp's gathers share cache lines); warps 0
// and 1 side by side in x, warps 2 and 3 below them.
__device__ __forceinline__ void pixel_of_thread(int& px, int& py) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  px = (warp & 1) * 8 + (lane & 7);
  py = (warp >> 1) * 4 + (lane >> 3);
}

struct Ray {
  float s[3], st[3], e[3];
  int steps;
  bool hit;
};

// getRaymarchStep / RayGridIntersectionDistances (raymarch_grid.cu.cc:109-200)
__device__ inline Ray ray_setup(const Cam& cam, int px, int py, const RayParams& p) {
  Ray r;
  const float dinv[3] = {1.0f / float(p.W), 1.0f / float(p.H), 1.0f / float(p.D)};
  const float zmax = float(max(p.D - 1, 1));
  idx_to_os(cam, px + 0.5f, py + 0.5f, 0.5f, dinv, false, r.s);
  idx_to_os(cam, px + 0.5f, py + 0.5f, zmax + 0.5f, dinv, false, r.e);
#pragma unroll
  for (int a = 0; a < 3; ++a) r.st[a] = (r.e[a] - r.s[a]) / zmax;
  r.steps = p.D;
  r.hit = true;
  if (p.bm == BORDER) {
    float v[3] = {r.e[0] - r.s[0], r.e[1] - r.s[1], r.e[2] - r.s[2]};
    const float il = rsqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const float dir[3] = {v[0] * il, v[1] * il, v[2] * il};
    const float bmax[3] = {float(p.din.x), float(p.din.y), float(p.din.z)};
    float tmin = -INFINITY, tmax = INFINITY;
    float tsm[3], tbg[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float half = bmax[a] * 0.5f + (-0.5f);
      const float co = r.s[a] - bmax[a] * 0.5f;
      const float inv = 1.0f / dir[a];
      const float n = inv * co;
      const float k = fabsf(inv) * half;
      tsm[a] = 0.0f - n - k;
      tbg[a] = k - n;
    }
    tmin = fmaxf(fmaxf(tsm[0], tsm[1]), tsm[2]);
    tmax = fminf(fminf(tbg[0], tbg[1]), tbg[2]);
    if (tmin > tmax || tmax < 0.0f) {
      r.hit = false;
      r.steps = 0;
      return r;
    }
    float e2[3], s2[3];
    const float t0 = fmaxf(tmin - 1.0f, 0.0f);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      e2[a] = r.s[a] + dir[a] * (tmax + 1.0f);
      s2[a] = r.s[a] + dir[a] * t0;
    }
    const float ss = sqrtf(r.st[0] * r.st[0] + r.st[1] * r.st[1] + r.st[2] * r.st[2]);
    const float d0 = s2[0] - e2[0], d1 = s2[1] - e2[1], d2 = s2[2] - e2[2];
    const float rl = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
    const float q = rl / ss;
    r.steps = (q < float(kMaxSteps)) ? int(q) + 2 : kMaxSteps;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      r.s[a] = s2[a];
      r.e[a] = e2[a];
    }
  }
  return r;
}

// Sample CIN channels at object-space position pos and expand to CB blend channels.
template <int CIN, int CB, class T, class S>
__device__ __forceinline__ void sample_cell(const T* __restrict__ g, const void* qg, const float pos[3],
                                            const RayParams& p, S cell[CB]) {
  const S px = S(pos[0] - 0.5f), py = S(pos[1] - 0.5f), pz = S(pos[2] - 0.5f);
  S v[CIN];
  if constexpr (quad_able<CIN, T>()) {
    if (qg) {
      v[0] = read_linear_quad<T>(static_cast<const typename QuadOf<T>::type*>(qg), px, py, pz, p.din, p.qd, p.bm);
#pragma unroll
      for (int c = 0; c < CB; ++c) cell[c] = (CIN == CB) ? v[0] : S(p.scale[c]) * v[0];
      return;
    }
  }
  if (p.fm == LINEAR) {
    read_linear<CIN>(g, px, py, pz, p.din, p.bm, v);
  } else if (p.fm == NEAREST) {
    read_nearest<CIN>(g, px, py, pz, p.din, p.bm, v);
  } else {
    int arg[CIN];
    int64_t ci[8];
    read_extremum<CIN>(g, px, py, pz, p.din, p.bm, p.fm == FMAX, v, arg, ci);
  }
  if (CIN == CB) {
#pragma unroll
    for (int c = 0; c < CB; ++c) cell[c] = v[c < CIN ? c : 0];
  } else {
#pragma unroll
    for (int c = 0; c < CB; ++c) cell[c] = S(p.scale[c]) * v[0];
  }
}

template <int CIN, int CB, class S>
__device__ __forceinline__ void scatter_cell(const RayParams& p, S* __restrict__ grad, float4* gq, const float pos[3],
                                             const S dcell[CB]) {
  const S px = S(pos[0] - 0.5f), py = S(pos[1] - 0.5f), pz = S(pos[2] - 0.5f);
  if constexpr (CIN == 1 && std::is_same<S, float>::value) {
    if (gq) {
      S g = S(0);
#pragma unroll
      for (int c = 0; c < CB; ++c) g += (CIN == CB) ? dcell[c] : S(p.scale[c]) * dcell[c];
      scatter_linear_quad(gq, px, py, pz, p.din, p.qd, p.bm, g);
      return;
    }
  }
  if (CIN == CB) {
    S g[CIN];
#pragma unroll
    for (int c = 0; c < CIN; ++c) g[c] = dcell[c < CB ? c : 0];
    scatter_linear<CIN>(grad, px, py, pz, p.din, p.bm, g);
  } else {
    S g[1] = {S(0)};
#pragma unroll
    for (int c = 0; c < CB; ++c) g[0] += S(p.scale[c]) * dcell[c];
    scatter_linear<1>(grad, px, py, pz, p.din, p.bm, g);
  }
}

// The block's camera, formed by warp 0; the caller synchronises the block.
__device__ __forceinline__ void load_cam(const RayParams& p, int slot, int b, int c, Cam& cam, CamScratch& sh) {
  if (p.cams) {
    const float* src = reinterpret_cast<const float*>(p.cams + slot);
    float* dst = reinterpret_cast<float*>(&cam);
    for (int i = threadIdx.x; i < int(sizeof(Cam) / sizeof(float)); i += blockDim.x) dst[i] = __ldg(src + i);
  } else if (threadIdx.x < 32) {
    build_cam_warp(p.M + 16 * b, p.V + 16 * c, p.P + 16 * c, p.F + 6 * c, cam, sh);
  }
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

// ----------------------------------------------------------------- forward
// This thread's pixel of tile ``tile`` of a W x H image; false outside the image.
__device__ __forceinline__ bool tile_pixel(const RayParams& p, int tile, int& px, int& py) {
  const int tiles_x = (p.W + kTileX - 1) / kTileX;
  pixel_of_thread(px, py);
  px += (tile % tiles_x) * kTileX;
  py += (tile / tiles_x) * kTileY;
  return px < p.W && py < p.H;
}

// Fused image L2 loss of one pixel: the gradient g_c = out_c - target_c on the
// first l2_lc channels (0 on the others) is written, sum g_c^2 returned.  With a
// background (renderer.py:779, 804-806) the light channels are first composited,
// out_c + background_c * t with t = exp(-d) the ray's transmittance, and the
// optical-depth channel receives -t * sum_c background_c * g_c.  ``pix`` is the
// pixel's index in the output (slot, y, x); its camera's background pixel is
// formed from it here, after the march, so the loop carries no extra index.
template <int CB, class S>
__device__ __forceinline__ S l2_pixel(const RayParams& p, int64_t pix, const S out[CB]) {
  const S* tg = static_cast<const S*>(p.l2_target) + pix * p.l2_lc;
  S* gr = static_cast<S*>(p.l2_grad) + pix * CB;
  S l = S(0);
  if constexpr (CB > 1) {
    if (p.l2_bkg) {
      const int64_t hw = int64_t(p.H) * p.W;
      const int64_t bq = p.sep ? (pix / hw) % p.ncam * hw + pix % hw : pix;
      const S* bk = static_cast<const S*>(p.l2_bkg) + bq * (CB - 1);
      const S t = ex(-out[CB - 1]);
      S sb = S(0);
#pragma unroll
      for (int k = 0; k < CB - 1; ++k) {
        const S g = k < p.l2_lc ? out[k] + bk[k] * t - tg[k] : S(0);
        gr[k] = g;
        l += g * g;
        sb += bk[k] * g;
      }
      gr[CB - 1] = -t * sb;
      return l;
    }
  }
#pragma unroll
  for (int k = 0; k < CB; ++k) {
    const S g = k < p.l2_lc ? out[k] - tg[k] : S(0);
    gr[k] = g;
    l += g * g;
  }
  return l;
}

// Adds 0.5 * the block's sum of ``v`` to *loss (one atomic per block); every
// thread of the block calls it.
template <class S>
__device__ __forceinline__ void l2_block_add(S v, S* loss) {
  __shared__ S part[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    S w = threadIdx.x < kThreads / 32 ? part[threadIdx.x] : S(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (threadIdx.x == 0) atomicAdd(loss, S(0.5) * w);
  }
}

// The forward of one 16x8 tile of rays of (batch b, output slot oslot).  With
// the fused loss it returns the pixel's sum of squared image differences (0
// outside the image), else 0.
template <int CIN, int CB, class T, class S>
__device__ __forceinline__ S fwd_tile(const RayParams& p, const Cam& cam, int b, int oslot, int tile) {
  int px, py;
  if (!tile_pixel(p, tile, px, py)) return S(0);
  const int64_t pix = (int64_t(oslot) * p.H + py) * p.W + px;
  const T* g = reinterpret_cast<const T*>(p.input) + int64_t(b) * p.din.count() * CIN;
  const void* qg = quad_of<CIN, T>(p, b);
  const Ray r = ray_setup(cam, px, py, p);
  S acc[CB];
#pragma unroll
  for (int k = 0; k < CB; ++k) acc[k] = S(0);
  if constexpr (quad_able<CIN, T>() && CB > 1) {
    // emission Beer-Lambert through the quad layout: the step's hot loop
    if (qg && p.blend == BEER_LAMBERT && r.hit) {
      const auto* q = static_cast<const typename QuadOf<T>::type*>(qg);
      float sc[CB];
#pragma unroll
      for (int k = 0; k < CB; ++k) sc[k] = p.scale[k];
      float pos[3] = {r.s[0], r.s[1], r.s[2]};
      float dd = 0.0f, L[CB - 1];
#pragma unroll
      for (int k = 0; k < CB - 1; ++k) L[k] = 0.0f;
      for (int i = 0; i < r.steps; ++i) {
        QuadPos qp;
        float v;
        quad_sample_fma<T>(q, pos[0] - 0.5f, pos[1] - 0.5f, pos[2] - 0.5f, p.din, p.qd, p.bm, qp, v);
        dd = fmaxf(dd + sc[CB - 1] * v, 0.0f);
        const float t = __expf(-dd);
#pragma unroll
        for (int k = 0; k < CB - 1; ++k) L[k] += t * (sc[k] * v);
#pragma unroll
        for (int a = 0; a < 3; ++a) pos[a] += r.st[a];
      }
      S res[CB];
#pragma unroll
      for (int k = 0; k < CB - 1; ++k) res[k] = L[k];
      res[CB - 1] = dd;
      S* out = reinterpret_cast<S*>(p.output) + pix * CB;
#pragma unroll
      for (int k = 0; k < CB; ++k) out[k] = res[k];
      return p.l2_target ? l2_pixel<CB, S>(p, pix, res) : S(0);
    }
  }
  if (r.hit) {
    float pos[3] = {r.s[0], r.s[1], r.s[2]};
    for (int i = 0; i < r.steps; ++i) {
      S cell[CB];
      sample_cell<CIN, CB>(g, qg, pos, p, cell);
      blend_step<CB>(acc, cell, p.blend);
#pragma unroll
      for (int a = 0; a < 3; ++a) pos[a] += r.st[a];
    }
  }
  S* out = reinterpret_cast<S*>(p.output) + pix * CB;
#pragma unroll
  for (int k = 0; k < CB; ++k) out[k] = acc[k];
  return p.l2_target ? l2_pixel<CB, S>(p, pix, acc) : S(0);
}

template <int CIN, int CB, class T, class S>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_raymarch_fwd(RayParams p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot;
  slot_to_bc(p, p.slot0 + blockIdx.y, b, c, oslot);
  load_cam(p, p.slot0 + blockIdx.y, b, c, cam, cam_sh);
  __syncthreads();
  const S l = fwd_tile<CIN, CB, T, S>(p, cam, b, oslot, blockIdx.x);
  if (p.l2_loss) l2_block_add<S>(l, static_cast<S*>(p.l2_loss));
}

// ------------------------------------------------------- exact backward
// Accumulator states are recomputed forward (checkpoints every K steps, then
// each segment re-marched into a small buffer and walked back), so the adjoint
// uses the forward's own positions and densities, not a subtraction.
template <int CIN, int CB, class T, class S>
__device__ __forceinline__ void bwd_exact_tile(const RayParams& p, const Cam& cam, int b, int oslot, int tile) {
  int px, py;
  if (!tile_pixel(p, tile, px, py)) return;
  const T* g = reinterpret_cast<const T*>(p.input) + int64_t(b) * p.din.count() * CIN;
  const void* qg = quad_of<CIN, T>(p, b);
  S* grad = reinterpret_cast<S*>(p.in_grad) + int64_t(b) * p.din.count() * CIN;
  float4* gq = gquad_of(p, b);
  const Ray r = ray_setup(cam, px, py, p);
  if (!r.hit || r.steps <= 0) return;
  S G[CB];
  const S* og = reinterpret_cast<const S*>(p.out_grad) + ((int64_t(oslot) * p.H + py) * p.W + px) * CB;
#pragma unroll
  for (int k = 0; k < CB; ++k) G[k] = og[k];

  if (!stateful<CB>(p.blend)) {
    // stateless blends: the adjoint of each step needs only the cell itself
    float pos[3] = {r.s[0], r.s[1], r.s[2]};
    for (int i = 0; i < r.steps; ++i) {
      S cell[CB], dcell[CB];
      sample_cell<CIN, CB>(g, qg, pos, p, cell);
      blend_adjoint<CB>(G, cell, S(0), p.blend, dcell);
      scatter_cell<CIN, CB>(p, grad, gq, pos, dcell);
#pragma unroll
      for (int a = 0; a < 3; ++a) pos[a] += r.st[a];
    }
    return;
  }

  // segment length K (multiple of kSeg) so that at most kMaxCkpt checkpoints are needed
  const int nseg_min = (r.steps + kMaxCkpt - 1) / kMaxCkpt;
  const int K = ((max(nseg_min, kSeg) + kSeg - 1) / kSeg) * kSeg;
  const int nck = (r.steps + K - 1) / K;
  float ck_pos[kMaxCkpt][3];
  S ck_a[kMaxCkpt];
  {
    float pos[3] = {r.s[0], r.s[1], r.s[2]};
    S a = S(0);
    for (int i = 0; i < r.steps; ++i) {
      if (i % K == 0) {
        const int k = i / K;
        ck_pos[k][0] = pos[0];
        ck_pos[k][1] = pos[1];
        ck_pos[k][2] = pos[2];
        ck_a[k] = a;
      }
      S cell[CB];
      sample_cell<CIN, CB>(g, qg, pos, p, cell);
      a = state_update(a, cell[CB - 1], p.blend);
#pragma unroll
      for (int q = 0; q < 3; ++q) pos[q] += r.st[q];
    }
  }
  float buf_pos[kSeg][3];
  S buf_cell[kSeg][CB];
  S buf_a[kSeg];
  for (int seg = nck - 1; seg >= 0; --seg) {
    const int i0 = seg * K, i1 = min(i0 + K, r.steps);
    const int nsub = (i1 - i0 + kSeg - 1) / kSeg;
    for (int sub = nsub - 1; sub >= 0; --sub) {
      const int j0 = i0 + sub * kSeg, j1 = min(j0 + kSeg, i1);
      float pos[3] = {ck_pos[seg][0], ck_pos[seg][1], ck_pos[seg][2]};
      S a = ck_a[seg];
      for (int i = i0; i < j0; ++i) {  // re-march to the sub-segment start (only when K > kSeg)
        S cell[CB];
        sample_cell<CIN, CB>(g, qg, pos, p, cell);
        a = state_update(a, cell[CB - 1], p.blend);
#pragma unroll
        for (int q = 0; q < 3; ++q) pos[q] += r.st[q];
      }
      for (int i = j0; i < j1; ++i) {
        const int j = i - j0;
        buf_pos[j][0] = pos[0];
        buf_pos[j][1] = pos[1];
        buf_pos[j][2] = pos[2];
        buf_a[j] = a;
        sample_cell<CIN, CB>(g, qg, pos, p, buf_cell[j]);
        a = state_update(a, buf_cell[j][CB - 1], p.blend);
#pragma unroll
        for (int q = 0; q < 3; ++q) pos[q] += r.st[q];
      }
      for (int j = j1 - j0 - 1; j >= 0; --j) {
        S dcell[CB];
        blend_adjoint<CB>(G, buf_cell[j], buf_a[j], p.blend, dcell);
        scatter_cell<CIN, CB>(p, grad, gq, buf_pos[j], dcell);
      }
    }
  }
}

template <int CIN, int CB, class T, class S>
__global__ void __launch_bounds__(kThreads) k_raymarch_bwd_exact(RayParams p) {
  if (p.flag && *p.flag == 0) return;  // Beer-Lambert with non-negative extinction: k_raymarch_bwd_bl
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot;
  slot_to_bc(p, p.slot0 + blockIdx.y, b, c, oslot);
  load_cam(p, p.slot0 + blockIdx.y, b, c, cam, cam_sh);
  __syncthreads();
  bwd_exact_tile<CIN, CB, T, S>(p, cam, b, oslot, blockIdx.x);
}

// ------------------------------------ exact Beer-Lambert backward, one pass
// With every extinction sample sigma_k >= 0 the density never reaches the
// max(d + sigma, 0) clamp, and the adjoint of the front-to-back blend
//   d_k = d_{k-1} + sigma_k,  t_k = exp(-d_k),  L_c += t_k * l_kc
// is, in forward order,
//   dl_kc     = t_k * gL_c
//   dsigma_k  = gD - sum_{j>=k} t_j (l_j . gL) = gD - (L . gL - W_{k-1}),
// W_{k-1} = sum_{j<k} t_j (l_j . gL) accumulated on the way and L the forward
// output.  One march replaces the checkpointed recomputation; the sign of the
// extinction channel is checked over the whole grid first (k_extinction_sign),
// and a launch that can see a negative sample runs k_raymarch_bwd_exact.
template <int CIN, int CB, class T, class S>
__device__ __forceinline__ void bwd_bl_tile(const RayParams& p, const Cam& cam, int b, int oslot, int tile) {
  int px, py;
  if (!tile_pixel(p, tile, px, py)) return;
  const T* g = reinterpret_cast<const T*>(p.input) + int64_t(b) * p.din.count() * CIN;
  const void* qg = quad_of<CIN, T>(p, b);
  S* grad = reinterpret_cast<S*>(p.in_grad) + int64_t(b) * p.din.count() * CIN;
  float4* gq = gquad_of(p, b);
  const Ray r = ray_setup(cam, px, py, p);
  if (!r.hit || r.steps <= 0) return;
  const int64_t o = ((int64_t(oslot) * p.H + py) * p.W + px) * CB;
  S G[CB];
  S lgf = S(0);
#pragma unroll
  for (int k = 0; k < CB; ++k) G[k] = reinterpret_cast<const S*>(p.out_grad)[o + k];
#pragma unroll
  for (int k = 0; k < CB - 1; ++k) lgf += G[k] * reinterpret_cast<const S*>(p.out_fwd)[o + k];
  const S gD = G[CB - 1];
  if constexpr (quad_able<CIN, T>() && std::is_same<S, float>::value) {
    if (qg && gq) {
      // one-channel emission through the quad layout: one set-up per sample for
      // the gather and the two vector atomics of its adjoint
      const auto* q = static_cast<const typename QuadOf<T>::type*>(qg);
      float sg = 0.0f;  // sum_c scale_c * gL_c
#pragma unroll
      for (int k = 0; k < CB - 1; ++k) sg += p.scale[k] * G[k];
      const float sl = p.scale[CB - 1];
      float dd = 0.0f, w = 0.0f;
      float pos[3] = {r.s[0], r.s[1], r.s[2]};
      for (int i = 0; i < r.steps; ++i) {
        QuadPos qp;
        float v;
        const bool in = quad_sample_fma<T>(q, pos[0] - 0.5f, pos[1] - 0.5f, pos[2] - 0.5f, p.din, p.qd, p.bm, qp, v);
        dd = dd + sl * v;
        const float t = __expf(-dd);
        // d rho = sum_c scale_c * t * gL_c + scale_sigma * (gD - (L.gL - W))
        const float gs = t * sg + sl * (float(gD) - (float(lgf) - w));
        w += t * (v * sg);
        if (in) scatter_quad_at(gq, qp, p.qd, gs);
#pragma unroll
        for (int a = 0; a < 3; ++a) pos[a] += r.st[a];
      }
      return;
    }
  }
  S d = S(0), w = S(0);
  float pos[3] = {r.s[0], r.s[1], r.s[2]};
  for (int i = 0; i < r.steps; ++i) {
    S cell[CB], dcell[CB];
    sample_cell<CIN, CB>(g, qg, pos, p, cell);
    d = d + cell[CB - 1];
    const S t = ex(-d);
    S lg = S(0);
#pragma unroll
    for (int k = 0; k < CB - 1; ++k) {
      lg += cell[k] * G[k];
      dcell[k] = t * G[k];
    }
    dcell[CB - 1] = gD - (lgf - w);
    w += t * lg;
    scatter_cell<CIN, CB>(p, grad, gq, pos, dcell);
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] += r.st[a];
  }
}

// The checkpointed adjoint as a call of its own (its registers and stack do not
// weigh on the one-pass kernel that calls it for launches with a possibly
// negative extinction sample).
template <int CIN, int CB, class T, class S>
__device__ __noinline__ void bwd_exact_tile_call(const RayParams& p, const Cam& cam, int b, int oslot, int tile) {
  bwd_exact_tile<CIN, CB, T, S>(p, cam, b, oslot, tile);
}

template <int CIN, int CB, class T, class S>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_raymarch_bwd_bl(const __grid_constant__ RayParams p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot;
  slot_to_bc(p, p.slot0 + blockIdx.y, b, c, oslot);
  load_cam(p, p.slot0 + blockIdx.y, b, c, cam, cam_sh);
  __syncthreads();
  if (*p.flag != 0)
    bwd_exact_tile_call<CIN, CB, T, S>(p, cam, b, oslot, blockIdx.x);
  else
    bwd_bl_tile<CIN, CB, T, S>(p, cam, b, oslot, blockIdx.x);
}

// Sets *flag when some voxel makes a negative extinction sample possible: a
// negative extinction channel (CIN == CB), or a one-channel density whose sign
// is opposite to the extinction scale.  Linear interpolation of non-negative
// values (border cells read as 0) is non-negative.
template <int CIN, int CB, class T>
__global__ void k_extinction_sign(const T* __restrict__ g, int64_t nvox, float sscale, int* flag) {
  int neg = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nvox; i += int64_t(gridDim.x) * blockDim.x) {
    const float v = float(ld(g + i * CIN + (CIN - 1)));
    neg |= (CIN == CB) ? (v < 0.0f) : (sscale * v < 0.0f);
  }
  if (__syncthreads_or(neg) && threadIdx.x == 0) atomicOr(flag, 1);
}

// --------------------------------------------------- reference backward
// scatterGrad3DInterpolated with per-voxel weight sums (sampling_v2.hpp:438-559)
template <int C, class S>
__device__ __forceinline__ void scatter_weighted(S* __restrict__ buf, S* __restrict__ wsum, S px, S py, S pz,
                                                 const Dims& d, int bm, const S g[C]) {
  if (bm == BORDER && !(px > S(-1) && px < S(d.x) && py > S(-1) && py < S(d.y) && pz > S(-1) && pz < S(d.z))) return;
  Tri<S> t;
  const S pp[3] = {px, py, pz};
  const int n[3] = {d.x, d.y, d.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const S f = floor(pp[a]);
    t.w[a] = pp[a] - f;
    int i0 = to_int_rz(f), i1 = to_int_rz(ceil(pp[a]));
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
    for (int c = 0; c < C; ++c) atomic_add(buf + i * C + c, g[c] * w);
    atomic_add(wsum + i, w);
  }
}

template <int CIN, int CB, class T, class S>
__global__ void __launch_bounds__(kThreads) k_raymarch_bwd_reference(RayParams p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot;
  slot_to_bc(p, p.slot0 + blockIdx.y, b, c, oslot);
  load_cam(p, p.slot0 + blockIdx.y, b, c, cam, cam_sh);
  __syncthreads();
  const int tiles_x = (p.W + kTileX - 1) / kTileX;
  int px, py;
  pixel_of_thread(px, py);
  px += (blockIdx.x % tiles_x) * kTileX;
  py += (blockIdx.x / tiles_x) * kTileY;
  if (px >= p.W || py >= p.H) return;
  const T* g = reinterpret_cast<const T*>(p.input) + int64_t(b) * p.din.count() * CIN;
  const void* qg = quad_of<CIN, T>(p, b);
  S* buf = reinterpret_cast<S*>(p.wbuf);
  S* wsum = reinterpret_cast<S*>(p.wsum);
  const Ray r = ray_setup(cam, px, py, p);
  if (!r.hit) return;
  const int64_t o = ((int64_t(oslot) * p.H + py) * p.W + px) * CB;
  S G[CB], acc[CB];
#pragma unroll
  for (int k = 0; k < CB; ++k) {
    G[k] = reinterpret_cast<const S*>(p.out_grad)[o + k];
    acc[k] = reinterpret_cast<const S*>(p.out_fwd)[o + k];
  }
  float pos[3] = {r.e[0], r.e[1], r.e[2]};
  for (int i = r.steps - 1; i >= 0; --i) {
    S cell[CB], dcell[CB];
    sample_cell<CIN, CB>(g, qg, pos, p, cell);
    blend_grad_reference<CB>(G, cell, acc, p.blend, dcell);
    const S qx = S(pos[0] - 0.5f), qy = S(pos[1] - 0.5f), qz = S(pos[2] - 0.5f);
    if (CIN == CB) {
      S gg[CIN];
#pragma unroll
      for (int k = 0; k < CIN; ++k) gg[k] = dcell[k < CB ? k : 0];
      scatter_weighted<CIN>(buf, wsum, qx, qy, qz, p.din, p.bm, gg);
    } else {
      S gg[1] = {S(0)};
#pragma unroll
      for (int k = 0; k < CB; ++k) gg[0] += S(p.scale[k]) * dcell[k];
      scatter_weighted<1>(buf, wsum, qx, qy, qz, p.din, p.bm, gg);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] -= r.st[a];
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
      (rc = check_aligned("raymarch", kScratchAlign, {{"cameras", a->cameras}, {"workspace", a->workspace}})) ||
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
  return p;
}

int num_slots(const RayParams& p) { return p.sep ? p.N * p.ncam : p.N; }

template <template <int, int, class, class> class K, class T, class S>
int dispatch_channels(int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p);

enum Which { FWD = 0, BWD_EXACT = 1, BWD_REF = 2, BWD_BL = 3, SIGN = 4 };

template <int CIN, int CB, class T, class S>
void launch(int which, dim3 grid, cudaStream_t st, const RayParams& p) {
  if (which == FWD) {
    k_raymarch_fwd<CIN, CB, T, S><<<grid, kThreads, 0, st>>>(p);
  } else if (which == BWD_EXACT) {
    k_raymarch_bwd_exact<CIN, CB, T, S><<<grid, kThreads, 0, st>>>(p);
  } else if (which == BWD_BL) {
    if (CB > 1) k_raymarch_bwd_bl<CIN, CB, T, S><<<grid, kThreads, 0, st>>>(p);
  } else if (which == SIGN) {
    const int64_t nvox = int64_t(p.N) * p.din.count();
    const int64_t nb = (nvox + 255) / 256;
    const unsigned blocks = unsigned(nb < 152 * 8 ? nb : 152 * 8);
    k_extinction_sign<CIN, CB, T><<<blocks, 256, 0, st>>>(static_cast<const T*>(p.input), nvox,
                                                         p.scale[CB - 1], const_cast<int*>(p.flag));
  } else {
    k_raymarch_bwd_reference<CIN, CB, T, S><<<grid, kThreads, 0, st>>>(p);
  }
}

template <class T, class S>
int launch_typed(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p) {
  if (cin == 1 && cb == 1) launch<1, 1, T, S>(which, grid, st, p);
  else if (cin == 2 && cb == 2) launch<2, 2, T, S>(which, grid, st, p);
  else if (cin == 4 && cb == 4) launch<4, 4, T, S>(which, grid, st, p);
  else if (cin == 1 && cb == 2) launch<1, 2, T, S>(which, grid, st, p);
  else if (cin == 1 && cb == 4) launch<1, 4, T, S>(which, grid, st, p);
  else return fail(NGT_ERR_UNSUPPORTED, "raymarch: unsupported channel combination");
  return NGT_OK;
}

int launch_dtype(int dtype, int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p) {
  switch (dtype) {
    case NGT_F32: return launch_typed<float, float>(which, cin, cb, grid, st, p);
    case NGT_F64: return launch_typed<double, double>(which, cin, cb, grid, st, p);
    case NGT_BF16: return launch_typed<__nv_bfloat16, float>(which, cin, cb, grid, st, p);
    case NGT_F16: return launch_typed<__half, float>(which, cin, cb, grid, st, p);
  }
  return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch: invalid dtype");
}

// ------------------------------------------------------ batched, persistent
// Many scenes of different grid, image and depth sizes in one launch: every
// (scene, camera, 16x8 tile) is one work item, taken by persistent blocks from
// a global counter; each block copies its item's camera from the per-scene
// camera block and runs the same tile code as the single-scene kernels.
constexpr int kMaxBatch = 32;

struct RayBatch {
  RayParams item[kMaxBatch];
  int tile_end[kMaxBatch];        // cumulative work items over the scenes
  int tiles_per_slot[kMaxBatch];  // tiles per (batch, camera) slot of each scene
  int count, total;
  int* counter;                   // work counter, zero at launch
  int* flags;                     // backward: per-scene extinction-sign flags
  // 32x8 blocks of the quad layouts and of the cell grids, back to back
  int qblock_end[kMaxBatch], qnbx[kMaxBatch], qnby[kMaxBatch];
  int cblock_end[kMaxBatch], cnbx[kMaxBatch], cnby[kMaxBatch];
};

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

template <int CIN, int CB, class T, class S, int WHICH>
__global__ void __launch_bounds__(kThreads, CIN == 1 ? 8 : 4) k_raymarch_batch(const __grid_constant__ RayBatch bp) {
  __shared__ Cam cam;
  __shared__ int s_work;
  for (;;) {
    __syncthreads();  // the previous item's readers of cam and s_work are done
    if (threadIdx.x == 0) s_work = atomicAdd(bp.counter, 1);
    __syncthreads();
    const int w = s_work;
    if (w >= bp.total) return;
    int it = 0;
    while (it < bp.count - 1 && bp.tile_end[it] <= w) ++it;
    const RayParams& p = bp.item[it];
    const int local = w - (it ? bp.tile_end[it - 1] : 0);
    const int slot = local / bp.tiles_per_slot[it], tile = local - slot * bp.tiles_per_slot[it];
    // the one-pass backward takes scenes with non-negative extinction, the
    // checkpointed one the others
    const bool checkpointed = WHICH != FWD && bp.flags[it] != 0;
    int b, c, oslot;
    slot_to_bc(p, slot, b, c, oslot);
    const float* src = reinterpret_cast<const float*>(p.cams + slot);
    float* dst = reinterpret_cast<float*>(&cam);
    for (int i = threadIdx.x; i < int(sizeof(Cam) / sizeof(float)); i += blockDim.x) dst[i] = __ldg(src + i);
    __syncthreads();
    if (WHICH == FWD)
      fwd_tile<CIN, CB, T, S>(p, cam, b, oslot, tile);
    else if (checkpointed || CB == 1)
      bwd_exact_tile_call<CIN, CB, T, S>(p, cam, b, oslot, tile);
    else
      bwd_bl_tile<CIN, CB, T, S>(p, cam, b, oslot, tile);
  }
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

// Extinction-sign check of every scene (blockIdx.y = scene) into bp.flags.
template <int CIN, int CB, class T>
__global__ void k_extinction_sign_batch(const __grid_constant__ RayBatch bp) {
  const RayParams& p = bp.item[blockIdx.y];
  const int64_t nvox = int64_t(p.N) * p.din.count();
  const T* g = static_cast<const T*>(p.input);
  int neg = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nvox; i += int64_t(gridDim.x) * blockDim.x) {
    const float v = float(ld(g + i * CIN + (CIN - 1)));
    neg |= (CIN == CB) ? (v < 0.0f) : (p.scale[CB - 1] * v < 0.0f);
  }
  if (__syncthreads_or(neg) && threadIdx.x == 0) atomicOr(bp.flags + blockIdx.y, 1);
}

template <int CIN, int CB, class T, class S>
void launch_batch(int which, unsigned blocks, cudaStream_t st, const RayBatch& bp) {
  if (which == FWD) {
    k_raymarch_batch<CIN, CB, T, S, FWD><<<blocks, kThreads, 0, st>>>(bp);
  } else if (which == BWD_BL) {
    k_raymarch_batch<CIN, CB, T, S, BWD_BL><<<blocks, kThreads, 0, st>>>(bp);
  } else {
    k_extinction_sign_batch<CIN, CB, T><<<dim3(blocks, unsigned(bp.count)), 256, 0, st>>>(bp);
  }
}

template <class T, class S>
int launch_batch_typed(int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp) {
  if (cin == 1 && cb == 2) launch_batch<1, 2, T, S>(which, blocks, st, bp);
  else if (cin == 1 && cb == 4) launch_batch<1, 4, T, S>(which, blocks, st, bp);
  else if (cin == 2 && cb == 2) launch_batch<2, 2, T, S>(which, blocks, st, bp);
  else if (cin == 4 && cb == 4) launch_batch<4, 4, T, S>(which, blocks, st, bp);
  else return fail(NGT_ERR_UNSUPPORTED, "raymarch batch: channels must be 1 (with emission 2 or 4), 2 or 4");
  return NGT_OK;
}

int launch_batch_dtype(int dtype, int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp) {
  switch (dtype) {
    case NGT_F32: return launch_batch_typed<float, float>(which, cin, cb, blocks, st, bp);
    case NGT_BF16: return launch_batch_typed<__nv_bfloat16, float>(which, cin, cb, blocks, st, bp);
    case NGT_F16: return launch_batch_typed<__half, float>(which, cin, cb, blocks, st, bp);
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

// A prepared quad layout: [extinction-sign word, 256 bytes][quad input].
constexpr size_t kQuadHeader = 256;

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
struct Layout {
  size_t flag, cams, quad, gquad, buf, wsum, total;
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

int launch_slots(int dtype, int which, int cin, int cb, int tiles, cudaStream_t st, RayParams& p) {
  const int slots = num_slots(p);
  for (int s0 = 0; s0 < slots; s0 += 65535) {
    p.slot0 = s0;
    const int rc = launch_dtype(dtype, which, cin, cb, dim3(tiles, min(65535, slots - s0)), st, p);
    if (rc) return rc;
  }
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

extern "C" size_t ngt_raymarch_quad_bytes(const ngt_raymarch_args* a) {
  return a && quad_case(a) ? kQuadHeader + quad_bytes(a) : 0;
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
  if (cudaMemsetAsync(q, 0, sizeof(int), st) != cudaSuccess) return check_launch("raymarch_quad memset");
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

extern "C" int ngt_raymarch_bwd(const ngt_raymarch_grad_args* a, void* stream) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd: null arguments");
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
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "raymarch_bwd: the forward output is required");
  if ((rc = check_aligned("raymarch_bwd", arith_bytes(a->fwd.dtype),
                          {{"output", a->output}, {"output_grad", a->output_grad}, {"input_grad", a->input_grad}})))
    return rc;
  if ((rc = check_prepared_quad(&a->fwd))) return rc;
  const Layout l = bwd_layout(a);
  if (!a->workspace || a->workspace_bytes < l.total)
    return fail(NGT_ERR_WORKSPACE, "raymarch_bwd: needs %zu workspace bytes", l.total);
  RayParams p = make_params(&a->fwd);
  p.out_fwd = a->output;
  p.out_grad = a->output_grad;
  p.in_grad = a->input_grad;
  cudaStream_t st = as_stream(stream);
  char* w = static_cast<char*>(a->workspace);
  const int64_t vox = p.din.count();
  const size_t cs = compute_size(a->fwd.dtype);
  const int tiles = ceil_div_u(p.W, kTileX) * ceil_div_u(p.H, kTileY);
  build_cams(p, &a->fwd, w + l.cams, st);

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
      rc = launch_slots(a->fwd.dtype, BWD_BL, cin, cb, tiles, st, p);  // one-pass, or checkpointed on the flag
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
int raymarch_bwd_batch(const ngt_raymarch_grad_args* items, int32_t count, int32_t blocks_per_sm, void* workspace,
                       size_t workspace_bytes, void* stream, bool reuse) {
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
  rc = launch_batch_dtype(dtype, BWD_BL, cin, cb, blocks, st, bp);
  if (rc) return rc;
  if (quad) k_quad_fold_batch<<<unsigned(bp.cblock_end[count - 1]), dim3(32, 8), 0, st>>>(bp);
  return check_launch(reuse ? "ngt_raymarch_bwd_batch_after_fwd" : "ngt_raymarch_bwd_batch");
}
}  // namespace

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
