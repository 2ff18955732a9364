// Kernels of the fused frustum raymarch: per-pixel ray through the volume, sample + blend
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
// This header holds the device code; each raymarch_<type>.cu translation unit
// instantiates the kernels of one storage type (compiled in parallel) and
// raymarch.cu holds the host entry points and the small set-up kernels.
#pragma once

#include "ngt_common.cuh"
#include "ngt_host.cuh"
#include "ngt_blend.cuh"
#include "ngt_quad.cuh"

namespace ngt {
// Types and launchers shared by the raymarch translation units.
namespace rm {

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
  const float4* rays;    // per-ray start, step and sample count (ngt_raymarch_rays) or null
  // with a ray table: the (slot, tile) items in descending order of their rays'
  // sample counts, block b of a 1-D launch taking item order[b]; null: block
  // (tile, slot) = (blockIdx.x, slot0 + blockIdx.y)
  const int* order;
  int tiles;             // tiles per slot
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
  // deterministic exact backward: fixed-point accumulators (one 64-bit integer
  // per input cell and channel), the pass statistics and the number of rays
  unsigned long long* fix;
  struct FixStats* fst;
  int64_t nrays;
  // sample cache (ngt_raymarch_args::sample_cache): every ray's first D density
  // samples, stored by the Beer-Lambert forward and read by the one-pass
  // backward when the tag word holds ``sample_tag`` (the forward writes it);
  // null: not kept
  float* samples;
  unsigned long long* sample_word;
  unsigned long long sample_tag;
};

// Deterministic exact backward.  Float atomics add the samples' contributions in
// whatever order the blocks run, so the sums vary in their last bits from run to
// run.  Here each contribution is rounded to a fixed-point integer of scale 2^E
// and added with 64-bit integer atomics: integer addition is associative, so
// every run gives the same sums, and the result is converted once at the end.
// A first pass over the same rays (SC_MAX) takes the largest |contribution| and
// the most samples of any ray; with |g| < 2^eg and rays * samples <= 2^en,
// E = 62 - eg - en keeps every cell's sum below 2^62 (no overflow) and resolves
// each contribution to 2^(en - 62) of the largest one.
enum ScatterMode { SC_ATOMIC = 0, SC_MAX = 1, SC_FIXED = 2 };

struct FixStats {
  unsigned gmax_bits;  // float bits of the largest |contribution| (non-negative, so ordered as integers)
  int samples_max;     // most samples of one ray
};

// per-thread statistics of the SC_MAX pass
struct FixAcc {
  float gmax;
  int samples;
};

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

enum Which { FWD = 0, BWD_EXACT = 1, BWD_REF = 2, BWD_BL = 3, SIGN = 4, BWD_EXACT_MAX = 5, BWD_EXACT_FIX = 6,
             BWD_BL_MAX = 7, BWD_BL_FIX = 8, FWD_L2_BWD = 9 };


// Launch one pass of the single-scene kernels (``which``) for the storage type in
// the name; defined in raymarch_<type>.cu.
int launch_f32(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p);
int launch_f64(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p);
int launch_bf16(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p);
int launch_f16(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p);
// The same for the persistent batch kernels (float and 16-bit storage).
int launch_batch_f32(int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp);
int launch_batch_bf16(int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp);
int launch_batch_f16(int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp);

}  // namespace rm

namespace {
using namespace rm;

__device__ __forceinline__ int fix_exponent(const FixStats* f, int64_t rays) {
  const float g = __uint_as_float(f->gmax_bits);
  if (!(g > 0.0f)) return 0;
  int eg;
  frexpf(g, &eg);  // g = m * 2^eg, m in [0.5, 1): |contribution| <= g < 2^eg
  const unsigned long long n = (unsigned long long)rays * (unsigned long long)max(f->samples_max, 1);
  const int en = n > 1 ? 64 - __clzll(n - 1) : 0;
  return 62 - eg - en;
}

__device__ __forceinline__ long long to_fixed(float v, int e) { return __float2ll_rn(ldexpf(v, e)); }
__device__ __forceinline__ long long to_fixed(double v, int e) { return __double2ll_rn(ldexp(v, e)); }
__device__ __forceinline__ float abs_up(float v) { return fabsf(v); }
__device__ __forceinline__ float abs_up(double v) { return __double2float_ru(fabs(v)); }

// scatter_linear with fixed-point integer accumulation
template <int C, class S>
__device__ __forceinline__ void scatter_fixed(unsigned long long* __restrict__ acc, S px, S py, S pz, const Dims& d,
                                              int bm, const S g[C], int e) {
  const Tri<S> t = tri_setup(px, py, pz, d, bm);
  if (bm == BORDER && !t.inside) return;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    bool ok;
    const int64_t i = tri_corner(t, k, d, ok);
    if (!ok) continue;
    const S w = tri_weight(t, k);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const long long v = to_fixed(mul_rn(g[c], w), e);
      if (v) atomicAdd(acc + i * C + c, (unsigned long long)v);
    }
  }
}

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

// The (slot, tile) item of this block.
__device__ __forceinline__ void block_item(const RayParams& p, int& slot, int& tile) {
  if (p.order) {
    const int it = __ldg(p.order + blockIdx.x);
    slot = it / p.tiles;
    tile = it - slot * p.tiles;
  } else {
    slot = p.slot0 + int(blockIdx.y);
    tile = int(blockIdx.x);
  }
}

// This thread's pixel within its 16x8 tile: each warp covers 8x4 pixels (rays
// that stay close in the grid, so a warp's gathers share cache lines); warps 0
// and 1 side by side in x, warps 2 and 3 below them.
__device__ __forceinline__ void pixel_of_thread(int& px, int& py) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  px = (warp & 1) * 8 + (lane & 7);
  py = (warp >> 1) * 4 + (lane >> 3);
}

// This thread's first cached sample: warp w of tile t of slot s owns D x 32
// floats, sample i of lane l at i * 32 + l.
__device__ __forceinline__ int64_t sample_slot(const RayParams& p, int slot, int tile) {
  const int tiles = ((p.W + kTileX - 1) / kTileX) * ((p.H + kTileY - 1) / kTileY);
  return ((int64_t(slot) * tiles + tile) * (kThreads / 32) + (threadIdx.x >> 5)) * int64_t(p.D) * 32 +
         (threadIdx.x & 31);
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

// Where a kernel takes its rays: RAYS_ANY reads the prepared table when the call
// has one and sets the ray up otherwise; the render's two hot kernels are
// instantiated for one source each (RAYS_TABLE / RAYS_SETUP), so they carry the
// registers of only one.
enum RaySource { RAYS_ANY = 0, RAYS_TABLE = 1, RAYS_SETUP = 2 };

// The ray of pixel (px, py) of output slot ``slot``: from the prepared ray table
// (ngt_raymarch_rays) or set up here in float arithmetic.
template <int RAYS = RAYS_ANY>
__device__ __forceinline__ Ray ray_of(const Cam& cam, int slot, int px, int py, const RayParams& p) {
  if (RAYS == RAYS_TABLE || (RAYS == RAYS_ANY && p.rays)) {
    const float4* q = p.rays + 2 * ((int64_t(slot) * p.H + py) * p.W + px);
    const float4 a = q[0], b = q[1];
    Ray r;
    r.s[0] = a.x;
    r.s[1] = a.y;
    r.s[2] = a.z;
    r.steps = __float_as_int(a.w);
    r.st[0] = b.x;
    r.st[1] = b.y;
    r.st[2] = b.z;
    r.hit = b.w != 0.0f;
    r.e[0] = r.e[1] = r.e[2] = 0.0f;  // the far end is only used by the reference backward, which sets up its own
    return r;
  }
  return ray_setup(cam, px, py, p);
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

template <int CIN, int CB, int MODE = SC_ATOMIC, class S>
__device__ __forceinline__ void scatter_cell(const RayParams& p, S* __restrict__ grad, float4* gq, const float pos[3],
                                             const S dcell[CB], FixAcc* fa = nullptr, int fe = 0) {
  const S px = S(pos[0] - 0.5f), py = S(pos[1] - 0.5f), pz = S(pos[2] - 0.5f);
  if constexpr (MODE != SC_ATOMIC) {
    // the deterministic passes: the sample's input-channel gradient, then its
    // statistics (SC_MAX) or its fixed-point scatter (SC_FIXED)
    S g[CIN];
    if (CIN == CB) {
#pragma unroll
      for (int c = 0; c < CIN; ++c) g[c] = dcell[c < CB ? c : 0];
    } else {
      g[0] = S(0);
#pragma unroll
      for (int c = 0; c < CB; ++c) g[0] += S(p.scale[c]) * dcell[c];
    }
    if constexpr (MODE == SC_MAX) {
#pragma unroll
      for (int c = 0; c < CIN; ++c) fa->gmax = fmaxf(fa->gmax, abs_up(g[c]));
      fa->samples += 1;
    } else {
      scatter_fixed<CIN>(p.fix + int64_t(grad - static_cast<S*>(p.in_grad)), px, py, pz, p.din, p.bm, g, fe);
    }
    return;
  }
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
template <int CIN, int CB, class T, class S, int RAYS = RAYS_ANY>
__device__ __forceinline__ S fwd_tile(const RayParams& p, const Cam& cam, int b, int oslot, int tile) {
  int px, py;
  if (!tile_pixel(p, tile, px, py)) return S(0);
  const int64_t pix = (int64_t(oslot) * p.H + py) * p.W + px;
  const T* g = reinterpret_cast<const T*>(p.input) + int64_t(b) * p.din.count() * CIN;
  const void* qg = quad_of<CIN, T>(p, b);
  const Ray r = ray_of<RAYS>(cam, oslot, px, py, p);
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
      float* sv = RAYS != RAYS_SETUP && p.samples ? p.samples + sample_slot(p, oslot, tile) : nullptr;
      const int ns = sv ? min(r.steps, p.D) : 0;
      for (int i = 0; i < r.steps; ++i) {
        QuadPos qp;
        float v;
        quad_sample_fma<T>(q, pos[0] - 0.5f, pos[1] - 0.5f, pos[2] - 0.5f, p.din, p.qd, p.bm, qp, v);
        if (i < ns) sv[int64_t(i) * 32] = v;
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

template <int CIN, int CB, class T, class S, int RAYS>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_raymarch_fwd(RayParams p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot, slot, tile;
  block_item(p, slot, tile);
  slot_to_bc(p, slot, b, c, oslot);
  load_cam(p, slot, b, c, cam, cam_sh);
  __syncthreads();
  const S l = fwd_tile<CIN, CB, T, S, RAYS>(p, cam, b, oslot, tile);
  if (p.l2_loss) l2_block_add<S>(l, static_cast<S*>(p.l2_loss));
  if (p.samples && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *p.sample_word = p.sample_tag;
}

// ------------------------------------------------------- exact backward
// Accumulator states are recomputed forward (checkpoints every K steps, then
// each segment re-marched into a small buffer and walked back), so the adjoint
// uses the forward's own positions and densities, not a subtraction.
template <int CIN, int CB, class T, class S, int MODE = SC_ATOMIC, int RAYS = RAYS_ANY>
__device__ __forceinline__ void bwd_exact_tile(const RayParams& p, const Cam& cam, int b, int oslot, int tile,
                                               FixAcc* fa = nullptr, int fe = 0) {
  int px, py;
  if (!tile_pixel(p, tile, px, py)) return;
  const T* g = reinterpret_cast<const T*>(p.input) + int64_t(b) * p.din.count() * CIN;
  const void* qg = quad_of<CIN, T>(p, b);
  S* grad = reinterpret_cast<S*>(p.in_grad) + int64_t(b) * p.din.count() * CIN;
  float4* gq = gquad_of(p, b);
  const Ray r = ray_of<RAYS>(cam, oslot, px, py, p);
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
      scatter_cell<CIN, CB, MODE>(p, grad, gq, pos, dcell, fa, fe);
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
        scatter_cell<CIN, CB, MODE>(p, grad, gq, buf_pos[j], dcell, fa, fe);
      }
    }
  }
}

// Block-wide maxima of the SC_MAX pass into the call's statistics.
__device__ __forceinline__ void fix_stats_add(const FixAcc& fa, FixStats* fst) {
  float g = fa.gmax;
  int n = fa.samples;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    g = fmaxf(g, __shfl_xor_sync(0xffffffffu, g, o));
    n = max(n, __shfl_xor_sync(0xffffffffu, n, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&fst->gmax_bits, __float_as_uint(g));
    atomicMax(&fst->samples_max, n);
  }
}

template <int CIN, int CB, class T, class S, int MODE = SC_ATOMIC>
__global__ void __launch_bounds__(kThreads) k_raymarch_bwd_exact(RayParams p) {
  if (p.flag && *p.flag == 0) return;  // Beer-Lambert with non-negative extinction: k_raymarch_bwd_bl
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot;
  slot_to_bc(p, p.slot0 + blockIdx.y, b, c, oslot);
  load_cam(p, p.slot0 + blockIdx.y, b, c, cam, cam_sh);
  __syncthreads();
  if constexpr (MODE == SC_ATOMIC) {
    bwd_exact_tile<CIN, CB, T, S>(p, cam, b, oslot, blockIdx.x);
  } else {
    FixAcc fa = {0.0f, 0};
    bwd_exact_tile<CIN, CB, T, S, MODE>(p, cam, b, oslot, blockIdx.x, &fa,
                                        MODE == SC_FIXED ? fix_exponent(p.fst, p.nrays) : 0);
    if constexpr (MODE == SC_MAX) fix_stats_add(fa, p.fst);
  }
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
// ``fresh``: this thread has just run the forward of its ray (the fused launch),
// so the samples it cached are there whatever the tag word says.
template <int CIN, int CB, class T, class S, int MODE = SC_ATOMIC, int RAYS = RAYS_ANY>
__device__ __forceinline__ void bwd_bl_tile(const RayParams& p, const Cam& cam, int b, int oslot, int tile,
                                            FixAcc* fa = nullptr, int fe = 0, bool fresh = false) {
  int px, py;
  if (!tile_pixel(p, tile, px, py)) return;
  const T* g = reinterpret_cast<const T*>(p.input) + int64_t(b) * p.din.count() * CIN;
  const void* qg = quad_of<CIN, T>(p, b);
  S* grad = reinterpret_cast<S*>(p.in_grad) + int64_t(b) * p.din.count() * CIN;
  float4* gq = gquad_of(p, b);
  const Ray r = ray_of<RAYS>(cam, oslot, px, py, p);
  if (!r.hit || r.steps <= 0) return;
  const int64_t o = ((int64_t(oslot) * p.H + py) * p.W + px) * CB;
  S G[CB];
  S lgf = S(0);
#pragma unroll
  for (int k = 0; k < CB; ++k) G[k] = reinterpret_cast<const S*>(p.out_grad)[o + k];
#pragma unroll
  for (int k = 0; k < CB - 1; ++k) lgf += G[k] * reinterpret_cast<const S*>(p.out_fwd)[o + k];
  const S gD = G[CB - 1];
  if constexpr (quad_able<CIN, T>() && std::is_same<S, float>::value && MODE == SC_ATOMIC) {
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
      // the forward's samples of these rays, when it kept them (a cache is tagged
      // with a ray table, so the instance that sets its rays up has none)
      const float* sv = RAYS != RAYS_SETUP && p.samples && (fresh || *p.sample_word == p.sample_tag)
                            ? p.samples + sample_slot(p, oslot, tile)
                            : nullptr;
      const int ns = sv ? min(r.steps, p.D) : 0;
      for (int i = 0; i < r.steps; ++i) {
        QuadPos qp;
        float v;
        bool in;
        if (i < ns) {
          in = quad_setup(pos[0] - 0.5f, pos[1] - 0.5f, pos[2] - 0.5f, p.din, p.qd, p.bm, qp);
          v = __ldcs(sv + int64_t(i) * 32);
        } else {
          in = quad_sample_fma<T>(q, pos[0] - 0.5f, pos[1] - 0.5f, pos[2] - 0.5f, p.din, p.qd, p.bm, qp, v);
        }
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
    scatter_cell<CIN, CB, MODE>(p, grad, gq, pos, dcell, fa, fe);
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] += r.st[a];
  }
}

// The checkpointed adjoint as a call of its own (its registers and stack do not
// weigh on the one-pass kernel that calls it for launches with a possibly
// negative extinction sample).
template <int CIN, int CB, class T, class S, int RAYS = RAYS_ANY>
__device__ __noinline__ void bwd_exact_tile_call(const RayParams& p, const Cam& cam, int b, int oslot, int tile) {
  bwd_exact_tile<CIN, CB, T, S, SC_ATOMIC, RAYS>(p, cam, b, oslot, tile);
}

template <int CIN, int CB, class T, class S, int RAYS>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_raymarch_bwd_bl(const __grid_constant__ RayParams p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot, slot, tile;
  block_item(p, slot, tile);
  slot_to_bc(p, slot, b, c, oslot);
  load_cam(p, slot, b, c, cam, cam_sh);
  __syncthreads();
  if (*p.flag != 0)
    bwd_exact_tile_call<CIN, CB, T, S, RAYS>(p, cam, b, oslot, tile);
  else
    bwd_bl_tile<CIN, CB, T, S, SC_ATOMIC, RAYS>(p, cam, b, oslot, tile);
}

// Forward, image L2 loss and one-pass backward of every ray in one launch.  The
// loss gradient of a pixel depends on that pixel's output alone, so the thread
// that marched a ray forward (writing its image pixel and loss gradient, and
// caching its samples) marches it again for the adjoint, reading back what it
// wrote: no other block's results are needed, and the image and its gradient
// are not read back by a second launch.  Launches with a possibly negative
// extinction sample take the checkpointed adjoint after the forward.
template <int CIN, int CB, class T, class S, int RAYS>
__global__ void __launch_bounds__(kThreads, 8) k_raymarch_fwd_bwd(const __grid_constant__ RayParams p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot, slot, tile;
  block_item(p, slot, tile);
  slot_to_bc(p, slot, b, c, oslot);
  load_cam(p, slot, b, c, cam, cam_sh);
  __syncthreads();
  const S l = fwd_tile<CIN, CB, T, S, RAYS>(p, cam, b, oslot, tile);
  l2_block_add<S>(l, static_cast<S*>(p.l2_loss));
  if (p.samples && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *p.sample_word = p.sample_tag;
  if (*p.flag != 0)
    bwd_exact_tile_call<CIN, CB, T, S, RAYS>(p, cam, b, oslot, tile);
  else
    bwd_bl_tile<CIN, CB, T, S, SC_ATOMIC, RAYS>(p, cam, b, oslot, tile, nullptr, 0, true);
}

// The deterministic passes of the exact Beer-Lambert backward (statistics, then
// fixed-point scatter): the one-pass adjoint, or the checkpointed one where the
// extinction-sign check failed, over the same rays as k_raymarch_bwd_bl.
template <int CIN, int CB, class T, class S, int MODE>
__global__ void __launch_bounds__(kThreads) k_raymarch_bwd_bl_det(const __grid_constant__ RayParams p) {
  __shared__ Cam cam;
  __shared__ CamScratch cam_sh;
  int b, c, oslot;
  slot_to_bc(p, p.slot0 + blockIdx.y, b, c, oslot);
  load_cam(p, p.slot0 + blockIdx.y, b, c, cam, cam_sh);
  __syncthreads();
  FixAcc fa = {0.0f, 0};
  const int fe = MODE == SC_FIXED ? fix_exponent(p.fst, p.nrays) : 0;
  if (*p.flag != 0)
    bwd_exact_tile<CIN, CB, T, S, MODE>(p, cam, b, oslot, blockIdx.x, &fa, fe);
  else
    bwd_bl_tile<CIN, CB, T, S, MODE>(p, cam, b, oslot, blockIdx.x, &fa, fe);
  if constexpr (MODE == SC_MAX) fix_stats_add(fa, p.fst);
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

template <int CIN, int CB, class T, class S>
void launch(int which, dim3 grid, cudaStream_t st, const RayParams& p) {
  if (which == FWD) {
    if (p.rays)
      k_raymarch_fwd<CIN, CB, T, S, RAYS_TABLE><<<grid, kThreads, 0, st>>>(p);
    else
      k_raymarch_fwd<CIN, CB, T, S, RAYS_SETUP><<<grid, kThreads, 0, st>>>(p);
  } else if (which == BWD_EXACT) {
    k_raymarch_bwd_exact<CIN, CB, T, S><<<grid, kThreads, 0, st>>>(p);
  } else if (which == BWD_BL) {
    if (CB > 1) {
      if (p.rays)
        k_raymarch_bwd_bl<CIN, CB, T, S, RAYS_TABLE><<<grid, kThreads, 0, st>>>(p);
      else
        k_raymarch_bwd_bl<CIN, CB, T, S, RAYS_SETUP><<<grid, kThreads, 0, st>>>(p);
    }
  } else if (which == FWD_L2_BWD) {
    if constexpr (CB > 1) {
      if (p.rays)
        k_raymarch_fwd_bwd<CIN, CB, T, S, RAYS_TABLE><<<grid, kThreads, 0, st>>>(p);
      else
        k_raymarch_fwd_bwd<CIN, CB, T, S, RAYS_SETUP><<<grid, kThreads, 0, st>>>(p);
    }
  } else if (which == BWD_EXACT_MAX) {
    k_raymarch_bwd_exact<CIN, CB, T, S, SC_MAX><<<grid, kThreads, 0, st>>>(p);
  } else if (which == BWD_EXACT_FIX) {
    k_raymarch_bwd_exact<CIN, CB, T, S, SC_FIXED><<<grid, kThreads, 0, st>>>(p);
  } else if (which == BWD_BL_MAX) {
    if (CB > 1) k_raymarch_bwd_bl_det<CIN, CB, T, S, SC_MAX><<<grid, kThreads, 0, st>>>(p);
  } else if (which == BWD_BL_FIX) {
    if (CB > 1) k_raymarch_bwd_bl_det<CIN, CB, T, S, SC_FIXED><<<grid, kThreads, 0, st>>>(p);
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
    if (WHICH == FWD) {
      fwd_tile<CIN, CB, T, S>(p, cam, b, oslot, tile);
      continue;
    }
    if (WHICH == FWD_L2_BWD) {  // the item's forward and loss, then its backward by the same threads
      const S l = fwd_tile<CIN, CB, T, S>(p, cam, b, oslot, tile);
      l2_block_add<S>(l, static_cast<S*>(p.l2_loss));
    }
    if (checkpointed || CB == 1)
      bwd_exact_tile_call<CIN, CB, T, S>(p, cam, b, oslot, tile);
    else
      bwd_bl_tile<CIN, CB, T, S>(p, cam, b, oslot, tile);
  }
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
  } else if (which == FWD_L2_BWD) {
    k_raymarch_batch<CIN, CB, T, S, FWD_L2_BWD><<<blocks, kThreads, 0, st>>>(bp);
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


}  // namespace
}  // namespace ngt
