// Fused semi-Lagrangian / MacCormack advection by a MAC-staggered velocity and
// its gradient: of a cell-centred grid (density) and of the velocity itself
// (each face component on its own staggered lattice).
//
// The reference composes this in TensorFlow: VelocityGrid.warp
// (data_structures.py:1690-1737) -- centred velocity (:1634-1654), lookup
// ``-u*dt`` (:1684-1688), SampleGridLut forward and back, correction
// ``fwd + 0.5*(data - back)``, MIN / MAX lookups and the MC_SMOOTH revert clamp --
// and VelocityGrid.warped (:1108-1164), which builds each component's lookup from
// the other components resampled at +-1/2 cell offsets (:1655-1682) and warps it
// the same way (_warp_vel_component, :1081-1106).  Here a warp is two kernels
// forward and three backward:
//
//   forward 1: lookup from the velocity, trilinear forward trace -> fwd field
//   forward 2: back-trace of fwd, correction, extrema of the forward trace's
//              corners, revert clamp                                -> output
//   backward 1: recompute the state, route the correction's gradient; scatter the
//               back-trace adjoint into the fwd-field gradient; lookup gradient
//               of the back-trace
//   backward 2: scatter the fwd-field gradient into the data gradient; lookup
//               gradient of the forward trace
//   backward 3: lookup gradient back to the faces (density: a gather over the two
//               faces of each cell; velocity: the identity channel plus the
//               adjoint of the +-1/2 offset resamples)
//
// Arithmetic of positions, interpolation and correction is explicitly rounded in
// the composition's order, so float32 results equal an op-by-op evaluation of
// the reference's formula and the clamp mask is reproduced exactly.
#include "ngt_common.cuh"
#include "ngt_gather.cuh"
#include "ngt_host.cuh"
#include "ngt_tma.cuh"

#include <atomic>
#include <mutex>

namespace ngt {
namespace {

constexpr int kBlock = 256;

template <class T>
using CT = typename Compute<T>::type;

// -------------------------------------------------------------- lookups
// lookup = centred(u) * (-dt) (data_structures.py:1634-1654, 1684-1688)
template <class T>
struct CenteredLookup {
  const T* vx;
  const T* vy;
  const T* vz;
  Dims d;  // cell lattice
  float dt;
  __device__ __forceinline__ void operator()(int x, int y, int z, CT<T> lut[3]) const {
    typedef CT<T> S;
    const S h = S(0.5);
    const S ux0 = S(ld(vx + (int64_t(z) * d.y + y) * (d.x + 1) + x));
    const S ux1 = S(ld(vx + (int64_t(z) * d.y + y) * (d.x + 1) + x + 1));
    const S uy0 = S(ld(vy + (int64_t(z) * (d.y + 1) + y) * d.x + x));
    const S uy1 = S(ld(vy + (int64_t(z) * (d.y + 1) + y + 1) * d.x + x));
    const S uz0 = S(ld(vz + (int64_t(z) * d.y + y) * d.x + x));
    const S uz1 = S(ld(vz + (int64_t(z + 1) * d.y + y) * d.x + x));
    const S ndt = S(-dt);
    lut[0] = mul_rn(mul_rn(add_rn(ux1, ux0), h), ndt);
    lut[1] = mul_rn(mul_rn(add_rn(uy1, uy0), h), ndt);
    lut[2] = mul_rn(mul_rn(add_rn(uz1, uz0), h), ndt);
  }
};

// Offset (added to the target index) at which component ``src`` is resampled on
// the lattice of component ``tgt`` (data_structures.py:1655-1682).
__device__ __forceinline__ float comp_offset(int src, int tgt, int axis) {
  if (axis == src) return 0.5f;   // source faces sit half a cell below along their own axis
  if (axis == tgt) return -0.5f;  // target faces sit half a cell below along theirs
  return 0.0f;
}

__host__ __device__ __forceinline__ Dims face_dims(const Dims& c, int comp) {
  return Dims{c.x + (comp == 0), c.y + (comp == 1), c.z + (comp == 2)};
}

// lookup of component ``tgt``: ``(-vel) * dt`` of all components on tgt's lattice
template <class T>
struct FaceLookup {
  const T* u[3];
  Dims cells;
  int tgt;
  int bm;
  float dt;
  __device__ __forceinline__ void operator()(int x, int y, int z, CT<T> lut[3]) const {
    typedef CT<T> S;
    const S ndt = S(dt);
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      S v;
      if (s == tgt) {
        v = S(ld(u[s] + flat(x, y, z, face_dims(cells, s))));
      } else {
        S o[1];
        read_linear<1>(u[s], add_rn(S(comp_offset(s, tgt, 0)), S(x)), add_rn(S(comp_offset(s, tgt, 1)), S(y)),
                       add_rn(S(comp_offset(s, tgt, 2)), S(z)), face_dims(cells, s), bm, o);
        v = o[0];
      }
      lut[s] = mul_rn(-v, ndt);
    }
  }
};

// The lookup that forward 1 of a face component stored (3 values per face).
template <class T>
struct StoredLookup {
  const CT<T>* lut;
  Dims d;
  __device__ __forceinline__ void operator()(int x, int y, int z, CT<T> out[3]) const {
    const int64_t i = flat(x, y, z, d) * 3;
    out[0] = lut[i];
    out[1] = lut[i + 1];
    out[2] = lut[i + 2];
  }
};

// Forward 1 and backward 2 of one channel of 16-bit data with a cell-centred or
// stored lookup are held to the f32 variants' register counts (32 and 48: 8 and 5
// resident 256-thread blocks per SM); left to themselves they take 33 and 50 and
// lose a block per SM.  Every other variant is unbounded (minimum blocks 0).
template <int C, class T, class LK>
__host__ __device__ constexpr bool mc_narrow16() {
  return C == 1 && sizeof(T) == 2 && !std::is_same<LK, FaceLookup<T>>::value;
}

// ------------------------------------------------------------ MacCormack core
template <class T>
struct McParams {
  const T* data;
  T* out;
  CT<T>* fwd;          // fwd field (compute type)
  const CT<T>* gout;
  CT<T>* gdata;
  CT<T>* gfwd;         // workspace: gradient w.r.t. the fwd field
  CT<T>* glut;         // workspace: gradient w.r.t. the lookup (3 per cell)
  CT<T>* buf;          // reference mode: unnormalised scatter
  unsigned* cnt;       // reference mode: sample counts
  CT<T>* gback;        // deterministic mode: back-trace gradient per cell (scattered in fixed point afterwards)
  CT<T>* gface[3];     // density, non-deterministic: face gradients accumulated by backward 2
  uint8_t* mask;       // MC_SMOOTH revert mask: written by forward 2, read by backward 1 (optional)
  CT<T>* ext;          // MC_SMOOTH: the forward trace's corner extrema (min, max per cell and channel),
                       //   written by forward 1, read instead of gathered again (optional)
  CT<T>* lut_out;      // forward 1 also stores its lookup here (3 per cell; optional)
  float dt;            // with gface: the lookup is centred(u) * (-dt)
  Dims d;
  int order, clamp, bm, reference;
  int accumulate;      // add (atomically) the direct data gradient instead of writing it
  int det;             // deterministic: no float scatter here, the fixed-point scatter follows
};

__device__ __forceinline__ void cell_of(int64_t i, const Dims& d, int& x, int& y, int& z) {
  x = int(i % d.x);
  y = int((i / d.x) % d.y);
  z = int(i / (int64_t(d.x) * d.y));
}

template <int C, class T, class LK>
__device__ __forceinline__ void mc_fwd1_at(const McParams<T>& p, const LK& lk, int x, int y, int z) {
  typedef CT<T> S;
  const int64_t i = flat(x, y, z, p.d);
  S lut[3];
  lk(x, y, z, lut);
  if (p.lut_out) {
#pragma unroll
    for (int k = 0; k < 3; ++k) p.lut_out[i * 3 + k] = lut[k];
  }
  S v[C];
  if (p.ext && p.order == 2 && p.clamp == NGT_CLAMP_MC_SMOOTH) {
    // the trilinear value and the corner extrema from one fetch of the eight
    // corners (read_linear and read_minmax: out-of-range BORDER corners read 0,
    // which is also what read_minmax's extrema start from when one is out)
    const Tri<S> t = tri_setup(add_rn(lut[0], S(x)), add_rn(lut[1], S(y)), add_rn(lut[2], S(z)), p.d, p.bm);
    S mn[C], mx[C];
    if (p.bm == BORDER && !t.inside) {
#pragma unroll
      for (int c = 0; c < C; ++c) v[c] = mn[c] = mx[c] = S(0);
    } else {
      S vc[8][C];
      tri_fetch<C>(p.data, t, p.d, vc);
      tri_combine<C>(vc, t, v);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        mn[c] = S(kFloatMax);
        mx[c] = S(-kFloatMax);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (vc[k][c] < mn[c]) mn[c] = vc[k][c];
          if (vc[k][c] > mx[c]) mx[c] = vc[k][c];
        }
      }
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
      p.fwd[i * C + c] = v[c];
      p.ext[(i * C + c) * 2 + 0] = mn[c];
      p.ext[(i * C + c) * 2 + 1] = mx[c];
    }
    return;
  }
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

template <int C, class T, class LK>
__global__ void __launch_bounds__(kBlock, (mc_narrow16<C, T, LK>() ? 8 : 0)) k_mc_fwd1(McParams<T> p, LK lk) {
  int x, y, z;
  if (!launch_cell(p.d, x, y, z)) return;
  mc_fwd1_at<C>(p, lk, x, y, z);
}

// Where forward 2's back-trace reads the fwd field's eight corners: global memory,
// or a brick of it staged in shared memory (global reads for corners outside it).
struct GlobalFetch {
  template <int C, class V, class S>
  __device__ __forceinline__ void operator()(const V* g, const Tri<S>& t, const Dims& d, S v[8][C]) const {
    tri_fetch<C>(g, t, d, v);
  }
};

// A one-channel brick of kBrickX x kBrickY x kBrickZ values whose element (0, 0, 0)
// is cell (ox, oy, oz) of the grid; corners outside it are read from ``g``.
constexpr int kTileX = 32, kTileY = 8, kTileZ = 4, kHalo = 4;
constexpr int kBrickX = kTileX + 2 * kHalo, kBrickY = kTileY + 2 * kHalo, kBrickZ = kTileZ + 2 * kHalo;

struct BrickFetch {
  const float* brick;
  int ox, oy, oz;
  bool ok;  // false: the brick did not arrive, every corner is read from global memory
  template <int C, class V, class S>
  __device__ __forceinline__ void operator()(const V* g, const Tri<S>& t, const Dims& d, S v[8][C]) const {
    // one base element and the upper corners' offsets (0 where the boundary rule
    // put both corners of an axis on one cell); the corners' order is tri_fetch's
    const int x0 = t.i0[0] - ox, y0 = t.i0[1] - oy, z0 = t.i0[2] - oz;
    const int dx = t.i1[0] - t.i0[0], dy = t.i1[1] - t.i0[1], dz = t.i1[2] - t.i0[2];
    const bool in = ok && C == 1 && unsigned(x0) < unsigned(kBrickX - 1) && unsigned(y0) < unsigned(kBrickY - 1) &&
                    unsigned(z0) < unsigned(kBrickZ - 1) && unsigned(dx) <= 1u && unsigned(dy) <= 1u &&
                    unsigned(dz) <= 1u;
    if (!in) {
      tri_fetch<C>(g, t, d, v);
      return;
    }
    const float* b = brick + (z0 * kBrickY + y0) * kBrickX + x0;
    const int oy = dy * kBrickX, oz = dz * (kBrickX * kBrickY);
    const float c[8] = {b[0], b[dx], b[oy], b[oy + dx], b[oz], b[oz + dx], b[oz + oy], b[oz + oy + dx]};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const bool valid = ((k & 1) ? t.ok1[0] : t.ok0[0]) && ((k & 2) ? t.ok1[1] : t.ok0[1]) &&
                         ((k & 4) ? t.ok1[2] : t.ok0[2]);
      v[k][0] = valid ? S(c[k]) : S(0);
    }
  }
};

template <int C, class S>
struct McState {
  S fwd[C], back[C], corr[C], res[C];
  bool mask[C];
};

// With ``stored`` the MC_SMOOTH mask is read from p.mask instead of being
// recomputed from the forward trace's corner extrema.
template <int C, class T, class S, class FE = GlobalFetch>
__device__ __forceinline__ void mc_state(const McParams<T>& p, int64_t i, int x, int y, int z, const S lut[3],
                                         McState<C, S>& s, S vb[8][C], Tri<S>& tb, bool stored = false,
                                         const FE& fe = FE()) {
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
    fe.template operator()<C>(p.fwd, tb, p.d, vb);
  }
  S mn[C], mx[C];
  const bool recompute = p.clamp == NGT_CLAMP_MC_SMOOTH && !(stored && p.mask);
  // the backward needs the corrected value only to recompute the mask or for the
  // NEGATIVE clamp; otherwise only the corners (vb) and the mask
  if (stored && !recompute && p.clamp != NGT_CLAMP_NEGATIVE) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      s.mask[c] = p.clamp == NGT_CLAMP_MC_SMOOTH && p.mask[i * C + c] != 0;
      s.fwd[c] = s.back[c] = s.corr[c] = s.res[c] = S(0);
    }
    return;
  }
  if (!(p.bm == BORDER && !tb.inside)) tri_combine<C>(vb, tb, s.back);
  if (recompute && p.ext) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      mn[c] = p.ext[(i * C + c) * 2 + 0];
      mx[c] = p.ext[(i * C + c) * 2 + 1];
    }
  } else if (recompute) {
    const S p1x = add_rn(lut[0], S(x)), p1y = add_rn(lut[1], S(y)), p1z = add_rn(lut[2], S(z));
    read_minmax<C>(p.data, p1x, p1y, p1z, p.d, p.bm, mn, mx);
  }
#pragma unroll
  for (int c = 0; c < C; ++c) {
    s.fwd[c] = p.fwd[i * C + c];
    const S rho = S(ld(p.data + i * C + c));
    s.corr[c] = add_rn(s.fwd[c], mul_rn(S(0.5), sub_rn(rho, s.back[c])));
    if (recompute)
      s.mask[c] = s.corr[c] < mn[c] || s.corr[c] > mx[c];
    else
      s.mask[c] = p.clamp == NGT_CLAMP_MC_SMOOTH && p.mask[i * C + c] != 0;
    s.res[c] = s.mask[c] ? s.fwd[c] : s.corr[c];
  }
}

template <int C, class T, class LK, class FE = GlobalFetch>
__device__ __forceinline__ void mc_fwd2_at(const McParams<T>& p, const LK& lk, int x, int y, int z,
                                           const FE& fe = FE()) {
  typedef CT<T> S;
  const int64_t i = flat(x, y, z, p.d);
  S lut[3];
  lk(x, y, z, lut);
  McState<C, S> s;
  S vb[8][C];
  Tri<S> tb;
  mc_state<C>(p, i, x, y, z, lut, s, vb, tb, false, fe);
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const S o = (p.clamp == NGT_CLAMP_NEGATIVE) ? fmax(s.res[c], S(0)) : s.res[c];
    p.out[i * C + c] = from_compute<T>(o);
    if (p.mask && p.clamp == NGT_CLAMP_MC_SMOOTH) p.mask[i * C + c] = s.mask[c] ? 1 : 0;
  }
}

template <int C, class T, class LK>
__global__ void __launch_bounds__(kBlock) k_mc_fwd2(McParams<T> p, LK lk) {
  int x, y, z;
  if (!launch_cell(p.d, x, y, z)) return;
  mc_fwd2_at<C>(p, lk, x, y, z);
}

template <class S>
__device__ __forceinline__ void put_direct(S* p, S v, int accumulate) {
  if (accumulate) atomic_add(p, v);
  else *p = v;
}

// backward 1: gradient of the correction; back-trace adjoint into gfwd.  Lanes
// past the row's end stay in the warp (inactive) for the warp-merged scatter.
// (x, y, z) is a cell of the grid; inactive lanes (padding, clamped onto the
// row's last cell) take part in the warp-merged scatter only.
template <int C, class T, class LK>
__device__ __forceinline__ void mc_bwd1_at(const McParams<T>& p, const LK& lk, int x, int y, int z, bool active) {
  typedef CT<T> S;
  const int64_t i = flat(x, y, z, p.d);
  if (p.gface[0] && active && !p.accumulate) {
    // clear the face gradients that backward 2 accumulates: each cell its lower
    // face per axis, the last cell of a line also the upper one
    S* fx = p.gface[0] + (int64_t(z) * p.d.y + y) * (p.d.x + 1) + x;
    S* fy = p.gface[1] + (int64_t(z) * (p.d.y + 1) + y) * p.d.x + x;
    S* fz = p.gface[2] + (int64_t(z) * p.d.y + y) * p.d.x + x;
    fx[0] = S(0);
    fy[0] = S(0);
    fz[0] = S(0);
    if (x == p.d.x - 1) fx[1] = S(0);
    if (y == p.d.y - 1) fy[p.d.x] = S(0);
    if (z == p.d.z - 1) fz[int64_t(p.d.x) * p.d.y] = S(0);
  }
  S lut[3];
  lk(x, y, z, lut);
  S g[C];
  S gl[3] = {S(0), S(0), S(0)};
  if (p.order == 1) {
    S v[C];
    if (p.clamp == NGT_CLAMP_NEGATIVE)
      read_linear<C>(p.data, add_rn(lut[0], S(x)), add_rn(lut[1], S(y)), add_rn(lut[2], S(z)), p.d, p.bm, v);
    if (!active) return;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      g[c] = p.gout[i * C + c];
      if (p.clamp == NGT_CLAMP_NEGATIVE && !(v[c] >= S(0))) g[c] = S(0);
      p.gfwd[i * C + c] = g[c];
      if (!p.accumulate) p.gdata[i * C + c] = S(0);
    }
  } else {
    McState<C, S> s;
    S vb[8][C];
    Tri<S> tb;
    mc_state<C>(p, i, x, y, z, lut, s, vb, tb, true);
    S gback[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      g[c] = p.gout[i * C + c];
      if (p.clamp == NGT_CLAMP_NEGATIVE && !(s.res[c] >= S(0))) g[c] = S(0);
      const S gc = s.mask[c] ? S(0) : g[c];
      gback[c] = -(S(0.5) * gc);
      if (active) put_direct(p.gdata + i * C + c, S(0.5) * gc, p.accumulate);  // direct term of the correction
    }
    const S p2x = add_rn(-lut[0], S(x)), p2y = add_rn(-lut[1], S(y)), p2z = add_rn(-lut[2], S(z));
    if (p.det) {
      if (active) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
          p.gfwd[i * C + c] = g[c];
          p.gback[i * C + c] = gback[c];
        }
      }
    } else if (p.reference) {
      if (active) {
#pragma unroll
        for (int c = 0; c < C; ++c) p.gfwd[i * C + c] = g[c];
        scatter_linear_counted<C>(p.buf, p.cnt, p2x, p2y, p2z, p.d, p.bm, gback);
      }
    } else {
      if (active) {
#pragma unroll
        for (int c = 0; c < C; ++c) atomic_add(p.gfwd + i * C + c, g[c]);
      }
      scatter_linear_warp<C>(p.gfwd, p2x, p2y, p2z, p.d, p.bm, gback, active);
    }
    if (!(p.bm == BORDER && !tb.inside)) {
      S dx[C], dy[C], dz[C];
      tri_gradient<C>(vb, tb, dx, dy, dz);
      // pos2 = idx - lut
#pragma unroll
      for (int c = 0; c < C; ++c) {
        gl[0] -= gback[c] * dx[c];
        gl[1] -= gback[c] * dy[c];
        gl[2] -= gback[c] * dz[c];
      }
    }
  }
  if (!active) return;
  p.glut[i * 3 + 0] = gl[0];
  p.glut[i * 3 + 1] = gl[1];
  p.glut[i * 3 + 2] = gl[2];
}

template <int C, class T, class LK>
__global__ void __launch_bounds__(kBlock, 5) k_mc_bwd1(McParams<T> p, LK lk) {
  int x, y, z;
  const bool active = launch_cell(p.d, x, y, z);
  if (__all_sync(0xffffffffu, !active)) return;
  if (!active) {  // padding lanes follow the last cell of the row, inactive
    x = min(x, p.d.x - 1);
    y = min(y, p.d.y - 1);
  }
  mc_bwd1_at<C>(p, lk, x, y, z, active);
}

// ------------------------------------------- fwd-field bricks staged by TMA
// Forward 2 of one-channel data reads the fwd field at the back-traced position
// idx - lookup, a few cells from the cell itself.  Here a block takes a 32 x 8 x
// 4 tile of cells; one TMA copy brings the fwd field over the tile and kHalo
// cells around it (a 40 x 16 x 12 brick, zeros outside the grid) into shared
// memory, and the eight corners of every trace that stays in the brick are read
// there -- traces of lookups of kHalo cells or more, and wrapped indices, read
// global memory as before.  The values and the arithmetic are those of the
// global-memory kernel, so the results are the same bits.  (Backward 1 reads the
// same corners but measured faster from global memory: its registers leave it
// four resident bricked blocks per SM against five unbricked.)  The block's
// wait for its brick is bounded by ``polls``; if it gives up, it counts the event
// in g_wait_timeouts, reads global memory for every corner and waits (bounded by
// kBrickWaitPolls) for the copy before it leaves, so no copy outlives its block.
constexpr int kBrickWaitPolls = 1 << 22;
__device__ unsigned long long g_wait_timeouts;

// 30 KB of brick per block leave room for seven blocks per SM; the registers are
// held to those of five (48).
template <int C, class T, class LK>
__global__ void __launch_bounds__(kTileX * kTileY, 5)
    k_mc_fwd2_brick(McParams<T> p, LK lk, const __grid_constant__ CUtensorMap tmap, int polls) {
  __shared__ alignas(128) float brick[kBrickZ * kBrickY * kBrickX];
  __shared__ alignas(8) uint64_t bar;
  const int tid = threadIdx.y * kTileX + threadIdx.x;
  const int x0 = int(blockIdx.x) * kTileX, y0 = int(blockIdx.y) * kTileY, z0 = int(blockIdx.z) * kTileZ;
  if (tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(&bar, unsigned(sizeof(brick)));
    tma_load_3d(brick, &tmap, x0 - kHalo, y0 - kHalo, z0 - kHalo, &bar);
  }
  const bool ok = mbar_wait_bounded(&bar, 0, polls);
  if (!ok && tid == 0) atomicAdd(&g_wait_timeouts, 1ull);
  const BrickFetch fe{brick, x0 - kHalo, y0 - kHalo, z0 - kHalo, ok};
  const int x = x0 + int(threadIdx.x), y = y0 + int(threadIdx.y);
  if (x < p.d.x && y < p.d.y) {
    for (int k = 0; k < kTileZ; ++k) {
      const int z = z0 + k;
      if (z >= p.d.z) break;
      mc_fwd2_at<C>(p, lk, x, y, z, fe);
    }
  }
  if (!ok) mbar_wait_bounded(&bar, 0, kBrickWaitPolls);  // the copy may still be landing in the brick
}

// sample sources of the deterministic (fixed-point) adjoint: the back-trace
// (value gback at idx - lut) and the forward trace (value gfwd at idx + lut)
template <int C, class T, class LK>
struct TraceSource {
  const CT<T>* val;
  LK lk;
  Dims d;
  int sign;  // +1 forward trace, -1 back-trace
  __device__ __forceinline__ bool operator()(int64_t s, CT<T> pos[3], CT<T> g[C]) const {
    typedef CT<T> S;
    int x, y, z;
    cell_of(s, d, x, y, z);
    S lut[3];
    lk(x, y, z, lut);
    const S sg = S(sign);
    pos[0] = add_rn(sg * lut[0], S(x));
    pos[1] = add_rn(sg * lut[1], S(y));
    pos[2] = add_rn(sg * lut[2], S(z));
#pragma unroll
    for (int c = 0; c < C; ++c) g[c] = val[s * C + c];
    return true;
  }
};

// add a normalised buffered scatter (reference mode) and clear the buffer
template <int C, class S>
__global__ void k_norm_add(S* __restrict__ target, S* __restrict__ buf, unsigned* __restrict__ cnt, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned k = cnt[i];
  if (k > 0) {
    const S w = S(1) / S(k);
#pragma unroll
    for (int c = 0; c < C; ++c) atomic_add(target + i * C + c, buf[i * C + c] * w);
  }
#pragma unroll
  for (int c = 0; c < C; ++c) buf[i * C + c] = S(0);
  cnt[i] = 0u;
}

// backward 2: forward-trace adjoint into the data gradient.  With gface set
// (density lookup centred(u) * (-dt)) the lookup gradient goes straight to the
// two faces of the cell along each axis (half each, times -dt).
// (x, y, z) is a cell of the grid; inactive lanes (padding, clamped onto the
// row's last cell) take part in the warp-merged scatter only.
template <int C, class T, class LK>
__device__ __forceinline__ void mc_bwd2_at(const McParams<T>& p, const LK& lk, int x, int y, int z, bool active) {
  typedef CT<T> S;
  const int64_t i = flat(x, y, z, p.d);
  S lut[3];
  lk(x, y, z, lut);
  const S p1x = add_rn(lut[0], S(x)), p1y = add_rn(lut[1], S(y)), p1z = add_rn(lut[2], S(z));
  S g[C];
#pragma unroll
  for (int c = 0; c < C; ++c) g[c] = p.gfwd[i * C + c];
  const Tri<S> t = tri_setup(p1x, p1y, p1z, p.d, p.bm);
  if (p.det) {
  } else if (p.reference) {
    if (active) scatter_linear_counted<C>(p.buf, p.cnt, p1x, p1y, p1z, p.d, p.bm, g);
  } else {
    scatter_linear_warp<C>(p.gdata, t, p.d, p.bm, g, active);
  }
  S gl[3] = {S(0), S(0), S(0)};
  if (active) {
    gl[0] = p.glut[i * 3 + 0];
    gl[1] = p.glut[i * 3 + 1];
    gl[2] = p.glut[i * 3 + 2];
  }
  if (active && !(p.bm == BORDER && !t.inside)) {
    S v[8][C], dx[C], dy[C], dz[C];
    tri_fetch<C>(p.data, t, p.d, v);
    tri_gradient<C>(v, t, dx, dy, dz);
    // pos1 = idx + lut
#pragma unroll
    for (int c = 0; c < C; ++c) {
      gl[0] += g[c] * dx[c];
      gl[1] += g[c] * dy[c];
      gl[2] += g[c] * dz[c];
    }
  }
  if (p.gface[0]) {
    const S h = S(-0.5) * S(p.dt);
    const S gx = gl[0] * h, gy = gl[1] * h, gz = gl[2] * h;
    // x faces: face x gets this cell's and the previous cell's share; lanes hold
    // consecutive cells of one row, so the previous lane's share comes by shuffle
    // and only the first lane of the warp and the row's last cell add to a second face
    const int lane = threadIdx.x & 31;
    const S gprev = __shfl_up_sync(0xffffffffu, gx, 1);
    const bool merged = lane > 0;  // padding lanes carry gx = 0 (gl = 0)
    if (!active) return;
    S* fx = p.gface[0] + (int64_t(z) * p.d.y + y) * (p.d.x + 1) + x;
    S* fy = p.gface[1] + (int64_t(z) * (p.d.y + 1) + y) * p.d.x + x;
    S* fz = p.gface[2] + (int64_t(z) * p.d.y + y) * p.d.x + x;
    atomic_add(fx, merged ? gx + gprev : gx);
    if (lane == 31 || x == p.d.x - 1) atomic_add(fx + 1, gx);
    atomic_add(fy, gy);
    atomic_add(fy + p.d.x, gy);
    atomic_add(fz, gz);
    atomic_add(fz + int64_t(p.d.x) * p.d.y, gz);
    return;
  }
  if (!active) return;
  p.glut[i * 3 + 0] = gl[0];
  p.glut[i * 3 + 1] = gl[1];
  p.glut[i * 3 + 2] = gl[2];
}

template <int C, class T, class LK>
__global__ void __launch_bounds__(kBlock, (mc_narrow16<C, T, LK>() ? 5 : 0)) k_mc_bwd2(McParams<T> p, LK lk) {
  int x, y, z;
  const bool active = launch_cell(p.d, x, y, z);
  if (__all_sync(0xffffffffu, !active)) return;
  if (!active) {  // padding lanes follow the last cell of the row, inactive
    x = min(x, p.d.x - 1);
    y = min(y, p.d.y - 1);
  }
  mc_bwd2_at<C>(p, lk, x, y, z, active);
}

// density backward 3: d u_c = -dt * d lut; each face receives half of its two cells
template <class S>
__global__ void __launch_bounds__(kBlock) k_centered_faces(const S* __restrict__ glut, S* __restrict__ gx,
                                                           S* __restrict__ gy, S* __restrict__ gz, Dims d, float dt) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nx = int64_t(d.x + 1) * d.y * d.z;
  const int64_t ny = int64_t(d.x) * (d.y + 1) * d.z;
  const int64_t nz = int64_t(d.x) * d.y * (d.z + 1);
  const S h = S(-0.5) * S(dt);
  if (i < nx) {
    const int x = int(i % (d.x + 1)), y = int((i / (d.x + 1)) % d.y), z = int(i / (int64_t(d.x + 1) * d.y));
    S s = S(0);
    if (x > 0) s += glut[flat(x - 1, y, z, d) * 3 + 0] * h;
    if (x < d.x) s += glut[flat(x, y, z, d) * 3 + 0] * h;
    gx[i] = s;
  } else if (i < nx + ny) {
    const int64_t j = i - nx;
    const int x = int(j % d.x), y = int((j / d.x) % (d.y + 1)), z = int(j / (int64_t(d.x) * (d.y + 1)));
    S s = S(0);
    if (y > 0) s += glut[flat(x, y - 1, z, d) * 3 + 1] * h;
    if (y < d.y) s += glut[flat(x, y, z, d) * 3 + 1] * h;
    gy[j] = s;
  } else if (i < nx + ny + nz) {
    const int64_t j = i - nx - ny;
    const int x = int(j % d.x), y = int((j / d.x) % d.y), z = int(j / (int64_t(d.x) * d.y));
    S s = S(0);
    if (z > 0) s += glut[flat(x, y, z - 1, d) * 3 + 2] * h;
    if (z < d.z) s += glut[flat(x, y, z, d) * 3 + 2] * h;
    gz[j] = s;
  }
}

// velocity backward 3 for component ``tgt``: the lookup channel of component s is
// (-u_s resampled on tgt's lattice) * dt; its gradient goes to u_s directly
// (s == tgt) or through the adjoint of the offset resample.
template <class S>
__global__ void __launch_bounds__(kBlock) k_face_lut_adjoint(const S* __restrict__ glut, S* gu0, S* gu1, S* gu2,
                                                             Dims cells, int tgt, int bm, float dt, int reference,
                                                             S* buf, unsigned* cnt) {
  const Dims d = face_dims(cells, tgt);
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= d.count()) return;
  int x, y, z;
  cell_of(i, d, x, y, z);
  S* gu[3] = {gu0, gu1, gu2};
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const S g = -(glut[i * 3 + s] * S(dt));
    if (s == tgt) {
      atomic_add(gu[s] + i, g);
    } else {
      const S gg[1] = {g};
      const S px = add_rn(S(comp_offset(s, tgt, 0)), S(x)), py = add_rn(S(comp_offset(s, tgt, 1)), S(y)),
              pz = add_rn(S(comp_offset(s, tgt, 2)), S(z));
      if (reference) {
        // one normalisation buffer per source component: buffers laid out back to back
        int64_t off = 0;
        for (int q = 0; q < s; ++q) off += face_dims(cells, q).count();
        scatter_linear_counted<1>(buf + off, cnt + off, px, py, pz, face_dims(cells, s), bm, gg);
      } else {
        scatter_linear<1>(gu[s], px, py, pz, face_dims(cells, s), bm, gg);
      }
    }
  }
}

// The exact lookup adjoint of all three components in gather form, for the
// faces of component s: the scatter of k_face_lut_adjoint reversed.  Component
// tgt's lookup resamples s at p = X + o with o = +1/2 along s, -1/2 along tgt and
// 0 along the third axis c (comp_offset): corners X_s, X_s + 1 and X_t - 1, X_t
// with weight 1/2 each, X_c with weight 1 (tri_setup; the ceil corner of the
// integer axis has weight 0).  Face F of s therefore gathers 1/4 of
// glut_tgt[X][s] from X_c = F_c, X_s in {F_s - 1, F_s} and the X_t whose t
// corners the boundary rule maps onto F_t -- X_t = F_t (its upper corner),
// X_t = F_t + 1 (its lower corner) and, at the edges, the clamped or wrapped
// corners; under BORDER the sample X_t = dims_t (outside: p + 1/2 = dims_t) and
// the lower corner of X_t = 0 drop out.  Plus the component's own lookup
// entry.  No atomics: one thread per face adds -dt times its sum to gu_s.
template <class S, int s>
__global__ void __launch_bounds__(kBlock) k_face_lut_gather(const S* __restrict__ glut0, const S* __restrict__ glut1,
                                                            const S* __restrict__ glut2, S* __restrict__ gus,
                                                            Dims cells, int bm, float dt) {
  const Dims d = face_dims(cells, s);
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= d.count()) return;
  int F[3];
  cell_of(i, d, F[0], F[1], F[2]);
  const S* glut[3] = {glut0, glut1, glut2};
  const int n[3] = {d.x, d.y, d.z};
  S acc = S(0);
#pragma unroll
  for (int tgt = 0; tgt < 3; ++tgt) {
    if (tgt == s) continue;
    const int c = 3 - s - tgt;
    const Dims T = face_dims(cells, tgt);
    const int nt = n[tgt];  // faces of s along tgt (tgt's lattice has nt + 1)
    // the X_t whose t corners land on F_t (at most four; both edge rules apply
    // to the one face of a single cell)
    int xt[4];
    int m = 0;
    const int ft = F[tgt];
    xt[m++] = ft;  // upper corner X_t = F_t (inside under BORDER: ft <= nt - 1)
    if (bm != BORDER || ft + 1 <= nt - 1) xt[m++] = ft + 1;  // lower corner X_t - 1 = F_t
    if (bm == CLAMP) {
      if (ft == 0) xt[m++] = 0;        // lower corner -1 clamps to 0
      if (ft == nt - 1) xt[m++] = nt;  // upper corner nt clamps to nt - 1
    } else if (bm == WRAP) {
      if (ft == nt - 1) xt[m++] = 0;  // lower corner -1 wraps to nt - 1
      if (ft == 0) xt[m++] = nt;      // upper corner nt wraps to 0
    }
    S part = S(0);
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const int xs = F[s] - 1 + ks;
      const int ns = s == 0 ? T.x : s == 1 ? T.y : T.z;
      if (xs < 0 || xs >= ns) continue;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (k >= m) break;
        int X[3];
        X[s] = xs;
        X[tgt] = xt[k];
        X[c] = F[c];
        part += glut[tgt][flat(X[0], X[1], X[2], T) * 3 + s];
      }
    }
    acc += S(0.25) * part;
  }
  acc += glut[s][i * 3 + s];
  gus[i] += -(acc * S(dt));
}

// ---------------------------------------------------- batched density warps
// Many grids of different sizes in one launch per phase: blockIdx.z runs over
// the concatenated z planes of all grids, blockIdx.x / y over the largest grid's
// rows (threads outside a grid's x / y extent are padding).
constexpr int kMaxAdvBatch = 32;

template <class T, class LK>
struct McBatch {
  McParams<T> item[kMaxAdvBatch];
  LK lk[kMaxAdvBatch];
  int block_end[kMaxAdvBatch];  // cumulative 32x8-cell blocks over the grids
  int nbx[kMaxAdvBatch];        // blocks per row of each grid
  int nby[kMaxAdvBatch];        // block rows per plane of each grid
  int count;
};

// One 32x8 block of cells of one grid per CUDA block, the grids' blocks back to
// back in a 1-D launch (no idle blocks for the smaller grids).
template <int C, class T, class LK, int PHASE>
__global__ void __launch_bounds__(kBlock) k_mc_batch(const __grid_constant__ McBatch<T, LK> bb) {
  int it = 0;
  const int w = int(blockIdx.x);
  while (it < bb.count - 1 && bb.block_end[it] <= w) ++it;
  const McParams<T>& p = bb.item[it];
  const int local = w - (it ? bb.block_end[it - 1] : 0);
  const int per_plane = bb.nbx[it] * bb.nby[it];
  const int z = local / per_plane, r = local - z * per_plane;
  const int by = r / bb.nbx[it], bx = r - by * bb.nbx[it];
  int x = bx * 32 + int(threadIdx.x), y = by * 8 + int(threadIdx.y);
  const bool active = x < p.d.x && y < p.d.y;
  if (PHASE == 0) {
    if (active) mc_fwd1_at<C>(p, bb.lk[it], x, y, z);
  } else if (PHASE == 1) {
    if (active && p.order == 2) mc_fwd2_at<C>(p, bb.lk[it], x, y, z);
  } else {
    if (__all_sync(0xffffffffu, !active)) return;
    if (!active) {
      x = min(x, p.d.x - 1);
      y = min(y, p.d.y - 1);
    }
    if (PHASE == 2)
      mc_bwd1_at<C>(p, bb.lk[it], x, y, z, active);
    else
      mc_bwd2_at<C>(p, bb.lk[it], x, y, z, active);
  }
}

// ------------------------------------------------------------------ host side
size_t compute_size(int dtype) { return dtype == NGT_F64 ? 8 : 4; }

int validate_common(int dtype, const int64_t* dhw, int order, int clamp, int boundary) {
  if (!positive_shape(dhw, 3)) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: shapes must be positive");
  if ((dhw[0] + 1) * (dhw[1] + 1) * (dhw[2] + 1) >= (int64_t(1) << 31))
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect: grid too large");
  if (dhw[0] + 1 > 65535) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: depth above 65534 cells");
  if (order != 1 && order != 2) return fail(NGT_ERR_INVALID_ARGUMENT, "Unsupported warp order '%d'", order);
  if (clamp < NGT_CLAMP_NONE || clamp > NGT_CLAMP_NEGATIVE) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: invalid clamp");
  // MC_SMOOTH is MacCormack's limiter: with order 1 it has no effect, as in
  // VelocityGrid.warp (data_structures.py:1709-1734)
  if (boundary < NGT_BORDER || boundary > NGT_WRAP) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: invalid boundary");
  if (dtype < NGT_F32 || dtype > NGT_F16) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: invalid dtype");
  return NGT_OK;
}

int validate(const ngt_advect_args* a) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: null arguments");
  int rc = validate_common(a->dtype, a->grid_dhw, a->order, a->clamp, a->boundary);
  if (rc) return rc;
  if (!valid_channels(a->channels)) return fail(NGT_ERR_INVALID_ARGUMENT, "Only 1,2 and 4 Channel supported.");
  if (!a->data || !a->vel_x || !a->vel_y || !a->vel_z) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: null pointer");
  if (a->order == 2 && !a->fwd_field) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: MacCormack needs fwd_field");
  if (a->velocity_dtype != NGT_F32 && a->velocity_dtype != a->dtype &&
      !(a->dtype == NGT_BF16 && a->velocity_dtype == NGT_F16))
    return fail(NGT_ERR_UNSUPPORTED, "advect: faces stored apart from the data in FP16 go with BF16 data only");
  const int vt = a->velocity_dtype == NGT_F32 ? a->dtype : a->velocity_dtype;
  if ((rc = check_aligned("advect", storage_bytes(a->dtype), {{"data", a->data}, {"output", a->output}})) ||
      (rc = check_aligned("advect", storage_bytes(vt), {{"vel_x", a->vel_x}, {"vel_y", a->vel_y},
                                                        {"vel_z", a->vel_z}})))
    return rc;
  return check_aligned("advect", arith_bytes(a->dtype),
                       {{"fwd_field", a->fwd_field}, {"extrema", a->extrema}, {"lookup", a->lookup}});
}

Dims cells_of(const int64_t* dhw) { return Dims{int(dhw[2]), int(dhw[1]), int(dhw[0])}; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (null when the
// driver does not offer it: the brick kernels are then not used).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    cudaGetLastError();  // a failed lookup leaves no error behind for the launches
  });
  return fn;
}

// The tensor map of a one-channel float field of grid d for the brick kernels;
// false when the field does not qualify (a row of a multiple of 4 floats, so its
// rows and planes start on 16 bytes; a 16-byte aligned base) or no encoder.
bool brick_map(const float* f, const Dims& d, CUtensorMap& m) {
  if (d.x % 4 != 0 || (reinterpret_cast<uintptr_t>(f) & 15) != 0) return false;
  const EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t dims[3] = {cuuint64_t(d.x), cuuint64_t(d.y), cuuint64_t(d.z)};
  const cuuint64_t strides[2] = {cuuint64_t(d.x) * 4, cuuint64_t(d.x) * d.y * 4};
  const cuuint32_t box[3] = {kBrickX, kBrickY, kBrickZ};
  const cuuint32_t elem[3] = {1, 1, 1};
  return fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(f), dims, strides, box, elem,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

dim3 brick_grid(const Dims& d) {
  return dim3(ceil_div_u(d.x, kTileX), ceil_div_u(d.y, kTileY), ceil_div_u(d.z, kTileZ));
}

// first-wait poll limit of the bricked kernels (ngt_set_wait_polls)
std::atomic<int> g_wait_polls{kBrickWaitPolls};

// Forward 2: through fwd-field bricks for one channel of float or 16-bit density
// whose field qualifies, else the global-memory kernel.
template <int C, class T, class LK>
void launch_fwd2(const McParams<T>& p, const LK& lk, cudaStream_t st) {
  // (the velocity self-advection's face lookups keep the global-memory kernel)
  if constexpr (C == 1 && !std::is_same<T, double>::value && !std::is_same<LK, FaceLookup<T>>::value) {
    CUtensorMap m;
    if (brick_map(p.fwd, p.d, m)) {
      k_mc_fwd2_brick<C, T, LK><<<brick_grid(p.d), dim3(kTileX, kTileY), 0, st>>>(p, lk, m, g_wait_polls.load());
      return;
    }
  }
  const CellLaunch l = cell_launch(p.d);
  k_mc_fwd2<C, T, LK><<<l.grid, l.block, 0, st>>>(p, lk);
}

template <int C, class T, class LK>
void launch_fwd(const McParams<T>& p, const LK& lk, cudaStream_t st) {
  const CellLaunch l = cell_launch(p.d);
  k_mc_fwd1<C, T, LK><<<l.grid, l.block, 0, st>>>(p, lk);
  if (p.order == 2) launch_fwd2<C, T, LK>(p, lk, st);
}

// bwd 1 + 2 of one warp; leaves the lookup gradient in p.glut
template <int C, class T, class LK>
int launch_bwd12(McParams<T>& p, const LK& lk, cudaStream_t st) {
  typedef CT<T> S;
  const int64_t n = p.d.count();
  if (p.reference) {
    if (cudaMemsetAsync(p.buf, 0, size_t(n) * C * sizeof(S), st) != cudaSuccess ||
        cudaMemsetAsync(p.cnt, 0, size_t(n) * sizeof(unsigned), st) != cudaSuccess)
      return check_launch("advect_bwd memset");
  } else if (!p.det && cudaMemsetAsync(p.gfwd, 0, size_t(n) * C * sizeof(S), st) != cudaSuccess) {
    return check_launch("advect_bwd memset");
  }
  const unsigned nb = ceil_div_u(n, kBlock);
  const CellLaunch l = cell_launch(p.d);
  k_mc_bwd1<C, T, LK><<<l.grid, l.block, 0, st>>>(p, lk);
  if (p.det && p.order == 2 &&
      fixed_adjoint<C, S>(TraceSource<C, T, LK>{p.gback, lk, p.d, -1}, n, p.d, p.bm, p.cnt, p.gfwd, 1, st) !=
          cudaSuccess)
    return check_launch("advect_bwd memset");
  if (p.reference && p.order == 2) k_norm_add<C, S><<<nb, kBlock, 0, st>>>(p.gfwd, p.buf, p.cnt, n);
  k_mc_bwd2<C, T, LK><<<l.grid, l.block, 0, st>>>(p, lk);
  if (p.det &&
      fixed_adjoint<C, S>(TraceSource<C, T, LK>{p.gfwd, lk, p.d, +1}, n, p.d, p.bm, p.cnt, p.gdata, 1, st) !=
          cudaSuccess)
    return check_launch("advect_bwd memset");
  if (p.reference) k_norm_add<C, S><<<nb, kBlock, 0, st>>>(p.gdata, p.buf, p.cnt, n);
  return NGT_OK;
}

template <class T>
McParams<T> density_params(const ngt_advect_args* a) {
  McParams<T> p = {};
  p.data = static_cast<const T*>(a->data);
  p.out = static_cast<T*>(a->output);
  p.fwd = static_cast<CT<T>*>(a->fwd_field);
  p.mask = static_cast<uint8_t*>(a->mask);
  p.ext = static_cast<CT<T>*>(a->extrema);
  p.d = cells_of(a->grid_dhw);
  p.order = a->order;
  p.clamp = a->clamp;
  p.bm = a->boundary;
  return p;
}

// The faces' lookup; V is the faces' storage type (the data's, or FP16 faces with
// BF16 data), its arithmetic the data's (float).
template <class V>
CenteredLookup<V> centered(const ngt_advect_args* a) {
  return CenteredLookup<V>{static_cast<const V*>(a->vel_x), static_cast<const V*>(a->vel_y),
                           static_cast<const V*>(a->vel_z), cells_of(a->grid_dhw), a->dt};
}

template <int C, class T, class V = T>
int density_fwd(const ngt_advect_args* a, cudaStream_t st) {
  McParams<T> p = density_params<T>(a);
  if (!a->lookup) {
    launch_fwd<C, T>(p, centered<V>(a), st);
  } else {
    // forward 1 averages the faces once and stores the lookup; forward 2 reads it
    const CellLaunch l = cell_launch(p.d);
    p.lut_out = static_cast<CT<T>*>(a->lookup);
    k_mc_fwd1<C, T, CenteredLookup<V>><<<l.grid, l.block, 0, st>>>(p, centered<V>(a));
    p.lut_out = nullptr;
    if (p.order == 2)
      launch_fwd2<C, T, StoredLookup<T>>(p, StoredLookup<T>{static_cast<const CT<T>*>(a->lookup), p.d}, st);
  }
  return check_launch("ngt_advect_maccormack_fwd");
}

template <int C, class T, class V = T>
int density_bwd(const ngt_advect_grad_args* g, cudaStream_t st) {
  typedef CT<T> S;
  McParams<T> p = density_params<T>(&g->fwd);
  const int64_t n = p.d.count();
  p.gout = static_cast<const S*>(g->output_grad);
  p.gdata = static_cast<S*>(g->data_grad);
  p.reference = g->grad_mode == NGT_GRAD_REFERENCE;
  p.det = !p.reference && g->deterministic;
  p.accumulate = g->accumulate ? 1 : 0;
  char* w = static_cast<char*>(g->workspace);
  p.gfwd = reinterpret_cast<S*>(w);
  w += size_t(n) * C * sizeof(S);
  p.glut = reinterpret_cast<S*>(w);
  w += size_t(n) * 3 * sizeof(S);
  if (p.reference) {
    p.buf = reinterpret_cast<S*>(w);
    w += size_t(n) * C * sizeof(S);
    p.cnt = reinterpret_cast<unsigned*>(w);
  } else if (p.det) {
    p.gback = reinterpret_cast<S*>(w);
    w += size_t(n) * C * sizeof(S);
    // the fixed-point sums (64-bit: 8-byte aligned; the workspace size allows for it)
    w = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(w) + 15) & ~uintptr_t(15));
    p.cnt = reinterpret_cast<unsigned*>(w);
  }
  const bool faces = g->vel_x_grad && g->vel_y_grad && g->vel_z_grad;
  if (faces && !p.det) {
    // backward 1 clears the face gradients, backward 2 accumulates them
    p.gface[0] = static_cast<S*>(g->vel_x_grad);
    p.gface[1] = static_cast<S*>(g->vel_y_grad);
    p.gface[2] = static_cast<S*>(g->vel_z_grad);
    p.dt = g->fwd.dt;
  }
  int rc = g->fwd.lookup
               ? launch_bwd12<C, T>(p, StoredLookup<T>{static_cast<const CT<T>*>(g->fwd.lookup), p.d}, st)
               : launch_bwd12<C, T>(p, centered<V>(&g->fwd), st);
  if (rc) return rc;
  if (faces && p.det) {
    const Dims& d = p.d;
    const int64_t nf = int64_t(d.x + 1) * d.y * d.z + int64_t(d.x) * (d.y + 1) * d.z + int64_t(d.x) * d.y * (d.z + 1);
    k_centered_faces<S><<<ceil_div_u(nf, kBlock), kBlock, 0, st>>>(p.glut, static_cast<S*>(g->vel_x_grad),
                                                                    static_cast<S*>(g->vel_y_grad),
                                                                    static_cast<S*>(g->vel_z_grad), d, g->fwd.dt);
  }
  return check_launch("ngt_advect_maccormack_bwd");
}

template <class T, class V = T>
int density_fwd_c(const ngt_advect_args* a, cudaStream_t st) {
  switch (a->channels) {
    case 1: return density_fwd<1, T, V>(a, st);
    case 2: return density_fwd<2, T, V>(a, st);
    default: return density_fwd<4, T, V>(a, st);
  }
}

template <class T, class V = T>
int density_bwd_c(const ngt_advect_grad_args* g, cudaStream_t st) {
  switch (g->fwd.channels) {
    case 1: return density_bwd<1, T, V>(g, st);
    case 2: return density_bwd<2, T, V>(g, st);
    default: return density_bwd<4, T, V>(g, st);
  }
}

// FP16 faces with BF16 data: the one mixed storage the density warp takes.
bool mixed_faces(const ngt_advect_args* a) {
  return a->velocity_dtype != NGT_F32 && a->velocity_dtype != a->dtype;
}

// ----------------------------------------------------------- velocity warp
int validate_vel(const ngt_advect_velocity_args* a) {
  if (!a) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_velocity: null arguments");
  int rc = validate_common(a->dtype, a->grid_dhw, a->order, a->clamp, a->boundary);
  if (rc) return rc;
  if (!a->vel_x || !a->vel_y || !a->vel_z) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_velocity: null pointer");
  if (a->order == 2 && (!a->fwd_x || !a->fwd_y || !a->fwd_z))
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect_velocity: MacCormack needs the fwd fields");
  if ((rc = check_aligned("advect_velocity", storage_bytes(a->dtype),
                          {{"vel_x", a->vel_x}, {"vel_y", a->vel_y}, {"vel_z", a->vel_z}, {"out_x", a->out_x},
                           {"out_y", a->out_y}, {"out_z", a->out_z}})))
    return rc;
  return check_aligned("advect_velocity", arith_bytes(a->dtype),
                       {{"fwd_x", a->fwd_x}, {"fwd_y", a->fwd_y}, {"fwd_z", a->fwd_z}, {"lookup[0]", a->lookup[0]},
                        {"lookup[1]", a->lookup[1]}, {"lookup[2]", a->lookup[2]}, {"extrema[0]", a->extrema[0]},
                        {"extrema[1]", a->extrema[1]}, {"extrema[2]", a->extrema[2]}});
}

template <class T>
FaceLookup<T> face_lookup(const ngt_advect_velocity_args* a, int tgt) {
  FaceLookup<T> lk;
  lk.u[0] = static_cast<const T*>(a->vel_x);
  lk.u[1] = static_cast<const T*>(a->vel_y);
  lk.u[2] = static_cast<const T*>(a->vel_z);
  lk.cells = cells_of(a->grid_dhw);
  lk.tgt = tgt;
  lk.bm = a->boundary;
  lk.dt = a->dt;
  return lk;
}

template <class T>
McParams<T> vel_params(const ngt_advect_velocity_args* a, int comp) {
  const void* data[3] = {a->vel_x, a->vel_y, a->vel_z};
  void* out[3] = {a->out_x, a->out_y, a->out_z};
  void* fwd[3] = {a->fwd_x, a->fwd_y, a->fwd_z};
  McParams<T> p = {};
  p.data = static_cast<const T*>(data[comp]);
  p.out = static_cast<T*>(out[comp]);
  p.fwd = static_cast<CT<T>*>(fwd[comp]);
  p.mask = static_cast<uint8_t*>(a->mask[comp]);
  p.ext = static_cast<CT<T>*>(a->extrema[comp]);
  p.d = face_dims(cells_of(a->grid_dhw), comp);
  p.order = a->order;
  p.clamp = a->clamp;
  p.bm = a->boundary;
  return p;
}

template <class T>
int vel_fwd(const ngt_advect_velocity_args* a, cudaStream_t st) {
  for (int c = 0; c < 3; ++c) {
    McParams<T> p = vel_params<T>(a, c);
    if (!a->lookup[c]) {
      launch_fwd<1, T>(p, face_lookup<T>(a, c), st);
      continue;
    }
    // forward 1 resamples the lookup once and stores it; forward 2 reads it
    const CellLaunch l = cell_launch(p.d);
    p.lut_out = static_cast<CT<T>*>(a->lookup[c]);
    k_mc_fwd1<1, T, FaceLookup<T>><<<l.grid, l.block, 0, st>>>(p, face_lookup<T>(a, c));
    p.lut_out = nullptr;
    if (p.order == 2)
      k_mc_fwd2<1, T, StoredLookup<T>><<<l.grid, l.block, 0, st>>>(
          p, StoredLookup<T>{static_cast<const CT<T>*>(a->lookup[c]), p.d});
  }
  return check_launch("ngt_advect_velocity_fwd");
}

int64_t max_faces(const int64_t* dhw) {
  const Dims c = cells_of(dhw);
  int64_t m = 0;
  for (int k = 0; k < 3; ++k) m = face_dims(c, k).count() > m ? face_dims(c, k).count() : m;
  return m;
}

int64_t all_faces(const int64_t* dhw) {
  const Dims c = cells_of(dhw);
  return face_dims(c, 0).count() + face_dims(c, 1).count() + face_dims(c, 2).count();
}

template <class T>
int vel_bwd(const ngt_advect_velocity_grad_args* g, cudaStream_t st) {
  typedef CT<T> S;
  const ngt_advect_velocity_args* a = &g->fwd;
  const Dims cells = cells_of(a->grid_dhw);
  const int reference = g->grad_mode == NGT_GRAD_REFERENCE;
  const int det = !reference && g->deterministic;
  const int64_t nmax = max_faces(a->grid_dhw), nall = all_faces(a->grid_dhw);
  char* w = static_cast<char*>(g->workspace);
  S* gfwd = reinterpret_cast<S*>(w);
  w += size_t(nmax) * sizeof(S);
  // the exact gradient keeps every component's lookup gradient for the gather
  S* gluts[3];
  for (int c = 0; c < 3; ++c) {
    gluts[c] = reinterpret_cast<S*>(w);
    if (!reference || c == 2) w += size_t(nmax) * 3 * sizeof(S);
  }
  S* glut = gluts[0];
  S* buf = nullptr;
  unsigned* cnt = nullptr;
  S* gback = nullptr;
  if (reference) {
    buf = reinterpret_cast<S*>(w);
    w += size_t(nall) * sizeof(S);
    cnt = reinterpret_cast<unsigned*>(w);
  } else if (det) {
    // the back-trace gradient, then the fixed-point sums (8-byte aligned)
    gback = reinterpret_cast<S*>(w);
    w += size_t(nmax) * sizeof(S);
    w = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(w) + 15) & ~uintptr_t(15));
    cnt = reinterpret_cast<unsigned*>(w);
  }
  S* gu[3] = {static_cast<S*>(g->vel_x_grad), static_cast<S*>(g->vel_y_grad), static_cast<S*>(g->vel_z_grad)};
  const void* go[3] = {g->grad_x, g->grad_y, g->grad_z};
  for (int c = 0; c < 3; ++c)
    if (cudaMemsetAsync(gu[c], 0, size_t(face_dims(cells, c).count()) * sizeof(S), st) != cudaSuccess)
      return check_launch("advect_velocity_bwd memset");
  for (int c = 0; c < 3; ++c) {
    McParams<T> p = vel_params<T>(a, c);
    p.gout = static_cast<const S*>(go[c]);
    p.gdata = gu[c];
    p.gfwd = gfwd;
    p.glut = reference ? glut : gluts[c];
    p.reference = reference;
    p.det = det;
    p.gback = gback;
    p.buf = buf;
    p.cnt = cnt;
    // added to the zeroed face gradients (the lookup adjoint adds the rest); in the
    // deterministic mode each cell's direct term is its only addition there before
    // the fixed-point sums, so the result does not depend on any order
    p.accumulate = 1;
    int rc = a->lookup[c]
                 ? launch_bwd12<1, T>(p, StoredLookup<T>{static_cast<const CT<T>*>(a->lookup[c]), p.d}, st)
                 : launch_bwd12<1, T>(p, face_lookup<T>(a, c), st);
    if (rc) return rc;
    if (!reference) continue;  // the exact lookup adjoint gathers once every component's is there
    if (cudaMemsetAsync(buf, 0, size_t(nall) * sizeof(S), st) != cudaSuccess ||
        cudaMemsetAsync(cnt, 0, size_t(nall) * sizeof(unsigned), st) != cudaSuccess)
      return check_launch("advect_velocity_bwd memset");
    k_face_lut_adjoint<S><<<ceil_div_u(p.d.count(), kBlock), kBlock, 0, st>>>(glut, gu[0], gu[1], gu[2], cells, c,
                                                                               a->boundary, a->dt, reference, buf, cnt);
    if (reference) {
      int64_t off = 0;
      for (int s = 0; s < 3; ++s) {
        const int64_t ns = face_dims(cells, s).count();
        if (s != c) k_norm_add<1, S><<<ceil_div_u(ns, kBlock), kBlock, 0, st>>>(gu[s], buf + off, cnt + off, ns);
        off += ns;
      }
    }
  }
  if (!reference) {
    const unsigned b0 = ceil_div_u(face_dims(cells, 0).count(), kBlock);
    const unsigned b1 = ceil_div_u(face_dims(cells, 1).count(), kBlock);
    const unsigned b2 = ceil_div_u(face_dims(cells, 2).count(), kBlock);
    k_face_lut_gather<S, 0><<<b0, kBlock, 0, st>>>(gluts[0], gluts[1], gluts[2], gu[0], cells, a->boundary, a->dt);
    k_face_lut_gather<S, 1><<<b1, kBlock, 0, st>>>(gluts[0], gluts[1], gluts[2], gu[1], cells, a->boundary, a->dt);
    k_face_lut_gather<S, 2><<<b2, kBlock, 0, st>>>(gluts[0], gluts[1], gluts[2], gu[2], cells, a->boundary, a->dt);
  }
  return check_launch("ngt_advect_velocity_bwd");
}

template <class F>
int by_dtype(int dtype, F&& f);

// ------------------------------------------------------------ batched warps
int validate_batch(const ngt_advect_args* const* a, int count, int& zsum, int& maxw, int& maxh) {
  if (count < 1 || count > kMaxAdvBatch)
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch: 1 to %d grids", kMaxAdvBatch);
  zsum = maxw = maxh = 0;
  int64_t blocks = 0;
  for (int i = 0; i < count; ++i) {
    const int rc = validate(a[i]);
    if (rc) return rc;
    if (!a[i]->output) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: null output");
    if (a[i]->dtype != a[0]->dtype || a[i]->channels != a[0]->channels)
      return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch: grids must share dtype and channels");
    if (mixed_faces(a[i])) return fail(NGT_ERR_UNSUPPORTED, "advect batch: faces in the data's storage type");
    blocks += ((a[i]->grid_dhw[2] + 31) / 32) * ((a[i]->grid_dhw[1] + 7) / 8) * a[i]->grid_dhw[0];
  }
  if (blocks >= (int64_t(1) << 31)) return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch: grids too large");
  return NGT_OK;
}

// Fills the 1-D block table of a batch; returns the number of blocks.
template <class T, class LK>
int block_table(McBatch<T, LK>& bb) {
  int total = 0;
  for (int k = 0; k < bb.count; ++k) {
    const Dims& d = bb.item[k].d;
    bb.nbx[k] = (d.x + 31) / 32;
    bb.nby[k] = (d.y + 7) / 8;
    total += bb.nbx[k] * bb.nby[k] * d.z;
    bb.block_end[k] = total;
  }
  return total;
}

template <int C, class T>
int density_fwd_batch(const ngt_advect_args* const* a, int count, int zsum, int maxw, int maxh, cudaStream_t st) {
  McBatch<T, CenteredLookup<T>> bb{};
  bb.count = count;
  bool mc = false;
  for (int k = 0; k < count; ++k) {
    bb.item[k] = density_params<T>(a[k]);
    bb.lk[k] = centered<T>(a[k]);
    mc = mc || a[k]->order == 2;
  }
  const dim3 grid(unsigned(block_table(bb))), block(32, 8);
  k_mc_batch<C, T, CenteredLookup<T>, 0><<<grid, block, 0, st>>>(bb);
  if (mc) k_mc_batch<C, T, CenteredLookup<T>, 1><<<grid, block, 0, st>>>(bb);
  return check_launch("ngt_advect_maccormack_fwd_batch");
}

// Workspace of a batched backward: [gfwd of every grid][glut of every grid].
size_t batch_bwd_bytes(const ngt_advect_grad_args* g, int count) {
  size_t n = 0, m = 0;
  for (int k = 0; k < count; ++k) {
    const int64_t cells = g[k].fwd.grid_dhw[0] * g[k].fwd.grid_dhw[1] * g[k].fwd.grid_dhw[2];
    const size_t cs = compute_size(g[k].fwd.dtype);
    n += size_t(cells) * size_t(g[k].fwd.channels) * cs;
    m += size_t(cells) * 3 * cs;
  }
  return n + m;
}

template <int C, class T>
int density_bwd_batch(const ngt_advect_grad_args* g, int count, int zsum, int maxw, int maxh, void* ws,
                      cudaStream_t st) {
  typedef CT<T> S;
  McBatch<T, CenteredLookup<T>> bb{};
  bb.count = count;
  size_t gfwd_bytes = 0;
  for (int k = 0; k < count; ++k)
    gfwd_bytes += size_t(g[k].fwd.grid_dhw[0] * g[k].fwd.grid_dhw[1] * g[k].fwd.grid_dhw[2]) * C * sizeof(S);
  char* wf = static_cast<char*>(ws);
  char* wl = wf + gfwd_bytes;
  for (int k = 0; k < count; ++k) {
    McParams<T> p = density_params<T>(&g[k].fwd);
    const int64_t n = p.d.count();
    p.gout = static_cast<const S*>(g[k].output_grad);
    p.gdata = static_cast<S*>(g[k].data_grad);
    p.gfwd = reinterpret_cast<S*>(wf);
    wf += size_t(n) * C * sizeof(S);
    p.glut = reinterpret_cast<S*>(wl);
    wl += size_t(n) * 3 * sizeof(S);
    p.gface[0] = static_cast<S*>(g[k].vel_x_grad);
    p.gface[1] = static_cast<S*>(g[k].vel_y_grad);
    p.gface[2] = static_cast<S*>(g[k].vel_z_grad);
    p.dt = g[k].fwd.dt;
    bb.item[k] = p;
    bb.lk[k] = centered<T>(&g[k].fwd);
  }
  if (cudaMemsetAsync(ws, 0, gfwd_bytes, st) != cudaSuccess) return check_launch("advect batch memset");
  const dim3 grid(unsigned(block_table(bb))), block(32, 8);
  k_mc_batch<C, T, CenteredLookup<T>, 2><<<grid, block, 0, st>>>(bb);
  k_mc_batch<C, T, CenteredLookup<T>, 3><<<grid, block, 0, st>>>(bb);
  return check_launch("ngt_advect_maccormack_bwd_batch");
}

template <class T>
int batch_fwd_c(const ngt_advect_args* const* a, int count, int zsum, int mw, int mh, cudaStream_t st) {
  switch (a[0]->channels) {
    case 1: return density_fwd_batch<1, T>(a, count, zsum, mw, mh, st);
    case 2: return density_fwd_batch<2, T>(a, count, zsum, mw, mh, st);
    default: return density_fwd_batch<4, T>(a, count, zsum, mw, mh, st);
  }
}

template <class T>
int batch_bwd_c(const ngt_advect_grad_args* g, int count, int zsum, int mw, int mh, void* ws, cudaStream_t st) {
  switch (g[0].fwd.channels) {
    case 1: return density_bwd_batch<1, T>(g, count, zsum, mw, mh, ws, st);
    case 2: return density_bwd_batch<2, T>(g, count, zsum, mw, mh, ws, st);
    default: return density_bwd_batch<4, T>(g, count, zsum, mw, mh, ws, st);
  }
}

}  // namespace
}  // namespace ngt

using namespace ngt;

extern "C" int ngt_wait_timeouts(uint64_t* count, int32_t reset) {
  if (!count) return fail(NGT_ERR_INVALID_ARGUMENT, "ngt_wait_timeouts: count is null");
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_wait_timeouts, sizeof(v)) != cudaSuccess) return check_launch("ngt_wait_timeouts");
  if (reset) {
    const unsigned long long zero = 0;
    if (cudaMemcpyToSymbol(g_wait_timeouts, &zero, sizeof(zero)) != cudaSuccess) return check_launch("ngt_wait_timeouts");
  }
  *count = uint64_t(v);
  return NGT_OK;
}

extern "C" int32_t ngt_set_wait_polls(int32_t polls) {
  return g_wait_polls.exchange(polls < 0 ? kBrickWaitPolls : int(polls));
}

extern "C" int ngt_advect_maccormack_fwd(const ngt_advect_args* a, void* stream) {
  int rc = validate(a);
  if (rc) return rc;
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "advect: null output");
  cudaStream_t st = as_stream(stream);
  if (mixed_faces(a)) return density_fwd_c<__nv_bfloat16, __half>(a, st);
  switch (a->dtype) {
    case NGT_F32: return density_fwd_c<float>(a, st);
    case NGT_F64: return density_fwd_c<double>(a, st);
    case NGT_BF16: return density_fwd_c<__nv_bfloat16>(a, st);
    default: return density_fwd_c<__half>(a, st);
  }
}

extern "C" size_t ngt_advect_maccormack_bwd_workspace_bytes(const ngt_advect_grad_args* g) {
  if (!g) return 0;
  const int64_t n = g->fwd.grid_dhw[0] * g->fwd.grid_dhw[1] * g->fwd.grid_dhw[2];
  const int64_t C = g->fwd.channels;
  const size_t cs = compute_size(g->fwd.dtype);
  size_t bytes = size_t(n) * size_t(C + 3) * cs;
  if (g->grad_mode == NGT_GRAD_REFERENCE) bytes += size_t(n) * (size_t(C) * cs + sizeof(unsigned));
  else if (g->deterministic)
    bytes += size_t(n) * size_t(C) * cs + fixed_bytes(cells_of(g->fwd.grid_dhw), int(C)) + 16;
  return bytes;
}

extern "C" int ngt_advect_maccormack_bwd(const ngt_advect_grad_args* g, void* stream) {
  if (!g) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_bwd: null arguments");
  int rc = validate(&g->fwd);
  if (rc) return rc;
  if (!g->output_grad || !g->data_grad) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_bwd: null pointer");
  if (g->grad_mode != NGT_GRAD_EXACT && g->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect_bwd: invalid grad_mode");
  if (g->accumulate && (g->grad_mode != NGT_GRAD_EXACT || g->deterministic))
    return fail(NGT_ERR_UNSUPPORTED, "advect_bwd: accumulate needs the exact, non-deterministic gradient");
  if ((rc = check_aligned("advect_bwd", arith_bytes(g->fwd.dtype),
                          {{"output_grad", g->output_grad}, {"data_grad", g->data_grad},
                           {"vel_x_grad", g->vel_x_grad}, {"vel_y_grad", g->vel_y_grad},
                           {"vel_z_grad", g->vel_z_grad}})) ||
      (rc = check_aligned("advect_bwd", kScratchAlign, {{"workspace", g->workspace}})))
    return rc;
  const size_t need = ngt_advect_maccormack_bwd_workspace_bytes(g);
  if (!g->workspace || g->workspace_bytes < need)
    return fail(NGT_ERR_WORKSPACE, "advect_bwd needs %zu workspace bytes", need);
  cudaStream_t st = as_stream(stream);
  if (mixed_faces(&g->fwd)) return density_bwd_c<__nv_bfloat16, __half>(g, st);
  switch (g->fwd.dtype) {
    case NGT_F32: return density_bwd_c<float>(g, st);
    case NGT_F64: return density_bwd_c<double>(g, st);
    case NGT_BF16: return density_bwd_c<__nv_bfloat16>(g, st);
    default: return density_bwd_c<__half>(g, st);
  }
}

extern "C" int ngt_advect_velocity_fwd(const ngt_advect_velocity_args* a, void* stream) {
  int rc = validate_vel(a);
  if (rc) return rc;
  if (!a->out_x || !a->out_y || !a->out_z) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_velocity: null output");
  cudaStream_t st = as_stream(stream);
  switch (a->dtype) {
    case NGT_F32: return vel_fwd<float>(a, st);
    case NGT_F64: return vel_fwd<double>(a, st);
    case NGT_BF16: return vel_fwd<__nv_bfloat16>(a, st);
    default: return vel_fwd<__half>(a, st);
  }
}

extern "C" size_t ngt_advect_velocity_bwd_workspace_bytes(const ngt_advect_velocity_grad_args* g) {
  if (!g) return 0;
  const size_t cs = compute_size(g->fwd.dtype);
  // fwd-field gradient, lookup gradients (every component's for the exact gather, one for the reference scatter)
  const bool reference = g->grad_mode == NGT_GRAD_REFERENCE;
  size_t bytes = size_t(max_faces(g->fwd.grid_dhw)) * (reference ? 4 : 10) * cs;
  if (reference) bytes += size_t(all_faces(g->fwd.grid_dhw)) * (cs + sizeof(unsigned));
  else if (g->deterministic)  // back-trace gradient and the fixed-point sums of the largest component lattice
    bytes += size_t(max_faces(g->fwd.grid_dhw)) * (cs + 8) + 256 + 16;
  return bytes;
}

extern "C" int ngt_advect_velocity_bwd(const ngt_advect_velocity_grad_args* g, void* stream) {
  if (!g) return fail(NGT_ERR_INVALID_ARGUMENT, "advect_velocity_bwd: null arguments");
  int rc = validate_vel(&g->fwd);
  if (rc) return rc;
  if (!g->grad_x || !g->grad_y || !g->grad_z || !g->vel_x_grad || !g->vel_y_grad || !g->vel_z_grad)
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect_velocity_bwd: null pointer");
  if (g->grad_mode != NGT_GRAD_EXACT && g->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "advect_velocity_bwd: invalid grad_mode");
  if ((rc = check_aligned("advect_velocity_bwd", arith_bytes(g->fwd.dtype),
                          {{"grad_x", g->grad_x}, {"grad_y", g->grad_y}, {"grad_z", g->grad_z},
                           {"vel_x_grad", g->vel_x_grad}, {"vel_y_grad", g->vel_y_grad},
                           {"vel_z_grad", g->vel_z_grad}})) ||
      (rc = check_aligned("advect_velocity_bwd", kScratchAlign, {{"workspace", g->workspace}})))
    return rc;
  const size_t need = ngt_advect_velocity_bwd_workspace_bytes(g);
  if (!g->workspace || g->workspace_bytes < need)
    return fail(NGT_ERR_WORKSPACE, "advect_velocity_bwd needs %zu workspace bytes", need);
  cudaStream_t st = as_stream(stream);
  switch (g->fwd.dtype) {
    case NGT_F32: return vel_bwd<float>(g, st);
    case NGT_F64: return vel_bwd<double>(g, st);
    case NGT_BF16: return vel_bwd<__nv_bfloat16>(g, st);
    default: return vel_bwd<__half>(g, st);
  }
}

extern "C" int ngt_advect_maccormack_fwd_batch(const ngt_advect_args* items, int32_t count, void* stream) {
  if (!items) return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch: null grids");
  const ngt_advect_args* a[kMaxAdvBatch];
  if (count < 1 || count > kMaxAdvBatch) return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch: 1 to %d grids", kMaxAdvBatch);
  for (int i = 0; i < count; ++i) a[i] = items + i;
  int zsum, mw, mh;
  const int rc = validate_batch(a, count, zsum, mw, mh);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  switch (items[0].dtype) {
    case NGT_F32: return batch_fwd_c<float>(a, count, zsum, mw, mh, st);
    case NGT_F64: return batch_fwd_c<double>(a, count, zsum, mw, mh, st);
    case NGT_BF16: return batch_fwd_c<__nv_bfloat16>(a, count, zsum, mw, mh, st);
    default: return batch_fwd_c<__half>(a, count, zsum, mw, mh, st);
  }
}

extern "C" size_t ngt_advect_maccormack_bwd_batch_workspace_bytes(const ngt_advect_grad_args* items, int32_t count) {
  return (items && count > 0 && count <= kMaxAdvBatch) ? batch_bwd_bytes(items, count) : 0;
}

extern "C" int ngt_advect_maccormack_bwd_batch(const ngt_advect_grad_args* items, int32_t count, void* workspace,
                                               size_t workspace_bytes, void* stream) {
  if (!items) return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch: null grids");
  if (count < 1 || count > kMaxAdvBatch) return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch: 1 to %d grids", kMaxAdvBatch);
  const ngt_advect_args* a[kMaxAdvBatch];
  for (int i = 0; i < count; ++i) {
    const ngt_advect_grad_args& g = items[i];
    a[i] = &g.fwd;
    if (!g.output_grad || !g.data_grad || !g.vel_x_grad || !g.vel_y_grad || !g.vel_z_grad)
      return fail(NGT_ERR_INVALID_ARGUMENT, "advect batch backward: null pointer");
    if (g.grad_mode != NGT_GRAD_EXACT || g.deterministic || g.accumulate)
      return fail(NGT_ERR_UNSUPPORTED, "advect batch backward: exact, non-deterministic, written gradients only");
    const int ra = check_aligned("advect batch backward", arith_bytes(g.fwd.dtype),
                                 {{"output_grad", g.output_grad}, {"data_grad", g.data_grad},
                                  {"vel_x_grad", g.vel_x_grad}, {"vel_y_grad", g.vel_y_grad},
                                  {"vel_z_grad", g.vel_z_grad}});
    if (ra) return ra;
  }
  int zsum, mw, mh;
  int rc = validate_batch(a, count, zsum, mw, mh);
  if (rc) return rc;
  if ((rc = check_aligned("advect batch backward", kScratchAlign, {{"workspace", workspace}}))) return rc;
  const size_t need = batch_bwd_bytes(items, count);
  if (!workspace || workspace_bytes < need)
    return fail(NGT_ERR_WORKSPACE, "advect batch backward needs %zu workspace bytes", need);
  cudaStream_t st = as_stream(stream);
  switch (items[0].fwd.dtype) {
    case NGT_F32: return batch_bwd_c<float>(items, count, zsum, mw, mh, workspace, st);
    case NGT_F64: return batch_bwd_c<double>(items, count, zsum, mw, mh, workspace, st);
    case NGT_BF16: return batch_bwd_c<__nv_bfloat16>(items, count, zsum, mw, mh, workspace, st);
    default: return batch_bwd_c<__half>(items, count, zsum, mw, mh, workspace, st);
  }
}
