// Depth reduce-blend of a frustum grid (NDHWC -> NHWC, or every prefix with
// keep_dims) and its gradients: kBlend / kBlendGrad of reduce_blend.cu.cc:34-80.
// One thread per (batch, pixel); consecutive threads read consecutive pixels of
// each depth slice, so every slice is read coalesced.
#include "ngt_common.cuh"
#include "ngt_host.cuh"
#include "ngt_blend.cuh"

namespace ngt {
namespace {

constexpr int kBlock = 256;
constexpr int kSeg = 16;
constexpr int kMaxCkpt = 64;

template <int C, class S>
struct RbParams {
  const S* in;
  S* out;
  const S* out_fwd;
  const S* out_grad;
  S* in_grad;
  int N, D, H, W;
  int blend, keep;
};

template <int C, class S>
__device__ __forceinline__ void load_cell(const RbParams<C, S>& p, int b, int d, int64_t pix, S cell[C]) {
  const S* q = p.in + ((int64_t(b) * p.D + d) * p.H * p.W + pix) * C;
#pragma unroll
  for (int c = 0; c < C; ++c) cell[c] = q[c];
}

template <int C, class S>
__global__ void __launch_bounds__(kBlock) k_rb_fwd(RbParams<C, S> p) {
  const int64_t hw = int64_t(p.H) * p.W;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= hw * p.N) return;
  const int b = int(t / hw);
  const int64_t pix = t % hw;
  S acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = S(0);
  for (int d = 0; d < p.D; ++d) {
    S cell[C];
    load_cell(p, b, d, pix, cell);
    blend_step<C>(acc, cell, p.blend);
    if (p.keep) {
      S* o = p.out + ((int64_t(b) * p.D + d) * hw + pix) * C;
#pragma unroll
      for (int c = 0; c < C; ++c) o[c] = acc[c];
    }
  }
  if (!p.keep) {
    S* o = p.out + (int64_t(b) * hw + pix) * C;
#pragma unroll
    for (int c = 0; c < C; ++c) o[c] = acc[c];
  }
}

// Exact adjoint: accumulator states recomputed forward from checkpoints.
template <int C, class S>
__global__ void __launch_bounds__(kBlock) k_rb_bwd_exact(RbParams<C, S> p) {
  const int64_t hw = int64_t(p.H) * p.W;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= hw * p.N) return;
  const int b = int(t / hw);
  const int64_t pix = t % hw;
  S G[C];
#pragma unroll
  for (int c = 0; c < C; ++c) G[c] = p.keep ? S(0) : p.out_grad[(int64_t(b) * hw + pix) * C + c];
  const int nseg_min = (p.D + kMaxCkpt - 1) / kMaxCkpt;
  const int K = ((max(nseg_min, kSeg) + kSeg - 1) / kSeg) * kSeg;
  const int nck = (p.D + K - 1) / K;
  S ck_a[kMaxCkpt];
  const bool st = stateful<C>(p.blend);
  if (st) {
    S a = S(0);
    for (int d = 0; d < p.D; ++d) {
      if (d % K == 0) ck_a[d / K] = a;
      S cell[C];
      load_cell(p, b, d, pix, cell);
      a = state_update(a, cell[C - 1], p.blend);
    }
  }
  S buf_a[kSeg];
  for (int seg = nck - 1; seg >= 0; --seg) {
    const int i0 = seg * K, i1 = min(i0 + K, p.D);
    const int nsub = (i1 - i0 + kSeg - 1) / kSeg;
    for (int sub = nsub - 1; sub >= 0; --sub) {
      const int j0 = i0 + sub * kSeg, j1 = min(j0 + kSeg, i1);
      if (st) {
        S a = ck_a[seg];
        for (int d = i0; d < j1; ++d) {
          if (d >= j0) buf_a[d - j0] = a;
          S cell[C];
          load_cell(p, b, d, pix, cell);
          a = state_update(a, cell[C - 1], p.blend);
        }
      }
      for (int d = j1 - 1; d >= j0; --d) {
        if (p.keep) {
#pragma unroll
          for (int c = 0; c < C; ++c) G[c] += p.out_grad[((int64_t(b) * p.D + d) * hw + pix) * C + c];
        }
        S cell[C], dcell[C];
        load_cell(p, b, d, pix, cell);
        blend_adjoint<C>(G, cell, st ? buf_a[d - j0] : S(0), p.blend, dcell);
        S* o = p.in_grad + ((int64_t(b) * p.D + d) * hw + pix) * C;
#pragma unroll
        for (int c = 0; c < C; ++c) o[c] = dcell[c];
      }
    }
  }
}

// kBlendGrad (reduce_blend.cu.cc:55-80)
template <int C, class S>
__global__ void __launch_bounds__(kBlock) k_rb_bwd_reference(RbParams<C, S> p) {
  const int64_t hw = int64_t(p.H) * p.W;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= hw * p.N) return;
  const int b = int(t / hw);
  const int64_t pix = t % hw;
  S G[C], prev[C];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    G[c] = p.keep ? S(0) : p.out_grad[(int64_t(b) * hw + pix) * C + c];
    prev[c] = p.keep ? S(0) : p.out_fwd[(int64_t(b) * hw + pix) * C + c];
  }
  for (int d = p.D - 1; d >= 0; --d) {
    if (p.keep) {
#pragma unroll
      for (int c = 0; c < C; ++c) {
        G[c] += p.out_grad[((int64_t(b) * p.D + d) * hw + pix) * C + c];
        prev[c] = p.out_fwd[((int64_t(b) * p.D + d) * hw + pix) * C + c];
      }
    }
    S cell[C], dcell[C];
    load_cell(p, b, d, pix, cell);
    blend_grad_reference<C>(G, cell, prev, p.blend, dcell);
    S* o = p.in_grad + ((int64_t(b) * p.D + d) * hw + pix) * C;
#pragma unroll
    for (int c = 0; c < C; ++c) o[c] = dcell[c];
  }
}

int validate(const ngt_reduce_blend_args* a) {
  if (!a || !a->input) return fail(NGT_ERR_INVALID_ARGUMENT, "reduce_blend: null pointer");
  if (!positive_shape(a->input_shape, 5)) return fail(NGT_ERR_INVALID_ARGUMENT, "reduce_blend: shapes must be positive");
  if (!valid_channels(a->input_shape[4])) return fail(NGT_ERR_INVALID_ARGUMENT, "Only 1,2 and 4 Channel supported.");
  if (a->dtype != NGT_F32 && a->dtype != NGT_F64) return fail(NGT_ERR_UNSUPPORTED, "reduce_blend: dtype must be F32 or F64");
  if (!(a->blending_mode == NGT_BEER_LAMBERT || a->blending_mode == NGT_ALPHA ||
        a->blending_mode == NGT_ALPHA_ADDITIVE || a->blending_mode == NGT_ADDITIVE))
    return fail(NGT_ERR_INVALID_ARGUMENT, "Unkown blend_mode");
  return check_aligned("reduce_blend", arith_bytes(a->dtype), {{"input", a->input}, {"output", a->output}});
}

template <int C, class S>
RbParams<C, S> params(const ngt_reduce_blend_args* a) {
  RbParams<C, S> p = {};
  p.in = static_cast<const S*>(a->input);
  p.out = static_cast<S*>(a->output);
  p.N = int(a->input_shape[0]);
  p.D = int(a->input_shape[1]);
  p.H = int(a->input_shape[2]);
  p.W = int(a->input_shape[3]);
  p.blend = a->blending_mode;
  p.keep = a->keep_dims ? 1 : 0;
  return p;
}

template <int C, class S>
int run(const ngt_reduce_blend_args* a, const ngt_reduce_blend_grad_args* g, cudaStream_t st) {
  RbParams<C, S> p = params<C, S>(a);
  const unsigned nb = ceil_div_u(int64_t(p.N) * p.H * p.W, kBlock);
  if (!g) {
    k_rb_fwd<C, S><<<nb, kBlock, 0, st>>>(p);
  } else {
    p.out_fwd = static_cast<const S*>(g->output);
    p.out_grad = static_cast<const S*>(g->output_grad);
    p.in_grad = static_cast<S*>(g->input_grad);
    if (g->grad_mode == NGT_GRAD_REFERENCE) k_rb_bwd_reference<C, S><<<nb, kBlock, 0, st>>>(p);
    else k_rb_bwd_exact<C, S><<<nb, kBlock, 0, st>>>(p);
  }
  return check_launch(g ? "ngt_reduce_blend_bwd" : "ngt_reduce_blend_fwd");
}

template <class S>
int run_c(const ngt_reduce_blend_args* a, const ngt_reduce_blend_grad_args* g, cudaStream_t st) {
  switch (a->input_shape[4]) {
    case 1: return run<1, S>(a, g, st);
    case 2: return run<2, S>(a, g, st);
    default: return run<4, S>(a, g, st);
  }
}

}  // namespace
}  // namespace ngt

using namespace ngt;

extern "C" int ngt_reduce_blend_fwd(const ngt_reduce_blend_args* a, void* stream) {
  int rc = validate(a);
  if (rc) return rc;
  if (!a->output) return fail(NGT_ERR_INVALID_ARGUMENT, "reduce_blend: null output");
  return a->dtype == NGT_F64 ? run_c<double>(a, nullptr, as_stream(stream)) : run_c<float>(a, nullptr, as_stream(stream));
}

extern "C" int ngt_reduce_blend_bwd(const ngt_reduce_blend_grad_args* g, void* stream) {
  if (!g) return fail(NGT_ERR_INVALID_ARGUMENT, "reduce_blend_bwd: null arguments");
  int rc = validate(&g->fwd);
  if (rc) return rc;
  if (!g->output_grad || !g->input_grad) return fail(NGT_ERR_INVALID_ARGUMENT, "reduce_blend_bwd: null pointer");
  if ((rc = check_aligned("reduce_blend_bwd", arith_bytes(g->fwd.dtype),
                          {{"output", g->output}, {"output_grad", g->output_grad}, {"input_grad", g->input_grad}})))
    return rc;
  if (g->grad_mode == NGT_GRAD_REFERENCE && !g->output)
    return fail(NGT_ERR_INVALID_ARGUMENT, "reduce_blend_bwd: reference mode needs the forward output");
  if (g->grad_mode != NGT_GRAD_EXACT && g->grad_mode != NGT_GRAD_REFERENCE)
    return fail(NGT_ERR_INVALID_ARGUMENT, "reduce_blend_bwd: invalid grad_mode");
  return g->fwd.dtype == NGT_F64 ? run_c<double>(&g->fwd, g, as_stream(stream))
                                 : run_c<float>(&g->fwd, g, as_stream(stream));
}
