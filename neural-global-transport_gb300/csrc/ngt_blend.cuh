// Front-to-back blend functions of the raymarch and reduce-blend operators
// (blending.hpp:9-243): the forward step, its exact local adjoint, and the
// reference's back-to-front ``blendGradients``.  The last channel is the
// density (Beer-Lambert) or alpha; with one channel every mode is additive.
#pragma once

#include "ngt_common.cuh"

namespace ngt {

template <class S> __device__ __forceinline__ S ex(S v);
template <> __device__ __forceinline__ float ex<float>(float v) { return expf(v); }
template <> __device__ __forceinline__ double ex<double>(double v) { return exp(v); }

// One front-to-back blend step (blending.hpp:9-243); channel CB-1 is density / alpha.
template <int CB, class S>
__device__ __forceinline__ void blend_step(S acc[CB], const S cell[CB], int mode) {
  if (CB == 1 || mode == ADDITIVE) {
#pragma unroll
    for (int c = 0; c < CB; ++c) acc[c] = acc[c] + cell[c];
    return;
  }
  const S a = acc[CB - 1], ai = cell[CB - 1];
  if (mode == BEER_LAMBERT) {
    const S d = fmax(a + ai, S(0));
    const S t = ex(-d);
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) acc[c] = acc[c] + t * cell[c];
    acc[CB - 1] = d;
  } else if (mode == ALPHA) {
    const S t = S(1) - a;
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) acc[c] = acc[c] + t * cell[c];
    acc[CB - 1] = a + t * ai;
  } else {  // ALPHA_ADDITIVE
    const S t = S(1) - ai;
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) acc[c] = acc[c] + t * cell[c];
    acc[CB - 1] = a + ai;
  }
}

template <int CB>
__device__ __forceinline__ bool stateful(int mode) {
  return CB > 1 && (mode == BEER_LAMBERT || mode == ALPHA);
}

template <class S>
__device__ __forceinline__ S state_update(S a, S ai, int mode) {
  return mode == BEER_LAMBERT ? fmax(a + ai, S(0)) : a + (S(1) - a) * ai;
}

// Exact local adjoint of one blend step given the accumulator's density / alpha
// before the step.  G holds d(out)/d(acc after the step) and becomes
// d(out)/d(acc before the step).
template <int CB, class S>
__device__ __forceinline__ void blend_adjoint(S G[CB], const S cell[CB], S a_prev, int mode, S dcell[CB]) {
  if (CB == 1 || mode == ADDITIVE) {
#pragma unroll
    for (int c = 0; c < CB; ++c) dcell[c] = G[c];
    return;
  }
  S lg = S(0);
#pragma unroll
  for (int c = 0; c < CB - 1; ++c) lg += cell[c] * G[c];
  const S ai = cell[CB - 1], ga = G[CB - 1];
  if (mode == BEER_LAMBERT) {
    const S x = a_prev + ai;
    const S m = x >= S(0) ? S(1) : S(0);
    const S t = ex(-fmax(x, S(0)));
    const S dd = m * (ga - t * lg);
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) dcell[c] = t * G[c];
    dcell[CB - 1] = dd;
    G[CB - 1] = dd;
  } else if (mode == ALPHA) {
    const S t = S(1) - a_prev;
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) dcell[c] = t * G[c];
    dcell[CB - 1] = t * ga;
    G[CB - 1] = ga * (S(1) - ai) - lg;
  } else {  // ALPHA_ADDITIVE
    const S t = S(1) - ai;
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) dcell[c] = t * G[c];
    dcell[CB - 1] = ga - lg;
  }
}

// blendGradients of blending.hpp, rebuilding the accumulator from the output.
template <int CB, class S>
__device__ __forceinline__ void blend_grad_reference(S G[CB], const S cell[CB], S acc[CB], int mode, S dcell[CB]) {
  if (CB == 1 || mode == ADDITIVE) {
#pragma unroll
    for (int c = 0; c < CB; ++c) dcell[c] = G[c];
    return;
  }
  S lg = S(0);
#pragma unroll
  for (int c = 0; c < CB - 1; ++c) lg += cell[c] * G[c];
  const S ai = cell[CB - 1], ga = G[CB - 1];
  if (mode == BEER_LAMBERT) {
    const S e = ex(-acc[CB - 1]);
    acc[CB - 1] = fmax(acc[CB - 1] - ai, S(0));
    const S dd = ga - e * lg;
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) dcell[c] = e * G[c];
    dcell[CB - 1] = dd;
    G[CB - 1] = dd;
  } else if (mode == ALPHA) {
    acc[CB - 1] = (S(1) - acc[CB - 1]) / (S(1) - ai);
    const S t = S(1) - acc[CB - 1];
    const S dd = (S(1) - ai) * ga - lg;
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) dcell[c] = t * G[c];
    dcell[CB - 1] = t * ga;
    G[CB - 1] = dd;
  } else {
    acc[CB - 1] = acc[CB - 1] - ai;
    const S t = S(1) - ai;
#pragma unroll
    for (int c = 0; c < CB - 1; ++c) dcell[c] = t * G[c];
    dcell[CB - 1] = ga - lg;
  }
}


}  // namespace ngt
