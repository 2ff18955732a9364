// Image L2 loss of the reconstruction step: gradient of 0.5*||image - target||^2
// on the first loss_channels channels, and the loss reduced per block (in the
// image's precision, double for F64) then added atomically.  Also the render's
// background composite and its adjoint.
#include "ngt_common.cuh"
#include "ngt_host.cuh"
#include "ngt_blend.cuh"

namespace ngt {
namespace {

constexpr int kBlock = 256;

template <class S>
__global__ void __launch_bounds__(kBlock) k_l2(int64_t pixels, int C, int LC, const S* __restrict__ img,
                                               const S* __restrict__ tgt, S* __restrict__ grad, S* loss) {
  __shared__ S part[kBlock / 32];
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  S acc = S(0);
  if (i < pixels) {
    for (int c = 0; c < C; ++c) {
      S g = S(0);
      if (c < LC) {
        g = img[i * C + c] - tgt[i * LC + c];
        acc += g * g;
      }
      grad[i * C + c] = g;
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    S v = threadIdx.x < kBlock / 32 ? part[threadIdx.x] : S(0);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) atomicAdd(loss, S(0.5) * v);
  }
}

// Background composite of a rendered image (Renderer.render_density,
// renderer.py:779-781, 804-806): the transmittance t = exp(-d) of each ray, d
// the image's last (optical depth) channel, attenuates the camera's background
// behind the light channels, out_c = image_c + background_c * t, and the depth
// channel is cut (cut_alpha).  One thread per pixel of the per-batch block of
// ``pixels`` (V * H * W); the background is shared by the batch entries.
template <class S>
__global__ void __launch_bounds__(kBlock) k_bkg_fwd(int64_t batch, int64_t pixels, int C, const S* __restrict__ img,
                                                    const S* __restrict__ bkg, S* __restrict__ out) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= pixels) return;
  const int L = C - 1;
  for (int64_t b = 0; b < batch; ++b) {
    const int64_t i = b * pixels + q;
    const S t = ex(-img[i * C + L]);
    for (int c = 0; c < L; ++c) out[i * L + c] = img[i * C + c] + bkg[q * L + c] * t;
  }
}

// Its adjoint: d image_c = g_c, d d = -t * sum_c background_c * g_c, and
// d background_c = sum over the batch of t * g_c (if requested).
template <class S>
__global__ void __launch_bounds__(kBlock) k_bkg_bwd(int64_t batch, int64_t pixels, int C, const S* __restrict__ img,
                                                    const S* __restrict__ bkg, const S* __restrict__ gout,
                                                    S* __restrict__ gimg, S* __restrict__ gbkg) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= pixels) return;
  const int L = C - 1;
  S gb[3] = {S(0), S(0), S(0)};
  for (int64_t b = 0; b < batch; ++b) {
    const int64_t i = b * pixels + q;
    const S t = ex(-img[i * C + L]);
    S sb = S(0);
    for (int c = 0; c < L; ++c) {
      const S g = gout[i * L + c];
      gimg[i * C + c] = g;
      sb += bkg[q * L + c] * g;
      gb[c] += t * g;
    }
    gimg[i * C + L] = -t * sb;
  }
  if (gbkg)
    for (int c = 0; c < L; ++c) gbkg[q * L + c] = gb[c];
}

int bkg_check(const char* op, int32_t dtype, int64_t batch, int64_t pixels, int32_t channels) {
  if (batch <= 0 || pixels <= 0) return fail(NGT_ERR_INVALID_ARGUMENT, "%s: invalid sizes", op);
  if (channels != 2 && channels != 4)
    return fail(NGT_ERR_INVALID_ARGUMENT, "%s: the image has 2 or 4 channels (light channels and optical depth)", op);
  if (dtype != NGT_F32 && dtype != NGT_F64) return fail(NGT_ERR_UNSUPPORTED, "%s: images are F32 or F64", op);
  return NGT_OK;
}

}  // namespace
}  // namespace ngt

using namespace ngt;

extern "C" int ngt_background_composite(int32_t dtype, int64_t batch, int64_t pixels, int32_t channels,
                                        const void* image, const void* background, void* output, void* stream) {
  int rc = bkg_check("background_composite", dtype, batch, pixels, channels);
  if (rc) return rc;
  if (!image || !background || !output) return fail(NGT_ERR_INVALID_ARGUMENT, "background_composite: null pointer");
  if ((rc = check_aligned("background_composite", arith_bytes(dtype),
                          {{"image", image}, {"background", background}, {"output", output}})))
    return rc;
  const unsigned nb = ceil_div_u(pixels, kBlock);
  if (dtype == NGT_F64)
    k_bkg_fwd<double><<<nb, kBlock, 0, as_stream(stream)>>>(batch, pixels, channels, (const double*)image,
                                                             (const double*)background, (double*)output);
  else
    k_bkg_fwd<float><<<nb, kBlock, 0, as_stream(stream)>>>(batch, pixels, channels, (const float*)image,
                                                            (const float*)background, (float*)output);
  return check_launch("ngt_background_composite");
}

extern "C" int ngt_background_composite_bwd(int32_t dtype, int64_t batch, int64_t pixels, int32_t channels,
                                            const void* image, const void* background, const void* output_grad,
                                            void* image_grad, void* background_grad, void* stream) {
  int rc = bkg_check("background_composite_bwd", dtype, batch, pixels, channels);
  if (rc) return rc;
  if (!image || !background || !output_grad || !image_grad)
    return fail(NGT_ERR_INVALID_ARGUMENT, "background_composite_bwd: null pointer");
  if ((rc = check_aligned("background_composite_bwd", arith_bytes(dtype),
                          {{"image", image}, {"background", background}, {"output_grad", output_grad},
                           {"image_grad", image_grad}, {"background_grad", background_grad}})))
    return rc;
  const unsigned nb = ceil_div_u(pixels, kBlock);
  if (dtype == NGT_F64)
    k_bkg_bwd<double><<<nb, kBlock, 0, as_stream(stream)>>>(batch, pixels, channels, (const double*)image,
                                                             (const double*)background, (const double*)output_grad,
                                                             (double*)image_grad, (double*)background_grad);
  else
    k_bkg_bwd<float><<<nb, kBlock, 0, as_stream(stream)>>>(batch, pixels, channels, (const float*)image,
                                                            (const float*)background, (const float*)output_grad,
                                                            (float*)image_grad, (float*)background_grad);
  return check_launch("ngt_background_composite_bwd");
}

extern "C" int ngt_image_l2_loss(int32_t dtype, int64_t pixels, int32_t channels, int32_t loss_channels,
                                 const void* image, const void* target, void* image_grad, void* loss, void* stream) {
  if (!image || !target || !image_grad || !loss) return fail(NGT_ERR_INVALID_ARGUMENT, "image_l2_loss: null pointer");
  if (pixels <= 0 || channels <= 0 || loss_channels <= 0 || loss_channels > channels)
    return fail(NGT_ERR_INVALID_ARGUMENT, "image_l2_loss: invalid sizes");
  if (dtype == NGT_F32 || dtype == NGT_F64) {
    const int rc = check_aligned("image_l2_loss", arith_bytes(dtype), {{"image", image}, {"target", target},
                                                                       {"image_grad", image_grad}, {"loss", loss}});
    if (rc) return rc;
  }
  const unsigned nb = ceil_div_u(pixels, kBlock);
  if (dtype == NGT_F64)
    k_l2<double><<<nb, kBlock, 0, as_stream(stream)>>>(pixels, channels, loss_channels, (const double*)image,
                                                        (const double*)target, (double*)image_grad, (double*)loss);
  else if (dtype == NGT_F32)
    k_l2<float><<<nb, kBlock, 0, as_stream(stream)>>>(pixels, channels, loss_channels, (const float*)image,
                                                       (const float*)target, (float*)image_grad, (float*)loss);
  else
    return fail(NGT_ERR_UNSUPPORTED, "image_l2_loss: images are F32 or F64");
  return check_launch("ngt_image_l2_loss");
}
