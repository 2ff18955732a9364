// Image L2 loss of the reconstruction step: gradient of 0.5*||image - target||^2
// on the first loss_channels channels, and the loss reduced per block (in the
// image's precision, double for F64) then added atomically.
#include "ngt_common.cuh"
#include "ngt_host.cuh"

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

}  // namespace
}  // namespace ngt

using namespace ngt;

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
