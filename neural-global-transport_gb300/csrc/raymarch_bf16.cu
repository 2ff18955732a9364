// The raymarch kernels instantiated for __nv_bfloat16 storage (float arithmetic).
#include "raymarch_kernels.cuh"

namespace ngt {
namespace rm {

int launch_bf16(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p) {
  return launch_typed<__nv_bfloat16, float>(which, cin, cb, grid, st, p);
}

int launch_batch_bf16(int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp) {
  return launch_batch_typed<__nv_bfloat16, float>(which, cin, cb, blocks, st, bp);
}

}  // namespace rm
}  // namespace ngt
