// The raymarch kernels instantiated for __half storage (float arithmetic).
#include "raymarch_kernels.cuh"

namespace ngt {
namespace rm {

int launch_f16(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p) {
  return launch_typed<__half, float>(which, cin, cb, grid, st, p);
}

int launch_batch_f16(int which, int cin, int cb, unsigned blocks, cudaStream_t st, const RayBatch& bp) {
  return launch_batch_typed<__half, float>(which, cin, cb, blocks, st, bp);
}

}  // namespace rm
}  // namespace ngt
