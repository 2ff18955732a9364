// The raymarch kernels instantiated for double storage (double arithmetic).
#include "raymarch_kernels.cuh"

namespace ngt {
namespace rm {

int launch_f64(int which, int cin, int cb, dim3 grid, cudaStream_t st, const RayParams& p) {
  return launch_typed<double, double>(which, cin, cb, grid, st, p);
}

}  // namespace rm
}  // namespace ngt
