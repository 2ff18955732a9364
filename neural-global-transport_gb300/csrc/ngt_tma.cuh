// Tensor-memory-accelerator (TMA) loads of 3-D bricks into shared memory, with
// their mbarrier completion, as inline PTX for sm_103a.
//
// A brick is a box of a row-major 3-D grid (x fastest) described by a tensor map
// (cuTensorMapEncodeTiled, looked up through the runtime's driver entry point so
// the library links no driver library).  One thread arms the block's mbarrier
// with the brick's byte count and issues the copy; every thread then waits on the
// barrier's phase.  Elements of the box outside the grid are filled with zeros by
// the copy.  The x coordinate of a box times the element size must be a multiple
// of 16 bytes, and the grid's row and plane strides multiples of 16 bytes; the
// host checks both before it picks a brick kernel.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace ngt {

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  // make the initialised barrier visible to the asynchronous (TMA) proxy
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Arm the barrier for ``bytes`` of transactions (this thread's arrival included).
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n"
      "  .reg .pred p;\n"
      "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "  selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for the barrier's phase ``parity`` to complete, giving up after
// ``limit`` polls (each poll may suspend the thread for a while in hardware);
// false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// The box of ``tmap`` at element coordinates (x, y, z) into shared memory ``dst``
// (16-byte aligned), completing on ``bar``.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tmap, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace ngt
