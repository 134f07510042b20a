// tma.cuh -- bulk tensor copies (TMA) into shared memory, with mbarrier
// completion and bounded waits.
//
// Host side: tensor maps of the compact cell fields (x fastest, row pitch P,
// plane pitch P*n2m, field pitch `cells`), encoded through the driver entry
// point that the runtime hands out (no link against libcuda), and cached per
// (address, shape, box) so that a captured step graph replays with the same
// kernel parameters.
//
// Device side: one elected thread arms an mbarrier with the byte count of a
// stage and issues the tile copies; every consumer waits on the barrier's
// phase parity with a wall-clock limit.  A wait that runs out reports it to
// the caller, which raises an error flag for the host and leaves the kernel
// without touching the stage.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdint.h>

namespace tma {

// ---------------------------------------------------------------------
// device
// ---------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes barrier initialisation and earlier generic-proxy accesses of shared
// memory visible to the async proxy (the tensor copies)
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for the phase of `parity` to complete; false after about `limit_ns`
// of wall-clock time (or 2^22 polls, whichever comes first).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns = 1000000000ull) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (int it = 0; it < (1 << 22); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63) == 63 && global_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// Tile copy global -> shared, completion counted on `bar` in bytes.  The
// innermost coordinate times the element size must be a multiple of 16
// bytes (the callers' tiles start at x = 32 t).
__device__ __forceinline__ void load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z,
                                        int w) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_addr(dst)),
      "l"((uint64_t)map), "r"(smem_addr(bar)), "r"(x), "r"(y), "r"(z), "r"(w)
      : "memory");
}

// ---------------------------------------------------------------------
// host
// ---------------------------------------------------------------------
// cuTensorMapEncodeTiled through the runtime's driver entry point; nullptr
// when the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 encode_fn();

// Tensor map of `nfield` compact fields (element size 4 or 8) of grid
// n1m x n2m x n3m with row pitch P (elements), fields `cells` elements
// apart, read in boxes box[0..3] (x, y, z, field); always rank 4.  Returns
// false when the driver refuses it (alignment, sizes) -- the caller then
// takes its non-TMA path.
bool encode_fields(CUtensorMap* out, const void* base, int elem_bytes, int n1m, int n2m, int n3m, int P,
                   size_t cells, int nfield, const int box[4]);

}  // namespace tma
