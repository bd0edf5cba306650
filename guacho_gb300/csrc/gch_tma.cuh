// gch_tma.cuh -- tensor-memory-accelerator (TMA) tile copies and the
// shared-memory mbarriers that signal their completion, as inline PTX for
// sm_103a.
//
// The stage kernels of the FP32 paths stage the halo ring of each x-y plane
// of their tile with cp.async.bulk.tensor: one elected warp issues the
// copies of a plane (the rows below and above the tile, and the columns left
// and right of it, every field at once through a 4-D tensor map over
// (x, field, y, z)), the copies report their bytes to an mbarrier, and the
// threads that convert halo cells wait on that mbarrier's phase.  Every wait
// is bounded: a wait that runs out reports failure and the kernel raises
// GCH_ERR_TIMEOUT instead of hanging.  The tensor maps cover this GPU's own
// arrays only; no copy uses cluster multicast.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gch {

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// one arrival expected per phase (the issuing thread's arrive.expect_tx)
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
// makes the initialisation visible to the async proxy (the TMA unit)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// arrive on the barrier and add `bytes` to the transaction count of the
// current phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for the phase with the given parity to complete, for at most about
// `limit_cycles` SM clock cycles; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity,
                                          long long limit_cycles = 2000000000LL) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit_cycles) return false;
  return true;
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later async-proxy accesses (a TMA copy that overwrites a buffer
// the threads have read or written).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// A 4-D tiled TMA load of the box at coordinates (c0, c1, c2, c3) of
// `tmap` (a CUtensorMap in global memory written before the launch) into
// shared memory at `dst` (16-byte aligned), completing on `bar`.
__device__ __forceinline__ void tma_load_4d(void* dst, const void* tmap, uint64_t* bar, int c0,
                                            int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
      "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
      : "memory");
}

// Tensor maps of one domain's stage sources, in device memory (built on the
// host with cuTensorMapEncodeTiled when the domain is created).  Each is a
// 4-D map over (x, field, y, z) of a padded structure-of-arrays array: dims
// (NX, neq, NY, NZ), strides (field, row, plane).
// The first stage reads u (8-byte values) or the stored primitives (FP32,
// when the domain keeps them); each source has its own pair of maps, chosen
// by the kernel's source type, so a map always matches the element size the
// kernel's box coordinates assume.
enum TmaMap : int {
  kTmaS1Rows = 0,    // stage-1 source u: one halo row, 36 x neq
  kTmaS1Sides = 1,   // stage-1 source u: 16 bytes wide x neq x TY rows
  kTmaS2Rows = 2,    // stage-2 source (up): one halo row, 36 x neq
  kTmaS2Sides = 3,   // stage-2 source: 16 bytes wide x neq x TY rows
  kTmaS1PRows = 4,   // stage-1 source primit: one halo row, 36 x neq
  kTmaS1PSides = 5,  // stage-1 source primit: 16 bytes wide x neq x TY rows
  kTmaCount = 6
};
constexpr int kTmaMapBytes = 128;  // sizeof(CUtensorMap)

}  // namespace gch
