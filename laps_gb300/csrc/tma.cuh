// Tensor-memory-accelerator tile loads for the column passes: one elected thread issues a
// 3-D cp.async.bulk.tensor copy of a column tile (TX adjacent kx columns, a whole y or z
// line) from HBM straight into shared memory, counted on an mbarrier that the block waits on.
// The tile lands as [line index][TX columns], the layout the column FFTs use (JS = TX).
//
// Tensor maps describe a work buffer of up to 19 fields as a 3-D array of 8-byte elements:
// dim 0 = kx (kxp complex = kxp * EW elements, EW = element size / 8), dim 1 = y,
// dim 2 = z + field * nz.  Waits are bounded: a wait that runs out reports
// LAPS_STATUS_DEVICE_TIMEOUT in the step status instead of spinning on.
#pragma once
#include <cuda.h>
#include <cstdint>
#include "engine.cuh"

namespace laps {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// make the initialised barriers visible to the async (TMA) proxy
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one arrival that also announces `bytes` of transactions for the current phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// bounded wait for the phase with the given parity; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < (1 << 20); i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// 3-D tile copy global -> shared, completion counted on `bar` (a CTA is its own cluster here)
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// 3-D tile prefetch global -> L2 (no shared memory, no completion to wait for): a hint that
// brings a tile the block will read with ordinary loads later into L2 ahead of use
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap* map, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z)
               : "memory");
}

// Column tile loader of one block: up to two input buffers (two mbarriers, one per buffer;
// a buffer reused for a later input waits on the barrier's next phase).
struct TileLoad {
  uint64_t* bar;      // 2 barriers in shared memory
  uint32_t phase[2];  // parity each barrier waits on next
  __device__ void init(uint64_t* b) {
    bar = b;
    phase[0] = phase[1] = 0;
    if (threadIdx.x == 0) {
      mbar_init(&bar[0], 1);
      mbar_init(&bar[1], 1);
      mbar_fence_init();
    }
    __syncthreads();
  }
  // elected thread: announce `bytes` on barrier b (call once per buffer fill, before the copies)
  __device__ void expect(int b, uint32_t bytes) {
    if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar[b], bytes);
  }
  __device__ void copy(int b, void* dst, const CUtensorMap* map, int x, int y, int z) {
    if (threadIdx.x == 0) tma_load_3d(dst, map, x, y, z, &bar[b]);
  }
  // every thread: wait for buffer b; false (after reporting) when the wait ran out
  __device__ bool wait(int b, StepState* st) {
    const bool ok = mbar_wait(&bar[b], phase[b]);
    phase[b] ^= 1u;
    if (!ok) atomicOr(&st->status, LAPS_STATUS_DEVICE_TIMEOUT);
    return __syncthreads_and(ok) != 0;
  }
};

}  // namespace laps
