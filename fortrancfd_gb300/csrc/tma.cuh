// TMA (cp.async.bulk.tensor) and mbarrier helpers for sm_103a, inline PTX.
//
// Every wait is bounded: after kWaitLimit polls it records an error in a
// global flag and returns false, so no kernel can spin forever on a copy that
// never lands.  The host checks the flag after each solve.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace gbmg {

constexpr int kWaitLimit = 1 << 18;

enum : int { kErrTmaTimeout = 1 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make barrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase with the given parity; false (and *err set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  for (int i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(err, kErrTmaTimeout);
  return false;
}

// 3D tiled load of one box into shared memory, completion on `bar`.
// x * element size must be a multiple of 16 bytes (the caller's contract).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// ---- host side --------------------------------------------------------------
// Encodes a 3D tiled map over a dense (nx, ny, nz) array of `elem` bytes per
// element with an (bx, by, 1) box, zero fill out of bounds.  Returns false
// when the driver rejects it (e.g. a row pitch that is not a multiple of 16).
bool make_tensor_map_3d(CUtensorMap* map, const void* base, CUtensorMapDataType type, int elem,
                        int nx, int ny, int nz, int bx, int by);

}  // namespace gbmg
