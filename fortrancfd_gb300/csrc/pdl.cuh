// Programmatic dependent launch (sm_90+; used on sm_103a).
//
// Kernels of one cycle are launched with the programmatic-stream-serialization
// attribute.  Each kernel first lets its successor start launching
// (griddepcontrol.launch_dependents: the successor's blocks are scheduled once
// every block of this grid has issued it), then waits for its predecessor to
// finish and flush (griddepcontrol.wait) before touching the predecessor's
// output.  The launch latency of the next kernel thus overlaps the tail of
// the current one.  Without the attribute both instructions are no-ops.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace gbmg {

__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// kernel<<<g, b, smem, s>>>(args...) with programmatic stream serialization
template <typename... Params, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(Params...), dim3 g, dim3 b, size_t smem,
                              cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = g;
  cfg.blockDim = b;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace gbmg
