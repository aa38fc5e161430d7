// Chained kernel launches with programmatic dependent launch (sm_90 and
// later; sm_103a here).
//
// The matvec and the Krylov steps are chains of short, dependent kernels
// on one stream. Launched with the programmatic-serialization attribute, a
// kernel may be scheduled while its predecessor is still running; it must
// then wait (griddepcontrol.wait) before it reads anything the predecessor
// writes. Every kernel of the chains starts with pdl_enter(): it first
// allows its own successor to be scheduled (griddepcontrol.launch_dependents,
// which takes effect once all of this grid's blocks have issued it or
// exited, i.e. once the grid is fully resident, so waiting successor blocks
// never hold resources this grid still needs) and then waits for its
// predecessor's completion and memory. The wait is the hardware's grid
// dependency, released when the predecessor grid completes; a kernel
// launched without the attribute passes through both instructions.
#pragma once

#include <cuda_runtime.h>

namespace lsg {

__device__ __forceinline__ void pdl_enter() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

// kernel<<<grid, block, smem, s>>>(args...) with programmatic stream
// serialization allowed.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace lsg
