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
//
// Completion is transitive (a kernel cannot finish before its own wait
// returned), but residency is not: because each kernel releases its
// successor before it waits, kernel K can become resident on an SM while
// K-2 or an earlier kernel of the chain still runs there. Lines that such
// an earlier kernel loads into that SM's L1 / read-only cache after K
// arrived are not refreshed when K-1 later rewrites the data from other
// SMs. So every read of data that some kernel of a chain writes (charges,
// potentials, Krylov vectors, coefficients) goes through ld_chain(), an
// L2-coherent load (ld.global.cg) that never hits a stale L1 line; only the
// operator's own blocks and index lists, which nothing rewrites while an
// operator lives, use the cached or streaming paths.
//
// The chains can be launched without the attribute (plain stream order):
// LS_PDL=0 in the environment, or ls_set_pdl(0) (include/ls_dafmm.h).
#pragma once

#include <cuda_runtime.h>

namespace lsg {

__device__ __forceinline__ void pdl_enter() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

// L2-coherent loads of chain-produced data (see above).
__device__ __forceinline__ double2 ld_chain(const double2* p) { return __ldcg(p); }
__device__ __forceinline__ float2 ld_chain(const float2* p) { return __ldcg(p); }
__device__ __forceinline__ float4 ld_chain(const float4* p) { return __ldcg(p); }
__device__ __forceinline__ double ld_chain(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_chain(const float* p) { return __ldcg(p); }

// 1: chains use programmatic dependent launch (default), 0: plain launches.
int pdl_enabled();
void set_pdl_enabled(int on);
// Whether the native FP64 matvec runs its near field beside the far-field
// chain (LS_NEAR_OVERLAP=0 in the environment: after it).
int near_overlap_enabled();
void set_near_overlap_enabled(int on);

// Raises the dynamic shared-memory limit of `kernel` on the current device
// to at least `bytes`. The limit is one setting per kernel and device for
// the whole process, shared by every operator and network: each call sets
// it to the largest value any caller has asked for on that device, so a
// caller that needs less never lowers it under another one's launches (two
// operators of different sizes used from two threads). Setting it on every
// call also restores it after a device reset. Thread-safe (capi.cpp).
cudaError_t raise_smem_limit(const void* kernel, int bytes);

// kernel<<<grid, block, smem, s>>>(args...) with programmatic stream
// serialization allowed (unless turned off, see pdl_enabled()).
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
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace lsg
