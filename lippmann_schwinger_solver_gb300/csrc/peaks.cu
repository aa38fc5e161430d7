// Measured arithmetic peaks (ls_measure_fma_peak): the FP64 and FP32 FMA
// rates of the device, the denominators of the compute rooflines of the
// native FP64 and the double-float kernels. And the issue cost of one small
// tensor-core MMA (ls_measure_mma_issue), the floor of the tensor-core
// block apply, whose MMAs are M = 128, N <= 64, K = 8 (TF32): below N = 128
// an MMA costs a fixed number of cycles whatever its N, so the block apply
// is bounded by MMAs issued, not by tensor FLOPs.
//
// Each thread runs kChains independent FMA chains for `iters` steps, so the
// pipe always has independent work and the loop overhead is a small share.
// The grid fills every SM several times over.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "ls_internal.h"

namespace lsg {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kMmaSmem = 64 * 1024;        // A (128 rows) in the first half, B (up to 256 rows) in the second
constexpr int kMmaLaunchSmem = 128 * 1024;  // more than half an SM's shared memory: one CTA per SM

template <class T>
__global__ void __launch_bounds__(kThreads) fma_chains_kernel(int iters, T b, T c, T* __restrict__ out) {
  T a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == (T)-1.2345) out[0] = s;  // keeps the chains; b and c make this practically never true
}

template <class T>
cudaError_t measure(int device, int iters, double* tflops) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return e;
  T* out = nullptr;
  if ((e = cudaMalloc(&out, sizeof(T))) != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8;
  const T mb = (T)0.999999, mc = (T)1e-7;
  float best = 0.f;
  for (int r = 0; r < 6 && e == cudaSuccess; ++r) {
    cudaEventRecord(a);
    fma_chains_kernel<T><<<blocks, kThreads>>>(iters, mb, mc, out);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (r > 0 && (best == 0.f || ms < best)) best = ms;  // launch 0 is the warm-up
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  const double flops = 2.0 * kChains * (double)iters * blocks * kThreads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return cudaSuccess;
}

// One CTA per SM; thread 0 issues `reps` back-to-back MMAs (M = 128, N = n,
// K = 8, TF32, operands zero in shared memory, no swizzle) into one
// accumulator and records the cycles of the issue loop; then commits and
// waits (bounded) for their completion. TMEM: 256 columns.
__global__ void __launch_bounds__(128) mma_issue_kernel(int n, int reps, long long* __restrict__ cycles,
                                                        int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  const int t = threadIdx.x;
  for (int i = t; i < kMmaSmem / 4; i += blockDim.x) reinterpret_cast<float*>(sm)[i] = 0.f;
  if (t < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
        (uint32_t)__cvta_generic_to_shared(&tbase)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(&bar);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tm = tbase;
  if (t == 0) {
    auto desc = [](uint32_t a) -> uint64_t {  // K-major, no swizzle: LBO 128, SBO 1024, version 1
      return (uint64_t)((a >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
             ((uint64_t)1 << 46);
    };
    const uint32_t base = (uint32_t)__cvta_generic_to_shared(sm);
    const uint64_t da = desc(base), db = desc(base + kMmaSmem / 2);
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    const long long t0 = clock64();
    for (int r = 0; r < reps; ++r)
      asm volatile("{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }" ::
                       "r"(tm), "l"(da), "l"(db), "r"(idesc), "r"(r > 0 ? 1 : 0));
    const long long t1 = clock64();
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_s) : "memory");
    uint32_t done = 0;
    for (long long it = 0; it < 20000000 && !done; ++it)
      asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                   : "=r"(done)
                   : "r"(bar_s)
                   : "memory");
    if (!done) atomicOr(err, 1);
    atomicAdd(reinterpret_cast<unsigned long long*>(cycles), (unsigned long long)(t1 - t0));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tm));
}

cudaError_t measure_mma(int device, int n, double* clocks) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return e;
  long long* cyc = nullptr;
  int* err = nullptr;
  if ((e = cudaMalloc(&cyc, sizeof(long long))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&err, sizeof(int))) != cudaSuccess) {
    cudaFree(cyc);
    return e;
  }
  constexpr int reps = 512;
  long long total = 0;
  int bad = 0;
  e = cudaFuncSetAttribute(mma_issue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMmaLaunchSmem);
  for (int r = 0; r < 2 && e == cudaSuccess; ++r) {  // launch 0 is the warm-up
    cudaMemset(cyc, 0, sizeof(long long));
    cudaMemset(err, 0, sizeof(int));
    mma_issue_kernel<<<sms, 128, kMmaLaunchSmem>>>(n, reps, cyc, err);
    if ((e = cudaDeviceSynchronize()) == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&total, cyc, sizeof(long long), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&bad, err, sizeof(int), cudaMemcpyDeviceToHost);
  }
  cudaFree(cyc);
  cudaFree(err);
  if (e != cudaSuccess) return e;
  if (bad) return cudaErrorLaunchTimeout;
  *clocks = (double)total / sms / reps;
  return cudaSuccess;
}

}  // namespace
}  // namespace lsg

extern "C" ls_status ls_measure_mma_issue(int device, int n, double* clocks_per_mma) {
  if (!clocks_per_mma || n < 16 || n > 256 || n % 16 != 0) {
    lsg::set_error("ls_measure_mma_issue: n must be a multiple of 16 in [16, 256]");
    return LS_E_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    lsg::set_error("ls_measure_mma_issue: no such CUDA device");
    return LS_E_CUDA;
  }
  const cudaError_t e = lsg::measure_mma(device, n, clocks_per_mma);
  if (e != cudaSuccess) {
    lsg::set_error(std::string("ls_measure_mma_issue: ") + cudaGetErrorString(e));
    return LS_E_CUDA;
  }
  return LS_OK;
}

extern "C" ls_status ls_measure_fma_peak(int device, int kind, double* tflops) {
  if (!tflops || (kind != 0 && kind != 1)) {
    lsg::set_error("ls_measure_fma_peak: bad argument");
    return LS_E_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    lsg::set_error("ls_measure_fma_peak: no such CUDA device");
    return LS_E_CUDA;
  }
  const cudaError_t e = kind == 0 ? lsg::measure<double>(device, 2048, tflops) : lsg::measure<float>(device, 65536, tflops);
  if (e != cudaSuccess) {
    lsg::set_error(std::string("ls_measure_fma_peak: ") + cudaGetErrorString(e));
    return LS_E_CUDA;
  }
  return LS_OK;
}
