// Stale-read probe for chains of kernels launched with programmatic
// dependent launch, in the pattern the library's kernel chains have.
//
// Each round launches three kernels on one stream:
//   reader (K-2): releases its successor, waits, idles for a bounded number
//                 of cycles, then reads all of X (64 KB, fits in one SM's L1);
//   writer (K-1): X[i] = round + 1;
//   check  (K)  : reads all of X and counts values != round + 1.
// Every kernel releases its successor before it waits (as the library's
// pdl_enter does), so the check kernel can already be resident on an SM
// while the reader still runs there and fills that SM's L1 with the old
// values. The probe counts stale values for each load instruction of the
// reader and of the check (ld.global, ld.global.nc, ld.global.cg), with and
// without the launch attribute. Grid: kBlocks x kThreads; every access is
// X[i] with i < kN or counts[0]; every wait is the hardware's grid
// dependency or a clock loop bounded by kIdleCycles.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

constexpr int kN = 16384;
constexpr int kBlocks = 152;
constexpr int kThreads = 256;
constexpr long long kIdleCycles = 20000;

__device__ __forceinline__ void enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <int MODE>
__device__ __forceinline__ float load(const float* p) {
  float v;
  if (MODE == 0) asm volatile("ld.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  else if (MODE == 1) asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  else asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}

template <int MODE>
__global__ void reader(const float* X, float* sink) {
  enter();
  const long long t0 = clock64();
  while (clock64() - t0 < kIdleCycles) {
  }
  float s = 0.f;
  for (int i = threadIdx.x; i < kN; i += blockDim.x) s += load<MODE>(X + i);
  if (s == -1.f) sink[0] = s;  // never true: keeps the loads
}

__global__ void writer(float* X, float v) {
  enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kN; i += gridDim.x * blockDim.x) X[i] = v;
}

template <int MODE>
__global__ void check(const float* X, float v, unsigned long long* counts) {
  enter();
  unsigned long long bad = 0;
  for (int i = threadIdx.x; i < kN; i += blockDim.x) bad += load<MODE>(X + i) != v;
  if (bad) atomicAdd(counts, bad);
}

template <class... KArgs, class... Args>
cudaError_t launch(void (*k)(KArgs...), bool pdl, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kBlocks);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s;
  cudaLaunchAttribute a[1];
  a[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  a[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = a;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

template <int RM, int CM>
int run(bool pdl, int rounds, float* X, float* sink, unsigned long long* counts, cudaStream_t s) {
  cudaMemsetAsync(counts, 0, sizeof(unsigned long long), s);
  launch(writer, false, s, X, 0.f);
  for (int r = 0; r < rounds; ++r) {
    launch(reader<RM>, pdl, s, (const float*)X, sink);
    launch(writer, pdl, s, X, (float)(r + 1));
    launch(check<CM>, pdl, s, (const float*)X, (float)(r + 1), counts);
  }
  unsigned long long h = 0;
  cudaMemcpyAsync(&h, counts, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    std::printf("error %s\n", cudaGetErrorString(e));
    return 1;
  }
  static const char* names[3] = {"ld.global", "ld.global.nc", "ld.global.cg"};
  std::printf("pdl=%d reader=%s check=%s rounds=%d stale=%llu\n", pdl ? 1 : 0, names[RM], names[CM], rounds, h);
  return 0;
}

int main(int argc, char** argv) {
  const int rounds = argc > 1 ? std::atoi(argv[1]) : 2000;
  float *X = nullptr, *sink = nullptr;
  unsigned long long* counts = nullptr;
  if (cudaMalloc(&X, kN * sizeof(float)) != cudaSuccess || cudaMalloc(&sink, sizeof(float)) != cudaSuccess ||
      cudaMalloc(&counts, sizeof(unsigned long long)) != cudaSuccess) {
    std::printf("error cudaMalloc\n");
    return 1;
  }
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  int rc = 0;
  for (int pdl = 1; pdl >= 0; --pdl) {
    rc |= run<0, 0>(pdl, rounds, X, sink, counts, s);
    rc |= run<0, 1>(pdl, rounds, X, sink, counts, s);
    rc |= run<0, 2>(pdl, rounds, X, sink, counts, s);
    rc |= run<1, 0>(pdl, rounds, X, sink, counts, s);
    rc |= run<1, 1>(pdl, rounds, X, sink, counts, s);
    rc |= run<1, 2>(pdl, rounds, X, sink, counts, s);
  }
  cudaFree(X);
  cudaFree(sink);
  cudaFree(counts);
  cudaStreamDestroy(s);
  return rc;
}
