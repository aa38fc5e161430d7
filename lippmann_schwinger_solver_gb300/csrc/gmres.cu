// GMRES driven by the device DAFMM matvec.
//
// The Krylov basis V (N x (m+1), column major) and all O(N) work live on
// the device. Orthogonalisation is classical Gram-Schmidt applied twice
// (CGS2): each pass is one multi-dot kernel (V^H w, deterministic
// two-stage reduction) and one update kernel (w -= V h). The tiny
// Hessenberg / Givens algebra runs on the host in FP64.
//
// The Arnoldi cycle is written once for the element type of its basis:
// double2 for the FP64 solvers, float2 for the inner solves of the
// mixed-precision refinement, whose corrections only need the accuracy of
// the FP32 operator they are solved with.
//
// Reference behaviour restated:
//  * classGMRES::gmres (GMRES_Hybrid/include/gmres.hpp:54-119): x0 = 0,
//    Givens-updated residual estimate |beta_{k+1}| / |b|, stop when it
//    drops to the threshold; here with the conjugate-linear inner product
//    and unitary complex rotations.
//  * GMRES / RestartedGMRES (GMRES/GMRES.cpp:257-319): fixed m, early exit
//    when H(j+1,j) < 1e-8, least squares on the (j+1) x j Hessenberg.

#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <vector>

#include "device.h"
#include "launch.h"

namespace lsg {

constexpr int kDotThreads = 128;
constexpr int kDotBlocks = 304;  // row chunks: partial sums per column (2 per SM)
constexpr int kDotCols = 8;      // columns per multi-dot block
constexpr int kAxpyBlocksMax = 152 * 8;  // grid_for()'s cap: per-block norm partials
// DGKS criterion of the conditional second Gram-Schmidt pass: it runs only
// when the first pass removed more than half of |w|^2 (|w'| < |w| / sqrt 2).
constexpr double kReorthRatio = 0.5;
constexpr int kFlexInner = 24;   // steps of a right-preconditioned inner cycle
// Inner targets at or above this relative reduction are left to plain
// GMRES: a few unpreconditioned steps reach them for less than the
// network's applications would cost.
constexpr double kFlexPlainTol = 1e-3;

template <class T> struct Cx;
template <> struct Cx<double2> {
  using R = double;
  static __host__ __device__ double2 make(double a, double b) { return make_double2(a, b); }
};
template <> struct Cx<float2> {
  using R = float;
  static __host__ __device__ float2 make(float a, float b) { return make_float2(a, b); }
};

// Krylov basis V (n x (m+1)) and two n-vectors of one element type.
template <class T>
struct Basis {
  T* V = nullptr;
  T* w = nullptr;
  T* r = nullptr;
  T* Z = nullptr;  // flexible GMRES: preconditioned directions z_k = M(v_k)
  int n = 0, cap = -1, zcap = -1;
  void release() {
    cudaFree(V); cudaFree(w); cudaFree(r); cudaFree(Z);
    V = w = r = Z = nullptr;
    n = 0;
    cap = zcap = -1;
  }
  cudaError_t ensure_z(int m) {
    if (Z && m <= zcap) return cudaSuccess;
    cudaFree(Z);
    Z = nullptr;
    zcap = -1;
    cudaError_t e = cudaMalloc(&Z, (size_t)n * sizeof(T) * (m + 1));
    if (e == cudaSuccess) zcap = m;
    return e;
  }
  cudaError_t ensure(int n_, int m) {
    if (n_ == n && m <= cap) return cudaSuccess;
    release();
    const size_t nb = (size_t)n_ * sizeof(T);
    cudaError_t e = cudaMalloc(&V, nb * (m + 1));
    if (e == cudaSuccess) e = cudaMalloc(&w, nb);
    if (e == cudaSuccess) e = cudaMalloc(&r, nb);
    if (e != cudaSuccess) {
      release();
      return e;
    }
    n = n_;
    cap = m;
    return cudaSuccess;
  }
};

// Column groups of a multi-dot over up to m + 1 basis vectors and w.
inline int n_counters(int m) { return (m + 2 + kDotCols - 1) / kDotCols; }

struct GmresWorkspace {
  Basis<double2> b64;
  Basis<float2> b32;
  // Mixed-precision refinement: FP64 residual, FP32 right-hand side and correction.
  double2* res = nullptr;
  float2* res32 = nullptr;
  float2* dx32 = nullptr;
  // FP64 inner basis over the FP32 operator: the correction, and the FP32
  // copies of a direction and its preconditioned image.
  double2* dx64 = nullptr;
  float2* pv32 = nullptr;
  float2* pz32 = nullptr;
  // Coefficients: per-block partial sums, CGS passes, |w|^2 (all FP64).
  double2* partial = nullptr;
  double2* h = nullptr;
  double2* h2 = nullptr;
  double2* nrm = nullptr;   // [0] |w|^2 of the new direction, [1] before and [2] after the first pass
  double* npartial = nullptr;  // per-block partial norms of the fused corrections
  unsigned* counters = nullptr;  // finished blocks per column group, + one for the corrections
  cudaEvent_t copied = nullptr;  // a step's coefficients are on the host
  cudaEvent_t orthogonalised = nullptr;  // a step's Gram-Schmidt kernels are done
  cudaStream_t side = nullptr;  // the coefficient copies, off the operator's stream
  double2* pinned = nullptr;     // host: h (m+2), h2 (m+2), |w|^2; page-locked so copies stay asynchronous
  int n = 0, cap = -1;
  int n_groups() const { return n_counters(cap); }
  void release_small() {
    cudaFree(res); cudaFree(res32); cudaFree(dx32); cudaFree(partial); cudaFree(h); cudaFree(h2); cudaFree(nrm);
    cudaFree(dx64); cudaFree(pv32); cudaFree(pz32); cudaFree(npartial); cudaFree(counters);
    res = partial = h = h2 = nrm = dx64 = nullptr;
    npartial = nullptr;
    counters = nullptr;
    res32 = dx32 = pv32 = pz32 = nullptr;
    if (copied) cudaEventDestroy(copied);
    if (orthogonalised) cudaEventDestroy(orthogonalised);
    if (side) cudaStreamDestroy(side);
    copied = orthogonalised = nullptr;
    side = nullptr;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    n = 0;
    cap = -1;
  }
  void release() {
    b64.release();
    b32.release();
    release_small();
  }
  // Coefficient buffers for up to m Arnoldi steps on n-vectors; kept
  // between solves and grown only when a solve needs more.
  cudaError_t ensure(int n_, int m) {
    if (n_ == n && m <= cap) return cudaSuccess;
    release_small();
    cudaError_t e = cudaMalloc(&res, (size_t)n_ * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&res32, (size_t)n_ * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&dx32, (size_t)n_ * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&dx64, (size_t)n_ * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&pv32, (size_t)n_ * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&pz32, (size_t)n_ * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&partial, (size_t)kDotBlocks * (m + 2) * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&h, (size_t)(m + 2) * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&h2, (size_t)(m + 2) * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&nrm, 3 * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&npartial, kAxpyBlocksMax * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&counters, (size_t)(n_counters(m) + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(counters, 0, (size_t)(n_counters(m) + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&orthogonalised, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&pinned, (size_t)(2 * (m + 2) + 1) * sizeof(double2));
    if (e != cudaSuccess) {
      release_small();
      return e;
    }
    n = n_;
    cap = m;
    return cudaSuccess;
  }
};

GmresWorkspace& workspace(DevOperator& d) {
  if (!d.gws) d.gws = new GmresWorkspace();
  return *d.gws;
}

void dev_free_gmres(DevOperator& d) {
  if (d.gws) {
    d.gws->release();
    delete d.gws;
    d.gws = nullptr;
  }
}

namespace {

// (x, y) <- (kx + partner's x, ky + partner's y) for the lane l ^ o.
template <class R>
__device__ __forceinline__ void shfl_add(R& x, R& y, R kx, R ky, int o) {
  x = kx + __shfl_xor_sync(0xffffffffu, x, o);
  y = ky + __shfl_xor_sync(0xffffffffu, y, o);
}

// True when the second Gram-Schmidt pass is not needed (DGKS): the first
// pass left at least kReorthRatio of |w|^2.
__device__ __forceinline__ bool reorth_skipped(const double2* nrm_w, const double2* nrm_r) {
  return ld_chain(nrm_r).x >= kReorthRatio * ld_chain(nrm_w).x;
}

// out[c] = sum_rows conj(V[row, c]) * w[row] for c < ncols and, with
// nrm_out, *nrm_out = |w|^2 (w taken as one more column).
// Block (x, y) owns a contiguous chunk of rows and the columns
// 8y .. 8y+7: each thread keeps eight sums, so it has eight independent
// loads in flight per row. GB300's FP64 pipe is narrow, so the warp
// reduction of the eight sums is a transposing butterfly: at each of the
// first three shuffle steps a lane keeps half of its columns and adds the
// partner's half, which leaves each group of four lanes one column (18
// adds per lane instead of 80). Each block leaves its sums in partial; the
// last block of a column group to finish (counted in counters[y]) adds the
// group's partials in a fixed order and resets the counter for the next
// launch, so the dot products take one launch and stay deterministic.
// With gate_w / gate_r (the second, conditional pass) the kernel writes
// zeros instead when reorth_skipped().
template <class T>
__global__ void __launch_bounds__(kDotThreads) gs_dot_kernel(const T* __restrict__ V, long long ldv, int ncols,
                                                             const T* __restrict__ w, int n,
                                                             double2* __restrict__ partial,
                                                             unsigned* __restrict__ counters,
                                                             double2* __restrict__ out, double2* __restrict__ nrm_out,
                                                             const double2* __restrict__ gate_w,
                                                             const double2* __restrict__ gate_r) {
  pdl_enter();
  using R = typename Cx<T>::R;
  __shared__ T red[kDotThreads / 32][kDotCols];
  __shared__ unsigned ticket;
  const int nv = ncols + (nrm_out ? 1 : 0);
  const int c0 = blockIdx.y * kDotCols;
  const int nc = min(kDotCols, nv - c0);
  if (gate_w && reorth_skipped(gate_w, gate_r)) {
    if (blockIdx.x == 0 && (int)threadIdx.x < nc && c0 + (int)threadIdx.x < ncols)
      out[c0 + threadIdx.x] = make_double2(0.0, 0.0);
    return;
  }
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * chunk;
  const int len = max(0, min(chunk, n - r0));
  R ar[kDotCols], ai[kDotCols];
#pragma unroll
  for (int j = 0; j < kDotCols; ++j) ar[j] = ai[j] = R(0);
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    const T b = ld_chain(w + r0 + i);
    T a[kDotCols];
#pragma unroll
    for (int j = 0; j < kDotCols; ++j)  // all loads first, so that they are in flight together
      a[j] = c0 + j < ncols ? ld_chain(V + (size_t)(c0 + j) * ldv + r0 + i)
                            : (j < nc ? b : Cx<T>::make(R(0), R(0)));
#pragma unroll
    for (int j = 0; j < kDotCols; ++j) {
      ar[j] = fma(a[j].x, b.x, ar[j]);
      ar[j] = fma(a[j].y, b.y, ar[j]);
      ai[j] = fma(a[j].x, b.y, ai[j]);
      ai[j] = fma(-a[j].y, b.x, ai[j]);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // Butterfly: after the steps 16, 8, 4 lane l holds column
  // 4 * bit4(l) + 2 * bit3(l) + bit2(l); steps 2 and 1 finish its sum.
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const bool hi = lane & 16;
    R sx = hi ? ar[j] : ar[j + 4], sy = hi ? ai[j] : ai[j + 4];
    shfl_add(sx, sy, hi ? ar[j + 4] : ar[j], hi ? ai[j + 4] : ai[j], 16);
    ar[j] = sx;
    ai[j] = sy;
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const bool hi = lane & 8;
    R sx = hi ? ar[j] : ar[j + 2], sy = hi ? ai[j] : ai[j + 2];
    shfl_add(sx, sy, hi ? ar[j + 2] : ar[j], hi ? ai[j + 2] : ai[j], 8);
    ar[j] = sx;
    ai[j] = sy;
  }
  {
    const bool hi = lane & 4;
    R sx = hi ? ar[0] : ar[1], sy = hi ? ai[0] : ai[1];
    shfl_add(sx, sy, hi ? ar[1] : ar[0], hi ? ai[1] : ai[0], 4);
    ar[0] = sx;
    ai[0] = sy;
  }
  for (int o = 2; o > 0; o >>= 1) {
    R sx = ar[0], sy = ai[0];
    shfl_add(sx, sy, ar[0], ai[0], o);
    ar[0] = sx;
    ai[0] = sy;
  }
  if ((lane & 3) == 0)
    red[wid][((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1)] = Cx<T>::make(ar[0], ai[0]);
  __syncthreads();
  if ((int)threadIdx.x < nc) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kDotThreads / 32; ++k) {
      a += (double)red[k][threadIdx.x].x;
      b += (double)red[k][threadIdx.x].y;
    }
    partial[(size_t)(c0 + threadIdx.x) * gridDim.x + blockIdx.x] = make_double2(a, b);
  }
  // The last block of the group adds the group's partial sums.
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(counters + blockIdx.y, 1u);
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  __threadfence();
  for (int t = wid; t < nc; t += kDotThreads / 32) {
    double a = 0.0, b = 0.0;
    for (int k = lane; k < (int)gridDim.x; k += 32) {
      const double2 p = __ldcg(partial + (size_t)(c0 + t) * gridDim.x + k);
      a += p.x;
      b += p.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      double2* d = c0 + t < ncols ? out + c0 + t : nrm_out;
      *d = make_double2(a, b);
    }
  }
  if (threadIdx.x == 0) counters[blockIdx.y] = 0;
}

// One Gram-Schmidt correction fused with the norm that follows it:
// w[i] -= sum_c V[i, c] * h[c], then *nrm_out = |w|^2 (the per-block
// partial norms added in a fixed order by the last block to finish, as in
// gs_dot_kernel). With gate_w / gate_r (the second, conditional pass) a
// skipped pass leaves w unchanged and copies *gate_r to *nrm_out.
template <class T>
__global__ void __launch_bounds__(256) axpy_norm_kernel(T* __restrict__ w, const T* __restrict__ V, long long ldv,
                                                        int ncols, const double2* __restrict__ h, int n,
                                                        double* __restrict__ npartial, unsigned* __restrict__ counter,
                                                        double2* __restrict__ nrm_out,
                                                        const double2* __restrict__ gate_w,
                                                        const double2* __restrict__ gate_r) {
  pdl_enter();
  using R = typename Cx<T>::R;
  __shared__ double red[8];
  __shared__ unsigned ticket;
  if (gate_w && reorth_skipped(gate_w, gate_r)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *nrm_out = ld_chain(gate_r);
    return;
  }
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    R sr = R(0), si = R(0);
    int c = 0;
    for (; c + 4 <= ncols; c += 4) {
      T v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = ld_chain(V + (size_t)(c + j) * ldv + i);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double2 hc = ld_chain(h + c + j);
        const R hx = (R)hc.x, hy = (R)hc.y;
        sr = fma(v[j].x, hx, sr);
        sr = fma(-v[j].y, hy, sr);
        si = fma(v[j].x, hy, si);
        si = fma(v[j].y, hx, si);
      }
    }
    for (; c < ncols; ++c) {
      const T v = ld_chain(V + (size_t)c * ldv + i);
      const double2 hc = ld_chain(h + c);
      const R hx = (R)hc.x, hy = (R)hc.y;
      sr = fma(v.x, hx, sr);
      sr = fma(-v.y, hy, sr);
      si = fma(v.x, hy, si);
      si = fma(v.y, hx, si);
    }
    const T o = ld_chain(w + i);
    const R nx = o.x - sr, ny = o.y - si;
    w[i] = Cx<T>::make(nx, ny);
    acc = fma((double)nx, (double)nx, acc);
    acc = fma((double)ny, (double)ny, acc);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) red[wid] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    npartial[blockIdx.x] = t;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(counter, 1u);
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  __threadfence();
  double t = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) t += __ldcg(npartial + k);
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  __syncthreads();
  if (lane == 0) red[wid] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) u += red[k];
    *nrm_out = make_double2(u, 0.0);
    *counter = 0;
  }
}

// w[i] += sign * sum_c V[i, c] * h[c]; the column loop is unrolled by 4 so
// that four independent loads of V are in flight per thread.
template <class T>
__global__ void __launch_bounds__(256) multi_axpy_kernel(T* __restrict__ w, const T* __restrict__ V, long long ldv,
                                                         int ncols, const double2* __restrict__ h, int n,
                                                         double sign) {
  pdl_enter();
  using R = typename Cx<T>::R;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    R sr = R(0), si = R(0);
    int c = 0;
    for (; c + 4 <= ncols; c += 4) {
      T v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = ld_chain(V + (size_t)(c + j) * ldv + i);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double2 hc = ld_chain(h + c + j);
        const R hx = (R)hc.x, hy = (R)hc.y;
        sr = fma(v[j].x, hx, sr);
        sr = fma(-v[j].y, hy, sr);
        si = fma(v[j].x, hy, si);
        si = fma(v[j].y, hx, si);
      }
    }
    for (; c < ncols; ++c) {
      const T v = ld_chain(V + (size_t)c * ldv + i);
      const double2 hc = ld_chain(h + c);
      const R hx = (R)hc.x, hy = (R)hc.y;
      sr = fma(v.x, hx, sr);
      sr = fma(-v.y, hy, sr);
      si = fma(v.x, hy, si);
      si = fma(v.y, hx, si);
    }
    T o = ld_chain(w + i);
    o.x += (R)sign * sr;
    o.y += (R)sign * si;
    w[i] = o;
  }
}

template <class T>
__global__ void scale_kernel(const T* __restrict__ a, T* __restrict__ b, double s, int n) {
  pdl_enter();
  using R = typename Cx<T>::R;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T v = ld_chain(a + i);
    b[i] = Cx<T>::make(v.x * (R)s, v.y * (R)s);
  }
}

// b = a / sqrt(nrm->x), or zeros when the norm is zero (breakdown; the
// vector is then never used).
template <class T>
__global__ void scale_by_norm_kernel(const T* __restrict__ a, T* __restrict__ b, const double2* __restrict__ nrm,
                                     int n) {
  pdl_enter();
  using R = typename Cx<T>::R;
  __shared__ R f;  // formed once per thread block (FP64 divides are slow on GB300)
  if (threadIdx.x == 0) {
    const double nn = ld_chain(nrm).x;
    f = nn > 0.0 ? (R)(1.0 / sqrt(nn)) : R(0);
  }
  __syncthreads();
  const R s = f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T v = ld_chain(a + i);
    b[i] = Cx<T>::make(v.x * s, v.y * s);
  }
}

template <class T>
__global__ void sub_kernel(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ c, int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T u = ld_chain(a + i), v = ld_chain(b + i);
    c[i] = Cx<T>::make(u.x - v.x, u.y - v.y);
  }
}

__global__ void to_f32_kernel(const double2* __restrict__ a, float2* __restrict__ b, int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 v = ld_chain(a + i);
    b[i] = make_float2((float)v.x, (float)v.y);
  }
}

// a += b, with b widened to FP64
__global__ void add_f32_kernel(double2* __restrict__ a, const float2* __restrict__ b, int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 u = ld_chain(a + i);
    const float2 v = ld_chain(b + i);
    u.x += (double)v.x;
    u.y += (double)v.y;
    a[i] = u;
  }
}

__global__ void to_f64_kernel(const float2* __restrict__ a, double2* __restrict__ b, int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 v = ld_chain(a + i);
    b[i] = make_double2((double)v.x, (double)v.y);
  }
}

// a += b (FP64)
__global__ void add_kernel(double2* __restrict__ a, const double2* __restrict__ b, int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 u = ld_chain(a + i);
    const double2 v = ld_chain(b + i);
    u.x += v.x;
    u.y += v.y;
    a[i] = u;
  }
}

using cdh = std::complex<double>;

int grid_for(int n) { return std::min((n + 255) / 256, 152 * 8); }

// h_dev[0:ncols) = V[:, 0:ncols)^H w and, with nrm_dev, *nrm_dev = |w|^2;
// with gate_w / gate_r the conditional second pass.
template <class T>
void multidot(const T* V, long long ldv, int ncols, const T* w, int n, GmresWorkspace& ws, double2* h_dev,
              double2* nrm_dev, const double2* gate_w, const double2* gate_r, cudaStream_t s) {
  const int nv = ncols + (nrm_dev ? 1 : 0);
  launch_pdl(gs_dot_kernel<T>, dim3(kDotBlocks, (nv + kDotCols - 1) / kDotCols), kDotThreads, 0, s, V, ldv, ncols, w,
             n, ws.partial, ws.counters, h_dev, nrm_dev, gate_w, gate_r);
}

// w -= V[:, 0:ncols) h_dev, then *nrm_dev = |w|^2 (see axpy_norm_kernel).
template <class T>
void correct(T* w, const T* V, long long ldv, int ncols, const double2* h_dev, int n, GmresWorkspace& ws,
             double2* nrm_dev, const double2* gate_w, const double2* gate_r, cudaStream_t s) {
  launch_pdl(axpy_norm_kernel<T>, grid_for(n), 256, 0, s, w, V, ldv, ncols, h_dev, n, ws.npartial,
             ws.counters + (ws.n_groups()), nrm_dev, gate_w, gate_r);
}

template <class T>
cudaError_t vnorm(const T* w, int n, GmresWorkspace& ws, cudaStream_t s, double& out) {
  multidot(static_cast<const T*>(nullptr), n, 0, w, n, ws, nullptr, ws.nrm, nullptr, nullptr, s);
  double2 hv;
  cudaError_t e = cudaMemcpyAsync(&hv, ws.nrm, sizeof(double2), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  out = std::sqrt(hv.x);
  return cudaSuccess;
}

// y = A x. An FP32 basis always uses the FP32 operator. An FP64 basis uses
// the FP64 operator (native or double-float kernels), or, with f32_op, the
// FP32 operator on FP64 vectors (x rounded to FP32 on load, y widened on
// store): the inner solves of the mixed-precision refinement with their
// Gram-Schmidt and Givens algebra in FP64.
cudaError_t apply(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool f32_op) {
  return f32_op ? dev_matvec_f32(d, x, y, s, false) : dev_matvec(d, x, y, s, false);
}
cudaError_t apply(DevOperator& d, const float2* x, float2* y, cudaStream_t s, bool) {
  return dev_matvec_f32v(d, x, y, s);
}

Basis<double2>& basis(GmresWorkspace& ws, const double2*) { return ws.b64; }
Basis<float2>& basis(GmresWorkspace& ws, const float2*) { return ws.b32; }

// z = M(v): M works on FP32 vectors, so an FP64 direction is rounded to FP32
// first and the result widened back.
cudaError_t precondition(Precond32* M, GmresWorkspace&, const float2* v, float2* z, int, cudaStream_t s) {
  return M->apply(v, z, s);
}
cudaError_t precondition(Precond32* M, GmresWorkspace& ws, const double2* v, double2* z, int n, cudaStream_t s) {
  launch_pdl(to_f32_kernel, grid_for(n), 256, 0, s, v, ws.pv32, n);
  cudaError_t e = M->apply(ws.pv32, ws.pz32, s);
  if (e != cudaSuccess) return e;
  launch_pdl(to_f64_kernel, grid_for(n), 256, 0, s, (const float2*)ws.pz32, z, n);
  return cudaGetLastError();
}

// One Arnoldi cycle from x0 (device, may be null for x0 = 0). Writes the
// updated solution into x. tol < 0 disables the residual stop; breakdown
// exits when H(k+1,k) < brk. With M (FP32 bases only) the cycle is flexible
// GMRES: step k applies A to z_k = M(v_k), keeps z_k, and the update is
// x = x0 + Z y instead of x0 + V y.
template <class T>
cudaError_t arnoldi_cycle(DevOperator& d, GmresWorkspace& ws, const T* b, const T* x0, T* x, int m, double tol,
                          double brk, double bnorm, std::vector<double>* hist, int& iters, bool& converged,
                          Precond32* M = nullptr, bool f32_op = false) {
  Basis<T>& B = basis(ws, b);
  cudaStream_t s = d.stream;
  const int n = d.N;
  cudaError_t e;
  if (M && (e = B.ensure_z(m)) != cudaSuccess) return e;
  // w = A v_k, or w = A M(v_k) with z_k kept.
  auto product = [&](int k) -> cudaError_t {
    const T* v = B.V + (size_t)k * n;
    if (!M) return apply(d, v, B.w, s, f32_op);
    T* z = B.Z + (size_t)k * n;
    cudaError_t pe = precondition(M, ws, v, z, n, s);
    return pe != cudaSuccess ? pe : apply(d, z, B.w, s, f32_op);
  };
  // r = b - A x0
  if (x0) {
    if ((e = apply(d, x0, B.w, s, f32_op)) != cudaSuccess) return e;
    launch_pdl(sub_kernel<T>, grid_for(n), 256, 0, s, b, B.w, B.r, n);
  } else {
    cudaMemcpyAsync(B.r, b, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  }
  double beta = 0.0;
  if ((e = vnorm(B.r, n, ws, s, beta)) != cudaSuccess) return e;
  if (hist && hist->empty()) hist->push_back(beta / bnorm);
  converged = false;
  iters = 0;
  if (beta == 0.0) {
    if (x != x0) {
      if (x0) cudaMemcpyAsync(x, x0, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, s);
      else cudaMemsetAsync(x, 0, (size_t)n * sizeof(T), s);
    }
    converged = true;
    return cudaStreamSynchronize(s);
  }
  launch_pdl(scale_kernel<T>, grid_for(n), 256, 0, s, B.r, B.V, 1.0 / beta, n);
  std::vector<std::vector<cdh>> H;  // columns, already rotated
  std::vector<cdh> cs, sn, g(1, cdh(beta, 0.0));
  int K = 0;
  // The product A v_{k+1} only needs v_{k+1} = w / |w|, which the device
  // forms itself, so it is queued before the host waits for step k's
  // coefficients: the host's Givens work and the wait hide behind it. A
  // converged or broken-down cycle leaves one unused product behind.
  if ((e = product(0)) != cudaSuccess) return e;
  double2* hp = ws.pinned;
  double2* hp2 = ws.pinned + (m + 2);
  double2* np = ws.pinned + 2 * (m + 2);
  for (int k = 0; k < m; ++k) {
    // Classical Gram-Schmidt with a conditional second pass (DGKS), all on
    // the device; one copy back per step. Pass 1: h = V^H w with |w|^2, then
    // w' = w - V h with |w'|^2. Pass 2 (h2 = V^H w', w'' = w' - V h2 with
    // |w''|^2) runs only when |w'|^2 < kReorthRatio |w|^2; otherwise both
    // of its kernels return at once, h2 = 0 and |w''|^2 = |w'|^2.
    double2* nrm_w = ws.nrm + 1;
    double2* nrm_1 = ws.nrm + 2;
    multidot(B.V, n, k + 1, B.w, n, ws, ws.h, nrm_w, nullptr, nullptr, s);
    correct(B.w, B.V, n, k + 1, ws.h, n, ws, nrm_1, nullptr, nullptr, s);
    multidot(B.V, n, k + 1, B.w, n, ws, ws.h2, nullptr, nrm_w, nrm_1, s);
    correct(B.w, B.V, n, k + 1, ws.h2, n, ws, ws.nrm, nrm_w, nrm_1, s);
    launch_pdl(scale_by_norm_kernel<T>, grid_for(n), 256, 0, s, B.w, B.V + (size_t)(k + 1) * n, ws.nrm, n);
    // The coefficients go to the host on a side stream, so that the next
    // operator apply follows the Gram-Schmidt kernels directly on the
    // operator's stream. The host waits for these copies before it queues the
    // next step's Gram-Schmidt kernels, the next writers of h, h2 and nrm.
    if ((e = cudaEventRecord(ws.orthogonalised, s)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(ws.side, ws.orthogonalised, 0)) != cudaSuccess) return e;
    cudaMemcpyAsync(hp, ws.h, (size_t)(k + 1) * sizeof(double2), cudaMemcpyDeviceToHost, ws.side);
    cudaMemcpyAsync(hp2, ws.h2, (size_t)(k + 1) * sizeof(double2), cudaMemcpyDeviceToHost, ws.side);
    cudaMemcpyAsync(np, ws.nrm, sizeof(double2), cudaMemcpyDeviceToHost, ws.side);
    if ((e = cudaEventRecord(ws.copied, ws.side)) != cudaSuccess) return e;
    if (k + 1 < m && (e = product(k + 1)) != cudaSuccess) return e;
    if ((e = cudaEventSynchronize(ws.copied)) != cudaSuccess) return e;
    std::vector<cdh> hk(k + 2);
    for (int i = 0; i <= k; ++i) hk[i] = cdh(hp[i].x + hp2[i].x, hp[i].y + hp2[i].y);
    const double wn = std::sqrt(np->x);
    hk[k + 1] = wn;
    const bool breakdown = (std::abs(hk[k + 1]) < brk);
    // Givens rotations (unitary): G = [[conj(c), conj(s)], [-s, c]].
    for (int i = 0; i < k; ++i) {
      const cdh t = std::conj(cs[i]) * hk[i] + std::conj(sn[i]) * hk[i + 1];
      hk[i + 1] = -sn[i] * hk[i] + cs[i] * hk[i + 1];
      hk[i] = t;
    }
    const double nr = std::sqrt(std::norm(hk[k]) + std::norm(hk[k + 1]));
    cdh c = nr == 0.0 ? cdh(1.0, 0.0) : hk[k] / nr;
    cdh sv = nr == 0.0 ? cdh(0.0, 0.0) : hk[k + 1] / nr;
    cs.push_back(c);
    sn.push_back(sv);
    hk[k] = std::conj(c) * hk[k] + std::conj(sv) * hk[k + 1];
    hk[k + 1] = 0.0;
    H.push_back(hk);
    g.push_back(-sv * g[k]);
    g[k] = std::conj(c) * g[k];
    K = k + 1;
    const double est = std::abs(g[k + 1]) / bnorm;
    if (hist) hist->push_back(est);
    if ((tol >= 0.0 && est <= tol) || breakdown) {
      converged = tol >= 0.0 && est <= tol;
      break;
    }
  }
  // Back substitution R y = g, then x = x0 + V y.
  std::vector<cdh> y(K);
  for (int i = K - 1; i >= 0; --i) {
    cdh sum = g[i];
    for (int j = i + 1; j < K; ++j) sum -= H[j][i] * y[j];
    y[i] = sum / H[i][i];
  }
  std::vector<double2> hbuf(K + 1);
  for (int i = 0; i < K; ++i) hbuf[i] = make_double2(y[i].real(), y[i].imag());
  cudaMemcpyAsync(ws.h, hbuf.data(), (size_t)K * sizeof(double2), cudaMemcpyHostToDevice, s);
  if (x0) {
    if (x != x0) cudaMemcpyAsync(x, x0, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  } else {
    cudaMemsetAsync(x, 0, (size_t)n * sizeof(T), s);
  }
  launch_pdl(multi_axpy_kernel<T>, grid_for(n), 256, 0, s, x, M ? B.Z : B.V, n, K, ws.h, n, 1.0);
  iters = K;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

}  // namespace

cudaError_t dev_gmres(DevOperator& d, const double2* b, double2* x, int max_iter, double tol,
                      std::vector<double>& hist, GmresResult& res) {
  GmresWorkspace& ws = workspace(d);
  cudaError_t e = ws.ensure(d.N, max_iter);
  if (e == cudaSuccess) e = ws.b64.ensure(d.N, max_iter);
  if (e != cudaSuccess) return e;
  double bn = 0.0;
  if ((e = vnorm(b, d.N, ws, d.stream, bn)) != cudaSuccess) return e;
  if (bn == 0.0) {
    cudaMemsetAsync(x, 0, (size_t)d.N * sizeof(double2), d.stream);
    res.iters = 0; res.rel_residual = 0.0; res.converged = true;
    hist.assign(1, 0.0);
    return cudaStreamSynchronize(d.stream);
  }
  hist.clear();
  int it = 0;
  bool conv = false;
  if ((e = arnoldi_cycle<double2>(d, ws, b, nullptr, x, max_iter, tol, 1e-300, bn, &hist, it, conv)) != cudaSuccess)
    return e;
  // True residual with the FP64 operator (the reference's "Err in GMRES").
  if ((e = dev_matvec(d, x, ws.b64.w, d.stream, false)) != cudaSuccess) return e;
  launch_pdl(sub_kernel<double2>, grid_for(d.N), 256, 0, d.stream, b, ws.b64.w, ws.b64.r, d.N);
  double rn = 0.0;
  if ((e = vnorm(ws.b64.r, d.N, ws, d.stream, rn)) != cudaSuccess) return e;
  res.iters = it;
  res.converged = conv;
  res.rel_residual = rn / bn;
  return cudaSuccess;
}

cudaError_t dev_gmres_restarted(DevOperator& d, const double2* b, double2* x, int m, int restarts) {
  GmresWorkspace& ws = workspace(d);
  cudaError_t e = ws.ensure(d.N, m);
  if (e == cudaSuccess) e = ws.b64.ensure(d.N, m);
  if (e != cudaSuccess) return e;
  double bn = 0.0;
  if ((e = vnorm(b, d.N, ws, d.stream, bn)) != cudaSuccess) return e;
  if (bn == 0.0) bn = 1.0;
  cudaMemsetAsync(x, 0, (size_t)d.N * sizeof(double2), d.stream);
  for (int r = 0; r < restarts; ++r) {
    int it = 0;
    bool conv = false;
    if ((e = arnoldi_cycle<double2>(d, ws, b, x, x, m, -1.0, 1e-8, bn, nullptr, it, conv)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Iterative refinement in FP64 around GMRES on the FP32 operator:
//   r = b - A64 x ; solve A32 d = r to a loose tolerance ; x += d
// until |b - A64 x| / |b| <= tol. The residual is always the FP64 one. The
// inner Arnoldi basis, its Gram-Schmidt and the Givens algebra are FP64 by
// default (d.inner_basis = LS_INNER_BASIS_F64): only the operator apply is
// FP32, with its vectors rounded on load and widened on store. With
// LS_INNER_BASIS_F32 the basis and its orthogonalisation are FP32 too
// (half the basis traffic). With a right preconditioner M the inner solves
// are flexible GMRES on A32 M, and with guess the iteration starts from
// x0 = guess(b) instead of 0.
cudaError_t dev_gmres_mixed_flex(DevOperator& d, const double2* b, double2* x, Precond32* M, Precond32* guess,
                                 int max_outer, int inner, double tol, std::vector<double>& hist, FlexReport& rep,
                                 double& relres) {
  const int n = d.N;
  const bool f64_basis = d.inner_basis == LS_INNER_BASIS_F64;
  GmresWorkspace& ws = workspace(d);
  cudaError_t e = ws.ensure(n, inner);
  if (e == cudaSuccess && !f64_basis) e = ws.b32.ensure(n, inner);
  if (e == cudaSuccess && (ws.b64.n != n || (f64_basis && ws.b64.cap < inner)))
    e = ws.b64.ensure(n, f64_basis ? inner : 1);
  if (e != cudaSuccess) return e;
  double2* r = ws.res;
  double bn = 0.0;
  if ((e = vnorm(b, n, ws, d.stream, bn)) != cudaSuccess) return e;
  hist.clear();
  rep = FlexReport();
  cudaMemsetAsync(x, 0, (size_t)n * sizeof(double2), d.stream);
  if (bn == 0.0) {  // b = 0: x = 0 exactly
    relres = 0.0;
    hist.push_back(0.0);
    return cudaStreamSynchronize(d.stream);
  }
  cudaMemcpyAsync(r, b, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream);
  relres = 1.0;
  if (guess && bn > 0.0) {
    // x0 = guess(b) in FP32; kept only if it beats x0 = 0.
    launch_pdl(to_f32_kernel, grid_for(n), 256, 0, d.stream, b, ws.res32, n);
    if ((e = guess->apply(ws.res32, ws.dx32, d.stream)) != cudaSuccess) return e;
    ++rep.n_precond;
    launch_pdl(add_f32_kernel, grid_for(n), 256, 0, d.stream, x, ws.dx32, n);
    if ((e = dev_matvec(d, x, ws.b64.w, d.stream, false)) != cudaSuccess) return e;
    ++rep.n_matvec;
    launch_pdl(sub_kernel<double2>, grid_for(n), 256, 0, d.stream, b, ws.b64.w, r, n);
    double rn = 0.0;
    if ((e = vnorm(r, n, ws, d.stream, rn)) != cudaSuccess) return e;
    rep.guess_residual = rn / bn;
    if (rep.guess_residual < 1.0) {
      relres = rep.guess_residual;
    } else {
      cudaMemsetAsync(x, 0, (size_t)n * sizeof(double2), d.stream);
      cudaMemcpyAsync(r, b, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream);
    }
  }
  hist.push_back(relres);
  for (int o = 0; o < max_outer && relres > tol; ++o) {
    int it = 0;
    bool conv = false;
    // Inner solve to roughly the FP32 operator accuracy. A preconditioned
    // cycle is capped at kFlexInner steps: a useful M converges well within
    // them, and a useless one costs no more than that before the outer test
    // below drops it.
    const double inner_tol = std::max(tol / std::max(relres, 1e-300), 1e-6);
    Precond32* Mo = (rep.fell_back || inner_tol >= kFlexPlainTol) ? nullptr : M;
    const int m_inner = Mo ? std::min(inner, kFlexInner) : inner;
    if (f64_basis) {
      if ((e = arnoldi_cycle<double2>(d, ws, r, nullptr, ws.dx64, m_inner, inner_tol, 1e-300,
                                      std::max(relres * bn, 1e-300), nullptr, it, conv, Mo, true)) != cudaSuccess)
        return e;
      launch_pdl(add_kernel, grid_for(n), 256, 0, d.stream, x, (const double2*)ws.dx64, n);
    } else {
      launch_pdl(to_f32_kernel, grid_for(n), 256, 0, d.stream, r, ws.res32, n);
      if ((e = arnoldi_cycle<float2>(d, ws, ws.res32, nullptr, ws.dx32, m_inner, inner_tol, 1e-300,
                                     std::max(relres * bn, 1e-300), nullptr, it, conv, Mo)) != cudaSuccess)
        return e;
      launch_pdl(add_f32_kernel, grid_for(n), 256, 0, d.stream, x, ws.dx32, n);
    }
    rep.n_matvec += it;
    if (Mo) rep.n_precond += it;
    if ((e = dev_matvec(d, x, ws.b64.w, d.stream, false)) != cudaSuccess) return e;
    ++rep.n_matvec;
    launch_pdl(sub_kernel<double2>, grid_for(n), 256, 0, d.stream, b, ws.b64.w, r, n);
    double rn = 0.0;
    if ((e = vnorm(r, n, ws, d.stream, rn)) != cudaSuccess) return e;
    const double prev = relres;
    relres = rn / bn;
    hist.push_back(relres);
    if (Mo && relres > 0.5 * prev) rep.fell_back = true;
  }
  return cudaSuccess;
}

cudaError_t dev_gmres_mixed(DevOperator& d, const double2* b, double2* x, int max_outer, int inner, double tol,
                            std::vector<double>& hist, int& n_matvec, double& relres) {
  FlexReport rep;
  cudaError_t e = dev_gmres_mixed_flex(d, b, x, nullptr, nullptr, max_outer, inner, tol, hist, rep, relres);
  n_matvec = rep.n_matvec;
  return e;
}

}  // namespace lsg
