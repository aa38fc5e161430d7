// GMRES driven by the device DAFMM matvec.
//
// The Krylov basis V (N x (m+1), column major) and all O(N) work live on
// the device. Orthogonalisation is classical Gram-Schmidt applied twice
// (CGS2): each pass is one multi-dot kernel (V^H w, deterministic
// two-stage reduction) and one update kernel (w -= V h). The tiny
// Hessenberg / Givens algebra runs on the host in FP64.
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

namespace lsg {

constexpr int kDotThreads = 128;
constexpr int kDotBlocks = 304;  // row chunks: partial sums per column (2 per SM)

struct GmresWorkspace {
  double2* V = nullptr;
  double2* w = nullptr;
  double2* r = nullptr;
  double2* dx = nullptr;   // correction of the mixed-precision refinement
  double2* res = nullptr;  // residual of the mixed-precision refinement
  double2* partial = nullptr;
  double2* h = nullptr;   // first CGS pass, then scratch
  double2* h2 = nullptr;  // second CGS pass
  double2* nrm = nullptr; // |w|^2
  cudaEvent_t copied = nullptr;  // step coefficients are on the host
  double2* pinned = nullptr;     // host: h (m+2), h2 (m+2), |w|^2 (1); page-locked so copies stay asynchronous
  int n = 0, cap = -1;
  void release() {
    cudaFree(V); cudaFree(w); cudaFree(r); cudaFree(dx); cudaFree(res); cudaFree(partial); cudaFree(h); cudaFree(h2);
    cudaFree(nrm);
    V = w = r = dx = res = partial = h = h2 = nrm = nullptr;
    if (copied) cudaEventDestroy(copied);
    copied = nullptr;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    n = 0;
    cap = -1;
  }
  // Buffers for n-vectors and up to m Arnoldi steps; kept between solves
  // and grown only when a solve needs more.
  cudaError_t ensure(int n_, int m) {
    if (n_ == n && m <= cap) return cudaSuccess;
    release();
    const size_t nb = (size_t)n_ * sizeof(double2);
    cudaError_t e = cudaMalloc(&V, nb * (m + 1));
    if (e == cudaSuccess) e = cudaMalloc(&w, nb);
    if (e == cudaSuccess) e = cudaMalloc(&r, nb);
    if (e == cudaSuccess) e = cudaMalloc(&dx, nb);
    if (e == cudaSuccess) e = cudaMalloc(&res, nb);
    if (e == cudaSuccess) e = cudaMalloc(&partial, (size_t)kDotBlocks * (m + 2) * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&h, (size_t)(m + 2) * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&h2, (size_t)(m + 2) * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&nrm, sizeof(double2));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&pinned, (size_t)(2 * (m + 2) + 1) * sizeof(double2));
    if (e != cudaSuccess) {
      release();
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


// partial[col * gridDim.x + block] = sum_{rows of block} conj(V[row, col]) * w[row].
// Block (x, y) owns a contiguous chunk of rows and the columns
// 8y .. 8y+7: each thread keeps eight sums, so it has eight independent
// loads of V in flight per row. GB300's FP64 pipe is narrow, so the warp
// reduction of the eight sums is a transposing butterfly: at each of the
// first three shuffle steps a lane keeps half of its columns and adds the
// partner's half, which leaves each group of four lanes one column (18
// FP64 adds per lane instead of 80). All orders are fixed: deterministic.
constexpr int kDotCols = 8;

__device__ __forceinline__ double2 shfl2(double2 v, int o) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}

__global__ void __launch_bounds__(kDotThreads) multidot_kernel(const double2* __restrict__ V, long long ldv, int ncols,
                                                               const double2* __restrict__ w, int n,
                                                               double2* __restrict__ partial) {
  __shared__ double2 red[kDotThreads / 32][kDotCols];
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * chunk;
  const int len = max(0, min(chunk, n - r0));
  const int c0 = blockIdx.y * kDotCols;
  const int nc = min(kDotCols, ncols - c0);
  double2 acc[kDotCols];
#pragma unroll
  for (int j = 0; j < kDotCols; ++j) acc[j] = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    const double2 b = w[r0 + i];
    double2 a[kDotCols];
#pragma unroll
    for (int j = 0; j < kDotCols; ++j)  // all loads first, so that they are in flight together
      a[j] = j < nc ? V[(size_t)(c0 + j) * ldv + r0 + i] : make_double2(0.0, 0.0);
#pragma unroll
    for (int j = 0; j < kDotCols; ++j) {
      acc[j].x = fma(a[j].x, b.x, acc[j].x);
      acc[j].x = fma(a[j].y, b.y, acc[j].x);
      acc[j].y = fma(a[j].x, b.y, acc[j].y);
      acc[j].y = fma(-a[j].y, b.x, acc[j].y);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // Butterfly: after the steps 16, 8, 4 lane l holds column
  // 4 * bit4(l) + 2 * bit3(l) + bit2(l); steps 2 and 1 finish its sum.
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const bool hi = lane & 16;
    const double2 keep = hi ? acc[j + 4] : acc[j];
    const double2 got = shfl2(hi ? acc[j] : acc[j + 4], 16);
    acc[j] = make_double2(keep.x + got.x, keep.y + got.y);
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const bool hi = lane & 8;
    const double2 keep = hi ? acc[j + 2] : acc[j];
    const double2 got = shfl2(hi ? acc[j] : acc[j + 2], 8);
    acc[j] = make_double2(keep.x + got.x, keep.y + got.y);
  }
  {
    const bool hi = lane & 4;
    const double2 keep = hi ? acc[1] : acc[0];
    const double2 got = shfl2(hi ? acc[0] : acc[1], 4);
    acc[0] = make_double2(keep.x + got.x, keep.y + got.y);
  }
  for (int o = 2; o > 0; o >>= 1) {
    const double2 got = shfl2(acc[0], o);
    acc[0] = make_double2(acc[0].x + got.x, acc[0].y + got.y);
  }
  if ((lane & 3) == 0) red[wid][((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1)] = acc[0];
  __syncthreads();
  if (threadIdx.x < nc) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kDotThreads / 32; ++k) { a += red[k][threadIdx.x].x; b += red[k][threadIdx.x].y; }
    partial[(size_t)(c0 + threadIdx.x) * gridDim.x + blockIdx.x] = make_double2(a, b);
  }
}

// out[col] (+)= sum_b partial[col * nb + b]: one warp per column, lanes
// stride over the partials, then a fixed shuffle tree (deterministic).
__global__ void reduce_partials_kernel(const double2* __restrict__ partial, int nb, int ncols,
                                       double2* __restrict__ out, int accumulate) {
  const int col = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (col >= ncols) return;
  double a = 0.0, b = 0.0;
  for (int k = lane; k < nb; k += 32) {
    const double2 p = partial[(size_t)col * nb + k];
    a += p.x;
    b += p.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    if (accumulate) { out[col].x += a; out[col].y += b; }
    else out[col] = make_double2(a, b);
  }
}

// w[i] += sign * sum_c V[i, c] * h[c]; the column loop is unrolled by 4 so
// that four independent loads of V are in flight per thread.
__global__ void __launch_bounds__(256) multi_axpy_kernel(double2* __restrict__ w, const double2* __restrict__ V,
                                                         long long ldv, int ncols, const double2* __restrict__ h,
                                                         int n, double sign) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double sr = 0.0, si = 0.0;
    int c = 0;
    for (; c + 4 <= ncols; c += 4) {
      const double2 v0 = V[(size_t)c * ldv + i], v1 = V[(size_t)(c + 1) * ldv + i];
      const double2 v2 = V[(size_t)(c + 2) * ldv + i], v3 = V[(size_t)(c + 3) * ldv + i];
      const double2 h0 = h[c], h1 = h[c + 1], h2 = h[c + 2], h3 = h[c + 3];
      sr = fma(v0.x, h0.x, sr); sr = fma(-v0.y, h0.y, sr); si = fma(v0.x, h0.y, si); si = fma(v0.y, h0.x, si);
      sr = fma(v1.x, h1.x, sr); sr = fma(-v1.y, h1.y, sr); si = fma(v1.x, h1.y, si); si = fma(v1.y, h1.x, si);
      sr = fma(v2.x, h2.x, sr); sr = fma(-v2.y, h2.y, sr); si = fma(v2.x, h2.y, si); si = fma(v2.y, h2.x, si);
      sr = fma(v3.x, h3.x, sr); sr = fma(-v3.y, h3.y, sr); si = fma(v3.x, h3.y, si); si = fma(v3.y, h3.x, si);
    }
    for (; c < ncols; ++c) {
      const double2 v = V[(size_t)c * ldv + i];
      const double2 hc = h[c];
      sr = fma(v.x, hc.x, sr);
      sr = fma(-v.y, hc.y, sr);
      si = fma(v.x, hc.y, si);
      si = fma(v.y, hc.x, si);
    }
    double2 o = w[i];
    o.x += sign * sr;
    o.y += sign * si;
    w[i] = o;
  }
}

__global__ void scale_kernel(const double2* __restrict__ a, double2* __restrict__ b, double s, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    b[i] = make_double2(a[i].x * s, a[i].y * s);
}

__global__ void sub_kernel(const double2* __restrict__ a, const double2* __restrict__ b, double2* __restrict__ c, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    c[i] = make_double2(a[i].x - b[i].x, a[i].y - b[i].y);
}

__global__ void add_inplace_kernel(double2* __restrict__ a, const double2* __restrict__ b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a[i].x += b[i].x;
    a[i].y += b[i].y;
  }
}

using cdh = std::complex<double>;

// b = a / sqrt(nrm->x), or zeros when the norm is zero (breakdown; the
// vector is then never used).
__global__ void scale_by_norm_kernel(const double2* __restrict__ a, double2* __restrict__ b,
                                     const double2* __restrict__ nrm, int n) {
  const double nn = nrm->x;
  const double s = nn > 0.0 ? 1.0 / sqrt(nn) : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    b[i] = make_double2(a[i].x * s, a[i].y * s);
}

int grid_for(int n) { return std::min((n + 255) / 256, 152 * 8); }

// h_dev[0:ncols) = V[:, 0:ncols)^H w
void multidot(const double2* V, long long ldv, int ncols, const double2* w, int n, double2* partial, double2* h_dev,
              int accumulate, cudaStream_t s) {
  multidot_kernel<<<dim3(kDotBlocks, (ncols + kDotCols - 1) / kDotCols), kDotThreads, 0, s>>>(V, ldv, ncols, w, n,
                                                                                              partial);
  reduce_partials_kernel<<<(ncols * 32 + 255) / 256, 256, 0, s>>>(partial, kDotBlocks, ncols, h_dev, accumulate);
}

cudaError_t vnorm(const double2* w, int n, double2* partial, double2* h_dev, cudaStream_t s, double& out) {
  multidot(w, n, 1, w, n, partial, h_dev, 0, s);
  double2 hv;
  cudaError_t e = cudaMemcpyAsync(&hv, h_dev, sizeof(double2), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  out = std::sqrt(hv.x);
  return cudaSuccess;
}

cudaError_t apply(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool f32) {
  return f32 ? dev_matvec_f32(d, x, y, s, false) : dev_matvec(d, x, y, s, false);
}

// One Arnoldi cycle from x0 (device, may be null for x0 = 0). Writes the
// updated solution into x. tol < 0 disables the residual stop; breakdown
// exits when H(k+1,k) < brk.
cudaError_t arnoldi_cycle(DevOperator& d, GmresWorkspace& ws, const double2* b, const double2* x0, double2* x, int m,
                          double tol, double brk, double bnorm, std::vector<double>* hist, int& iters,
                          bool& converged, bool f32) {
  cudaStream_t s = d.stream;
  const int n = d.N;
  cudaError_t e;
  // r = b - A x0
  if (x0) {
    if ((e = apply(d, x0, ws.w, s, f32)) != cudaSuccess) return e;
    sub_kernel<<<grid_for(n), 256, 0, s>>>(b, ws.w, ws.r, n);
  } else {
    cudaMemcpyAsync(ws.r, b, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, s);
  }
  double beta = 0.0;
  if ((e = vnorm(ws.r, n, ws.partial, ws.h, s, beta)) != cudaSuccess) return e;
  if (hist && hist->empty()) hist->push_back(beta / bnorm);
  converged = false;
  iters = 0;
  if (beta == 0.0) {
    if (x != x0) {
      if (x0) cudaMemcpyAsync(x, x0, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, s);
      else cudaMemsetAsync(x, 0, (size_t)n * sizeof(double2), s);
    }
    converged = true;
    return cudaStreamSynchronize(s);
  }
  scale_kernel<<<grid_for(n), 256, 0, s>>>(ws.r, ws.V, 1.0 / beta, n);
  std::vector<std::vector<cdh>> H;  // columns, already rotated
  std::vector<cdh> cs, sn, g(1, cdh(beta, 0.0));
  std::vector<double2> hbuf(m + 2);
  int K = 0;
  // The product A v_{k+1} only needs v_{k+1} = w / |w|, which the device
  // forms itself, so it is queued before the host waits for step k's
  // coefficients: the host's Givens work and the wait hide behind it. A
  // converged or broken-down cycle leaves one unused product behind.
  if ((e = apply(d, ws.V, ws.w, s, f32)) != cudaSuccess) return e;
  for (int k = 0; k < m; ++k) {
    // CGS2, both passes and the norm on the device; one copy back per step.
    multidot(ws.V, n, k + 1, ws.w, n, ws.partial, ws.h, 0, s);
    multi_axpy_kernel<<<grid_for(n), 256, 0, s>>>(ws.w, ws.V, n, k + 1, ws.h, n, -1.0);
    multidot(ws.V, n, k + 1, ws.w, n, ws.partial, ws.h2, 0, s);
    multi_axpy_kernel<<<grid_for(n), 256, 0, s>>>(ws.w, ws.V, n, k + 1, ws.h2, n, -1.0);
    multidot(ws.w, n, 1, ws.w, n, ws.partial, ws.nrm, 0, s);
    scale_by_norm_kernel<<<grid_for(n), 256, 0, s>>>(ws.w, ws.V + (size_t)(k + 1) * n, ws.nrm, n);
    double2* hp = ws.pinned;
    double2* hp2 = ws.pinned + (m + 2);
    double2* np = ws.pinned + 2 * (m + 2);
    cudaMemcpyAsync(hp, ws.h, (size_t)(k + 1) * sizeof(double2), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hp2, ws.h2, (size_t)(k + 1) * sizeof(double2), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(np, ws.nrm, sizeof(double2), cudaMemcpyDeviceToHost, s);
    if ((e = cudaEventRecord(ws.copied, s)) != cudaSuccess) return e;
    if (k + 1 < m && (e = apply(d, ws.V + (size_t)(k + 1) * n, ws.w, s, f32)) != cudaSuccess) return e;
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
  for (int i = 0; i < K; ++i) hbuf[i] = make_double2(y[i].real(), y[i].imag());
  cudaMemcpyAsync(ws.h, hbuf.data(), (size_t)K * sizeof(double2), cudaMemcpyHostToDevice, s);
  if (x0) {
    if (x != x0) cudaMemcpyAsync(x, x0, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, s);
  } else {
    cudaMemsetAsync(x, 0, (size_t)n * sizeof(double2), s);
  }
  multi_axpy_kernel<<<grid_for(n), 256, 0, s>>>(x, ws.V, n, K, ws.h, n, 1.0);
  iters = K;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

}  // namespace

cudaError_t dev_gmres(DevOperator& d, const double2* b, double2* x, int max_iter, double tol,
                      std::vector<double>& hist, GmresResult& res, bool use_f32) {
  GmresWorkspace& ws = workspace(d);
  cudaError_t e = ws.ensure(d.N, max_iter);
  if (e != cudaSuccess) return e;
  double bn = 0.0;
  if ((e = vnorm(b, d.N, ws.partial, ws.h, d.stream, bn)) != cudaSuccess) return e;
  if (bn == 0.0) {
    cudaMemsetAsync(x, 0, (size_t)d.N * sizeof(double2), d.stream);
    res.iters = 0; res.rel_residual = 0.0; res.converged = true;
    hist.assign(1, 0.0);
    return cudaStreamSynchronize(d.stream);
  }
  hist.clear();
  int it = 0;
  bool conv = false;
  if ((e = arnoldi_cycle(d, ws, b, nullptr, x, max_iter, tol, 1e-300, bn, &hist, it, conv, use_f32)) != cudaSuccess) return e;
  // True residual with the FP64 operator (the reference's "Err in GMRES").
  if ((e = dev_matvec(d, x, ws.w, d.stream, false)) != cudaSuccess) return e;
  sub_kernel<<<grid_for(d.N), 256, 0, d.stream>>>(b, ws.w, ws.r, d.N);
  double rn = 0.0;
  if ((e = vnorm(ws.r, d.N, ws.partial, ws.h, d.stream, rn)) != cudaSuccess) return e;
  res.iters = it;
  res.converged = conv;
  res.rel_residual = rn / bn;
  return cudaSuccess;
}

cudaError_t dev_gmres_restarted(DevOperator& d, const double2* b, double2* x, int m, int restarts) {
  GmresWorkspace& ws = workspace(d);
  cudaError_t e = ws.ensure(d.N, m);
  if (e != cudaSuccess) return e;
  double bn = 0.0;
  if ((e = vnorm(b, d.N, ws.partial, ws.h, d.stream, bn)) != cudaSuccess) return e;
  if (bn == 0.0) bn = 1.0;
  cudaMemsetAsync(x, 0, (size_t)d.N * sizeof(double2), d.stream);
  for (int r = 0; r < restarts; ++r) {
    int it = 0;
    bool conv = false;
    if ((e = arnoldi_cycle(d, ws, b, x, x, m, -1.0, 1e-8, bn, nullptr, it, conv, false)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Iterative refinement in FP64 around GMRES on the FP32 operator:
//   r = b - A64 x ; solve A32 d = r to a loose tolerance ; x += d
// until |b - A64 x| / |b| <= tol. The residual is always the FP64 one.
cudaError_t dev_gmres_mixed(DevOperator& d, const double2* b, double2* x, int max_outer, int inner, double tol,
                            std::vector<double>& hist, int& n_matvec, double& relres) {
  const int n = d.N;
  GmresWorkspace& ws = workspace(d);
  cudaError_t e = ws.ensure(n, inner);
  if (e != cudaSuccess) return e;
  // r and dx must survive the inner cycles, which use ws.r and ws.w.
  double2* r = ws.res;
  double2* dx = ws.dx;
  double bn = 0.0;
  if ((e = vnorm(b, n, ws.partial, ws.h, d.stream, bn)) != cudaSuccess) goto done;
  hist.clear();
  n_matvec = 0;
  cudaMemsetAsync(x, 0, (size_t)n * sizeof(double2), d.stream);
  cudaMemcpyAsync(r, b, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream);
  relres = 1.0;
  hist.push_back(1.0);
  for (int o = 0; o < max_outer && relres > tol; ++o) {
    int it = 0;
    bool conv = false;
    // Inner solve to roughly the FP32 operator accuracy.
    const double inner_tol = std::max(tol / std::max(relres, 1e-300), 1e-6);
    if ((e = arnoldi_cycle(d, ws, r, nullptr, dx, inner, inner_tol, 1e-300, std::max(relres * bn, 1e-300), nullptr, it,
                           conv, true)) != cudaSuccess)
      goto done;
    n_matvec += it;
    add_inplace_kernel<<<grid_for(n), 256, 0, d.stream>>>(x, dx, n);
    if ((e = dev_matvec(d, x, ws.w, d.stream, false)) != cudaSuccess) goto done;
    ++n_matvec;
    sub_kernel<<<grid_for(n), 256, 0, d.stream>>>(b, ws.w, r, n);
    double rn = 0.0;
    if ((e = vnorm(r, n, ws.partial, ws.h, d.stream, rn)) != cudaSuccess) goto done;
    relres = rn / bn;
    hist.push_back(relres);
  }
done:
  return e;
}

}  // namespace lsg
