// The assembly's precomputation quadratures on the GPU
// (NearFieldInteraction1::evaluateV, NearFieldInteraction1.hpp:98-128, and
// FarFieldInteraction::evaluateC, FarFieldInteraction.hpp:115-160, over the
// adaptive panel tree of domain2D.hpp:46-138).
//
// Every integral is over [-1,1]^2 with the host's adaptive rule (quad2d in
// assemble.cpp): a panel whose four children reproduce its 10 x 10
// Gauss-Legendre value within kQuadEps (absolute) is a leaf and contributes
// its own value; leaves are summed in depth-first order, children in the
// order (-,-), (+,-), (+,+), (-,+). The integrands:
//   near (kind 0): H0(k |X - p|) T_a(p_x) T_b(p_y), H0 = J0 + i Y0, for a
//                  target X in the source box's normalised coordinates;
//   far  (kind 1): J_n(k |p|) e^{-i n arg p} T_a(p_x) T_b(p_y).
// One warp per integral: the 100 points of a panel are spread over the
// lanes and summed with an xor butterfly, which leaves every lane the same
// bits, so all lanes take the same refinement decisions. The panels waiting
// to be visited sit on a per-warp stack in shared memory; a stack overflow
// or more than kQMaxPanels panels marks the batch failed (the host then
// integrates everything itself), so every loop ends.
//
// The values differ from the host's in the last bits (CUDA's j0 / y0 / j1
// against libstdc++'s, another summation order), which the 6-digit rounding
// of the reference's text cache removes in all but rare cases.

#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "ls_internal.h"

namespace lsg {

namespace {

constexpr int kQWarps = 8;                   // warps (integrals) per block
constexpr int kQStack = 96;                  // panels on a warp's stack
constexpr long long kQMaxPanels = 1 << 16;   // panels visited per integral before giving up
constexpr int kQOrder = 10;                  // Gauss-Legendre points per panel side
constexpr double kQEps = 1e-7;               // the host's refinement test

__constant__ double c_gx[kQOrder];
__constant__ double c_gw[kQOrder];

struct QPanel {
  double xc, yc, xr, yr, vr, vi;
};

// J_n(x), 0 <= n <= 15, x > 0: forward recurrence from J_0, J_1 where it is
// stable (x > n), else Miller's backward recurrence from order
// 2((max(n, x) + 20 + sqrt(60 max)) / 2), rescaled when it grows past 1e10
// and normalised to whichever of J_0, J_1 is larger (the same method as the
// host's bessel_jy_orders). The library's jn recurs forward for every
// order, which loses all digits of J_n(x) for x well below n.
__device__ double bessel_jn(int n, double x) {
  const double j0v = j0(x);
  if (n == 0) return j0v;
  const double j1v = j1(x);
  if (n == 1) return j1v;
  if (x > n) {
    double jm = j0v, jc = j1v;
    for (int k = 1; k < n; ++k) {
      const double jp = (2.0 * k / x) * jc - jm;
      jm = jc;
      jc = jp;
    }
    return jc;
  }
  const int base = n > (int)x ? n : (int)x;
  const int m = 2 * ((base + 20 + (int)sqrt(60.0 * base)) / 2);
  double fp = 0.0, f = 1.0, fn = 0.0, f1 = 0.0;
  for (int j = m; j > 0; --j) {
    const double fm = (2.0 * j / x) * f - fp;
    fp = f;
    f = fm;
    if (fabs(f) > 1e10) {
      f *= 1e-10;
      fp *= 1e-10;
      fn *= 1e-10;
      f1 *= 1e-10;
    }
    if (j == n) fn = fp;
    if (j == 1) f1 = fp;
  }
  // f = F_0, f1 = F_1, fn = F_n (all scaled alike)
  const double sc = fabs(j0v) >= fabs(j1v) ? j0v / f : j1v / f1;
  return fn * sc;
}

__device__ __forceinline__ void integrand(const QuadTask& t, double x, double y, double& fr, double& fi) {
  const double ta = cos((double)t.a * acos(x)), tb = cos((double)t.b * acos(y));
  if (t.kind == 0) {
    const double dx = t.xx - x, dy = t.xy - y;
    const double arg = t.k * sqrt(dx * dx + dy * dy);
    fr = (j0(arg) * ta) * tb;
    fi = (y0(arg) * ta) * tb;
  } else {
    const double arg = t.k * sqrt(x * x + y * y);
    const double th = atan2(y, x);
    const int an = t.n < 0 ? -t.n : t.n;
    double J = bessel_jn(an, arg);
    if (t.n < 0 && (an & 1)) J = -J;
    double s, c;
    sincos((double)t.n * th, &s, &c);
    fr = (J * c * ta) * tb;
    fi = (-J * s * ta) * tb;
  }
}

// The panel's 10 x 10 rule, summed over the warp (every lane gets the sum).
__device__ __forceinline__ void panel_value(const QuadTask& t, QPanel& p, int lane) {
  double sr = 0.0, si = 0.0;
  for (int q = lane; q < kQOrder * kQOrder; q += 32) {
    const int a = q / kQOrder, b = q - a * kQOrder;
    const double x = p.xc + p.xr * c_gx[a], y = p.yc + p.yr * c_gx[b];
    double fr, fi;
    integrand(t, x, y, fr, fi);
    const double w = c_gw[a] * c_gw[b];
    sr = fma(w, fr, sr);
    si = fma(w, fi, si);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  const double area = p.xr * p.yr;
  p.vr = sr * area;
  p.vi = si * area;
}

__global__ void __launch_bounds__(kQWarps * 32) quad_kernel(const QuadTask* __restrict__ tasks, int n_tasks,
                                                            double2* __restrict__ out, int* __restrict__ failed) {
  __shared__ QPanel stack[kQWarps][kQStack];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int task = blockIdx.x * kQWarps + warp;
  if (task >= n_tasks) return;
  const QuadTask t = tasks[task];
  QPanel* st = stack[warp];
  QPanel root{0.0, 0.0, 1.0, 1.0, 0.0, 0.0};
  panel_value(t, root, lane);
  if (lane == 0) st[0] = root;
  __syncwarp();
  int top = 1;
  long long visited = 0;
  double tr = 0.0, ti = 0.0;
  bool ok = true;
  while (top > 0) {
    const QPanel p = st[top - 1];
    __syncwarp();
    --top;
    if (++visited > kQMaxPanels || top + 4 > kQStack) {
      ok = false;
      break;
    }
    const double hx = 0.5 * p.xr, hy = 0.5 * p.yr;
    QPanel c[4] = {{p.xc - hx, p.yc - hy, hx, hy, 0.0, 0.0}, {p.xc + hx, p.yc - hy, hx, hy, 0.0, 0.0},
                   {p.xc + hx, p.yc + hy, hx, hy, 0.0, 0.0}, {p.xc - hx, p.yc + hy, hx, hy, 0.0, 0.0}};
    for (int l = 0; l < 4; ++l) panel_value(t, c[l], lane);
    double er = p.vr, ei = p.vi;
    for (int l = 0; l < 4; ++l) {
      er -= c[l].vr;
      ei -= c[l].vi;
    }
    if (hypot(er, ei) < kQEps) {
      tr += p.vr;
      ti += p.vi;
    } else {
      if (lane == 0)
        for (int l = 3; l >= 0; --l) st[top + (3 - l)] = c[l];
      __syncwarp();
      top += 4;
    }
  }
  if (lane == 0) {
    out[task] = make_double2(tr, ti);
    if (!ok) atomicOr(failed, 1);
  }
}

}  // namespace

bool gpu_quadrature(int device, const std::vector<QuadTask>& tasks, const std::vector<double>& gx,
                    const std::vector<double>& gw, std::vector<cd>& out) {
  if (device < 0 || tasks.empty() || (int)gx.size() != kQOrder || (int)gw.size() != kQOrder) return false;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const int n = (int)tasks.size();
  QuadTask* dt = nullptr;
  double2* dout = nullptr;
  int* dfail = nullptr;
  cudaStream_t s = nullptr;
  bool ok = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&dt, sizeof(QuadTask) * (size_t)n) == cudaSuccess &&
            cudaMalloc(&dout, sizeof(double2) * (size_t)n) == cudaSuccess &&
            cudaMalloc(&dfail, sizeof(int)) == cudaSuccess &&
            cudaMemcpyToSymbolAsync(c_gx, gx.data(), sizeof(double) * kQOrder, 0, cudaMemcpyHostToDevice, s) ==
                cudaSuccess &&
            cudaMemcpyToSymbolAsync(c_gw, gw.data(), sizeof(double) * kQOrder, 0, cudaMemcpyHostToDevice, s) ==
                cudaSuccess &&
            cudaMemcpyAsync(dt, tasks.data(), sizeof(QuadTask) * (size_t)n, cudaMemcpyHostToDevice, s) ==
                cudaSuccess &&
            cudaMemsetAsync(dfail, 0, sizeof(int), s) == cudaSuccess;
  std::vector<double2> h;
  int failed = 1;
  if (ok) {
    quad_kernel<<<(n + kQWarps - 1) / kQWarps, kQWarps * 32, 0, s>>>(dt, n, dout, dfail);
    h.resize((size_t)n);
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(h.data(), dout, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
         cudaMemcpyAsync(&failed, dfail, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
         cudaStreamSynchronize(s) == cudaSuccess && failed == 0;
  }
  cudaFree(dt);
  cudaFree(dout);
  cudaFree(dfail);
  if (s) cudaStreamDestroy(s);
  cudaGetLastError();
  if (!ok) return false;
  out.resize((size_t)n);
  for (int i = 0; i < n; ++i) out[i] = cd(h[i].x, h[i].y);
  return true;
}

}  // namespace lsg
