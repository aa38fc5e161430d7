// Grid resampling kernels and the network preconditioner (nn_precond.h).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "nn_precond.h"

namespace lsg {

namespace {

// dst[v][g] (stride, offset in floats) = sum_r w[r][g] x[v][leaf(g) * rank + r]
// (weights stored node-major so that a warp's loads are contiguous);
// ssq[v] += |.|^2 when ssq is given. Grid y = vector.
template <class T>
__global__ void nodes_to_grid_kernel(int GG, int rank, const float* __restrict__ w, const int* __restrict__ leaf,
                                     const T* __restrict__ x, long long xstride, float* __restrict__ dst,
                                     int dstride, int doff, long long dvstride, float* __restrict__ ssq) {
  __shared__ float red[32];
  const int v = blockIdx.y;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  float ar = 0.f, ai = 0.f;
  if (g < GG) {
    const T* xl = x + v * xstride + (long long)leaf[g] * rank;
    for (int r = 0; r < rank; ++r) {
      const float c = w[(long long)r * GG + g];
      ar = fmaf(c, (float)xl[r].x, ar);
      ai = fmaf(c, (float)xl[r].y, ai);
    }
    float* d = dst + v * dvstride + (long long)g * dstride + doff;
    d[0] = ar;
    d[1] = ai;
  }
  if (!ssq) return;
  float acc = ar * ar + ai * ai;
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) a += red[i];
    atomicAdd(&ssq[v], a);
  }
}

__device__ __forceinline__ void catmull_rom(float t, float w[4]) {
  const float t2 = t * t, t3 = t2 * t;
  w[0] = 0.5f * (-t3 + 2.f * t2 - t);
  w[1] = 0.5f * (3.f * t3 - 5.f * t2 + 2.f);
  w[2] = 0.5f * (-3.f * t3 + 4.f * t2 + t);
  w[3] = 0.5f * (t3 - t2);
}

// z[i] = add[i] + bicubic interpolation of the grid field f ([G*G][2]) at
// node i, whose continuous grid coordinates are uv[i] (grid point ix at ix).
// Clears *ssq_reset (the preconditioner's accumulator, consumed by the
// kernels before this one) for the next application.
__global__ void grid_to_nodes_kernel(int N, int G, const float2* __restrict__ uv, const float* __restrict__ f,
                                     const float2* __restrict__ add, float2* __restrict__ z,
                                     float* __restrict__ ssq_reset) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (ssq_reset && i == 0) *ssq_reset = 0.f;
  if (i >= N) return;
  const float2 p = uv[i];
  const float fx = floorf(p.x), fy = floorf(p.y);
  float wx[4], wy[4];
  catmull_rom(p.x - fx, wx);
  catmull_rom(p.y - fy, wy);
  const int x0 = (int)fx - 1, y0 = (int)fy - 1;
  float ar = 0.f, ai = 0.f;
  if (add) {
    ar = add[i].x;
    ai = add[i].y;
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int ix = min(max(x0 + a, 0), G - 1);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int iy = min(max(y0 + b, 0), G - 1);
      const float c = wx[a] * wy[b];
      const long long g = (long long)ix * G + iy;
      ar = fmaf(c, f[2 * g], ar);
      ai = fmaf(c, f[2 * g + 1], ai);
    }
  }
  z[i] = make_float2(ar, ai);
}

double cheb_t(double x, int n) {
  double t0 = 1.0, t1 = x;
  if (n == 0) return t0;
  for (int k = 1; k < n; ++k) {
    const double t2 = 2.0 * x * t1 - t0;
    t0 = t1;
    t1 = t2;
  }
  return t1;
}

}  // namespace

LeafInterpolator::LeafInterpolator(const HostOperator& h) : op(h) {
  L = h.cfg.L;
  rank = h.rank;
  side = 1 << h.cfg.nLevelsUniform;
  rad = L / side;
  const int nl = h.n_leaves;
  // Leaf centres (mean of their nodes) and the leaf at each cell of the leaf grid.
  cx.assign(nl, 0.0);
  cy.assign(nl, 0.0);
  table.assign((size_t)side * side, 0);
  for (int t = 0; t < nl; ++t) {
    double sx = 0.0, sy = 0.0;
    for (int r = 0; r < rank; ++r) {
      sx += h.px[(size_t)t * rank + r];
      sy += h.py[(size_t)t * rank + r];
    }
    cx[t] = sx / rank;
    cy[t] = sy / rank;
    table[(size_t)cell(cx[t]) * side + cell(cy[t])] = t;
  }
  for (int d = 0; d < h.cfg.degreeOfBases; ++d)
    for (int a = 0; a < d + 1; ++a) bases.push_back({a, d - a});
}

int LeafInterpolator::cell(double v) const {
  return std::min(std::max((int)std::floor((v + L) / (2 * rad)), 0), side - 1);
}

int LeafInterpolator::row(double x, double y, double* w) const {
  const int t = table[(size_t)cell(x) * side + cell(y)];
  const double Px = (x - cx[t]) / rad, Py = (y - cy[t]) / rad;
  const int nb = (int)bases.size();
  double tb[64];
  for (int l = 0; l < nb && l < 64; ++l) tb[l] = cheb_t(Px, bases[l].first) * cheb_t(Py, bases[l].second);
  for (int r = 0; r < rank; ++r) {
    double s = 0.0;
    for (int l = 0; l < nb; ++l) s += tb[l] * op.Qpinv[(size_t)l * rank + r];
    w[r] = s;
  }
  return t;
}

void grid_sampling_weights(const HostOperator& h, int G, std::vector<float>& w, std::vector<int>& leaf) {
  const LeafInterpolator li(h);
  const double L = h.cfg.L;
  const int rank = h.rank;
  w.assign((size_t)G * G * rank, 0.f);
  leaf.assign((size_t)G * G, 0);
  std::vector<double> row(rank);
  for (int ix = 0; ix < G; ++ix)
    for (int iy = 0; iy < G; ++iy) {
      const int g = ix * G + iy;
      leaf[g] = li.row(L * (-1.0 + (2.0 * ix + 1.0) / G), L * (-1.0 + (2.0 * iy + 1.0) / G), row.data());
      for (int r = 0; r < rank; ++r) w[(size_t)g * rank + r] = (float)row[r];
    }
}

void grid_contrast(const ls_config& cfg, int G, std::vector<float>& q) {
  q.assign((size_t)G * G, 0.f);
  const double L = cfg.L;
  for (int ix = 0; ix < G; ++ix)
    for (int iy = 0; iy < G; ++iy)
      q[(size_t)ix * G + iy] = (float)contrast_at(cfg, L * (-1.0 + (2.0 * ix + 1.0) / G), L * (-1.0 + (2.0 * iy + 1.0) / G));
}

bool GridSampler::init(const HostOperator& h, int grid, std::string& err) {
  release();
  std::vector<float> hg, hw;
  std::vector<int> hl;
  grid_sampling_weights(h, grid, hg, hl);
  G = grid;
  rank = h.rank;
  const size_t GG = (size_t)grid * grid;
  hw.resize(hg.size());
  for (size_t g = 0; g < GG; ++g)
    for (int r = 0; r < rank; ++r) hw[(size_t)r * GG + g] = hg[g * rank + r];
  cudaError_t e = cudaMalloc(&w, hw.size() * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&leaf, hl.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(w, hw.data(), hw.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(leaf, hl.data(), hl.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    err = std::string("grid sampler upload: ") + cudaGetErrorString(e);
    release();
    return false;
  }
  return true;
}

void GridSampler::release() {
  cudaFree(w);
  cudaFree(leaf);
  w = nullptr;
  leaf = nullptr;
  G = rank = 0;
}

cudaError_t GridSampler::sample(const double2* x, int nvec, long long N, float2* out, cudaStream_t s) const {
  const int GG = G * G;
  nodes_to_grid_kernel<double2><<<dim3((unsigned)((GG + 255) / 256), (unsigned)nvec), 256, 0, s>>>(GG, rank, w, leaf, x, N, reinterpret_cast<float*>(out), 2, 0, 2LL * GG, nullptr);
  return cudaGetLastError();
}

bool NnPrecond::init(const HostOperator& h, FnoNet* n, std::string& err) {
  release();
  net = n;
  const int G = n->shape.grid;
  if (!gs.init(h, G, err)) return false;
  N = h.N;
  const long long GG = (long long)G * G;
  std::vector<float> hin((size_t)GG * kFnoIn, 0.f), q;
  grid_contrast(h.cfg, G, q);
  for (long long g = 0; g < GG; ++g) {
    const int ix = (int)(g / G), iy = (int)(g % G);
    float* f = &hin[(size_t)g * kFnoIn];
    f[0] = q[(size_t)g];
    f[3] = (float)(h.cfg.kappa / kFnoKappaScale);
    f[4] = (float)(-1.0 + (2.0 * ix + 1.0) / G);
    f[5] = (float)(-1.0 + (2.0 * iy + 1.0) / G);
  }
  std::vector<float2> uv((size_t)N);
  for (int i = 0; i < N; ++i)
    uv[i] = make_float2((float)((h.px[i] / h.cfg.L + 1.0) * 0.5 * G - 0.5),
                        (float)((h.py[i] / h.cfg.L + 1.0) * 0.5 * G - 0.5));
  cudaError_t e = cudaMalloc(&in, hin.size() * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&out, (size_t)GG * kFnoOut * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&ssq, sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(ssq, 0, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&nodes, uv.size() * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemcpy(in, hin.data(), hin.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(nodes, uv.data(), uv.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();  // the clear of ssq is asynchronous
  if (e != cudaSuccess) {
    err = std::string("preconditioner upload: ") + cudaGetErrorString(e);
    release();
    return false;
  }
  return true;
}

void NnPrecond::release() {
  if (fwd) cudaGraphExecDestroy(fwd);
  fwd = nullptr;
  gs.release();
  cudaFree(nodes);
  cudaFree(in);
  cudaFree(out);
  cudaFree(ssq);
  nodes = nullptr;
  in = out = ssq = nullptr;
  N = 0;
}

cudaError_t NnPrecond::capture() {
  if (fwd) cudaGraphExecDestroy(fwd);
  fwd = nullptr;
  cudaError_t e = net->ensure(1);  // no allocation may happen while capturing
  if (e != cudaSuccess) return e;
  cudaStream_t cs = nullptr;
  if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) return e;
  cudaGraph_t g = nullptr;
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const cudaError_t fe = net->forward(1, in, out, ssq, cs);
    e = cudaStreamEndCapture(cs, &g);
    if (fe != cudaSuccess) e = fe;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&fwd, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    fwd = nullptr;
    cudaGetLastError();
    return e;
  }
  fwd_generation = net->generation;
  return cudaSuccess;
}

cudaError_t NnPrecond::apply(const float2* v, float2* z, cudaStream_t s) {
  const int G = gs.G, GG = G * G;
  cudaError_t e;
  // ssq is zero here: set at init and cleared by the last kernel of every application.
  nodes_to_grid_kernel<float2><<<dim3((unsigned)((GG + 255) / 256), 1), 256, 0, s>>>(GG, gs.rank, gs.w, gs.leaf, v, 0, in, kFnoIn, 1, 0, ssq);
  if (net->fused_ok()) {
    // One cooperative launch for the whole network.
    if ((e = net->forward(1, in, out, ssq, s)) != cudaSuccess) return e;
  } else {
    if (!fwd || fwd_generation != net->generation || net->cap < 1) capture();
    if (fwd && fwd_generation == net->generation) {
      if ((e = cudaGraphLaunch(fwd, s)) != cudaSuccess) return e;
    } else if ((e = net->forward(1, in, out, ssq, s)) != cudaSuccess) {
      return e;
    }
  }
  grid_to_nodes_kernel<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(N, G, nodes, out, v, z, ssq);
  ++applies;
  return cudaGetLastError();
}

}  // namespace lsg
