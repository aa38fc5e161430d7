// Grid resampling between the operator's Chebyshev nodes and the square
// grid of the spectral neural operator, and the network used as a right
// preconditioner of the mixed-precision flexible GMRES (nn_precond.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "device.h"
#include "fno.h"
#include "ls_internal.h"

namespace lsg {

// Scale of the kappa input channel: the net sees kappa / kFnoKappaScale.
constexpr double kFnoKappaScale = 40.0;

// Grid point g = ix * G + iy sits at (x, y) = L (-1 + (2 ix + 1) / G, -1 + (2 iy + 1) / G).
// Nodes -> grid: the reference's Chebyshev-Q+ interpolation
// (GMRES_Hybrid/LippmannSchwinger/main/hybridTrueValidation_gmres.cpp:187-219):
// in the leaf that contains the point, c = Q^+ phi_leaf and
// psi(x) = sum_l c_l T_a(l)((x - cx) / r) T_b(l)((y - cy) / r). Folded here
// into one weight row per grid point: psi(g) = sum_r w[g][r] phi[leaf(g)][r].
struct GridSampler {
  int G = 0, rank = 0;
  float* w = nullptr;   // [G*G][rank]
  int* leaf = nullptr;  // [G*G]
  bool init(const HostOperator& h, int grid, std::string& err);
  void release();
  // out[v][g] = psi_v(g) for nvec FP64 vectors x[v * N ...] (device).
  cudaError_t sample(const double2* x, int nvec, long long N, float2* out, cudaStream_t s) const;
};

// Host side of the reference's Chebyshev-Q+ interpolation at arbitrary
// points (hybridTrueValidation_gmres.cpp:187-219): the containing leaf of a
// uniform tree (points on the domain's upper edges go to the last leaf) and
// the row w with psi(x, y) = sum_r w[r] phi[leaf * rank + r].
struct LeafInterpolator {
  const HostOperator& op;
  double L = 1.0, rad = 1.0;
  int rank = 0, side = 1;
  std::vector<double> cx, cy;
  std::vector<int> table;
  std::vector<std::pair<int, int>> bases;
  explicit LeafInterpolator(const HostOperator& h);
  int cell(double v) const;
  int row(double x, double y, double* w) const;  // returns the leaf
};

// Host computation of the weight rows and leaf of every grid point.
void grid_sampling_weights(const HostOperator& h, int grid, std::vector<float>& w, std::vector<int>& leaf);
// q at the grid points (host), from the operator's contrast plugin.
void grid_contrast(const ls_config& cfg, int grid, std::vector<float>& q);

// z = M(v) = v + N(v): the residual-like vector v is sampled on the grid,
// scaled to unit RMS, mapped by the network together with the contrast and
// kappa to the predicted correction A^-1 v - v (the multiple-scattering
// part of the density), interpolated back to the nodes (bicubic,
// Catmull-Rom) at the original scale, and added to v. A network that
// predicts nothing leaves M = I.
struct NnPrecond : Precond32 {
  FnoNet* net = nullptr;
  GridSampler gs;
  int N = 0;
  float2* nodes = nullptr;  // continuous grid coordinates of the nodes
  float* in = nullptr;      // [G*G][6]: q, field (2), kappa, x, y
  float* out = nullptr;     // [G*G][2]
  float* ssq = nullptr;     // |sampled field|^2
  int applies = 0;
  // Where the fused single-sample pass (one cooperative launch) is not
  // available, the network's layer-by-layer forward pass on (in, out) is
  // captured once as a CUDA graph and replayed by every application (its
  // 22 launches cost more than their kernels for one sample); recaptured
  // when the net's buffers move.
  cudaGraphExec_t fwd = nullptr;
  unsigned long long fwd_generation = 0;
  cudaError_t capture();
  bool init(const HostOperator& h, FnoNet* net, std::string& err);
  void release();
  cudaError_t apply(const float2* v, float2* z, cudaStream_t s) override;
};

}  // namespace lsg
