// ls_dafmm.hpp - C++ facade over the C ABI (ls_dafmm.h) with the reference's
// tree / matvec / GMRES API surface (vaishna77/Lippmann_Schwinger_Solver):
//
//   inputsToDFMM                 GMRES/GMRES.cpp:129-138
//   userkernel                   GMRES/GMRES.cpp:100-127 (contrast choice, plane wave, RHS)
//   DFMM                         GMRES/GMRES.cpp:140-255 (FMMTreeInitialisation, MatVecProduct)
//   GMRES / RestartedGMRES       GMRES/GMRES.cpp:257-319
//   classGMRES::gmres            GMRES_Hybrid/include/gmres.hpp:54-119
//
// Vec is std::vector<std::complex<double>> (contiguous interleaved complex,
// the layout of the reference's Eigen::VectorXcd). Header only; link with
// -llsdafmm. Errors throw ls::Error carrying the C ABI status and message.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ls_dafmm.h"
#include "ls_fno.h"

namespace ls {

using Vec = std::vector<std::complex<double>>;

struct pts2D {
  double x, y;
};

class Error : public std::runtime_error {
 public:
  Error(ls_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  ls_status status;
};

inline void check(ls_status s, const char* where) {
  if (s != LS_OK) throw Error(s, std::string(where) + ": " + ls_last_error());
}

struct inputsToDFMM {
  int nCones_LFR = 16;
  int nChebNodes = 6;
  double L = 1.0;
  int yes2DFMM = 1;
  int TOL_POW = 8;
  int degreeOfBases = 6;
  int treeAdaptivity = 5;  // adaptive tree: contrast resolved to 10^-treeAdaptivity
  int nLevelsUniform = 4;  // uniform tree: its depth
  // 1: the adaptive quadtree that GMRES/GMRES.cpp:164-165 builds
  // (createAdaptiveTree + makeLevelRestriction_Tree); 0: the uniform tree
  // of createUniformTree (the line the reference leaves commented out),
  // which the benchmark workloads use.
  int treeAdaptive = 0;
};

// Contrast plugin: Qchoice 0..5 as in the reference, 6 = Gaussian bumps.
struct userkernel {
  double kappa = 10.0;
  int Qchoice = 0;
  std::vector<double> bump_cx, bump_cy, bump_a, bump_w;
  std::complex<double> IncidenceFunction(const pts2D r) const {
    return std::exp(std::complex<double>(0.0, 1.0) * kappa * r.x);
  }
};

class DFMM {
 public:
  inputsToDFMM inputs;
  userkernel kernel;
  std::vector<pts2D> gridPoints;
  bool findPhi = true;
  int device = 0;
  ls_op* op = nullptr;
  int N = 0;

  DFMM(const inputsToDFMM& in, const userkernel& k) : inputs(in), kernel(k) {}
  DFMM(const DFMM&) = delete;
  DFMM& operator=(const DFMM&) = delete;
  ~DFMM() { ls_op_destroy(op); }

  ls_config config() const {
    ls_config c{};
    c.nCones_LFR = inputs.nCones_LFR;
    c.nChebNodes = inputs.nChebNodes;
    c.yes2DFMM = inputs.yes2DFMM;
    c.TOL_POW = inputs.TOL_POW;
    c.degreeOfBases = inputs.degreeOfBases;
    c.nLevelsUniform = inputs.nLevelsUniform;
    c.tree_adaptive = inputs.treeAdaptive;
    c.treeAdaptivity = inputs.treeAdaptivity;
    c.Qchoice = kernel.Qchoice;
    c.findPhi = findPhi ? 1 : 0;
    c.reference_rounding = 1;
    c.L = inputs.L;
    c.kappa = kernel.kappa;
    c.n_bumps = (int)kernel.bump_cx.size();
    for (int i = 0; i < c.n_bumps && i < LS_MAX_BUMPS; ++i) {
      c.bump_cx[i] = kernel.bump_cx[i];
      c.bump_cy[i] = kernel.bump_cy[i];
      c.bump_a[i] = kernel.bump_a[i];
      c.bump_w[i] = kernel.bump_w[i];
    }
    return c;
  }

  void FMMTreeInitialisation() {
    ls_config c = config();
    check(ls_op_create(&c, device, &op), "ls_op_create");
    ls_op_info_t info;
    check(ls_op_info(op, &info), "ls_op_info");
    N = info.N;
    std::vector<double> xy(2 * (size_t)N);
    check(ls_op_points(op, xy.data()), "ls_op_points");
    gridPoints.resize(N);
    for (int i = 0; i < N; ++i) gridPoints[i] = {xy[2 * i], xy[2 * i + 1]};
  }

  void MatVecProduct(const Vec& b, Vec& output) {
    output.resize(b.size());
    check(ls_matvec_host(op, reinterpret_cast<const double*>(b.data()), reinterpret_cast<double*>(output.data())),
          "ls_matvec_host");
  }

  Vec RHS() const {
    Vec b(N);
    check(ls_op_rhs(op, reinterpret_cast<double*>(b.data())), "ls_op_rhs");
    return b;
  }

  // Kernels behind the FP64 products (LS_F64_NATIVE or LS_F64_DOUBLE_FLOAT).
  void setF64Kernels(int kernels) { check(ls_op_set_f64_kernels(op, kernels), "ls_op_set_f64_kernels"); }

  // Right-hand sides for plane waves from the directions thetas (radians):
  // -kappa^2 q(x) exp(i kappa (x1 cos t + x2 sin t)); t = 0 is RHS().
  std::vector<Vec> RHSAngles(const std::vector<double>& thetas) const {
    std::vector<double> q(N);
    check(ls_op_contrast(op, q.data()), "ls_op_contrast");
    std::vector<Vec> out;
    const double k = kernel.kappa;
    for (double t : thetas) {
      Vec b(N);
      for (int i = 0; i < N; ++i) {
        const double ph = k * (gridPoints[i].x * std::cos(t) + gridPoints[i].y * std::sin(t));
        b[i] = -k * k * q[i] * std::exp(std::complex<double>(0.0, ph));
      }
      out.push_back(std::move(b));
    }
    return out;
  }

  // The density phi at other points, by the reference's Chebyshev-Q+
  // interpolation (hybridTrueValidation_gmres.cpp:187-219, "Psi_non_grid").
  Vec Interpolate(const std::vector<pts2D>& pts, const Vec& phi) const {
    std::vector<double> xy(2 * pts.size());
    for (size_t i = 0; i < pts.size(); ++i) {
      xy[2 * i] = pts[i].x;
      xy[2 * i + 1] = pts[i].y;
    }
    Vec out(pts.size());
    check(ls_op_interpolate(op, (int)pts.size(), xy.data(), reinterpret_cast<const double*>(phi.data()),
                            reinterpret_cast<double*>(out.data())),
          "ls_op_interpolate");
    return out;
  }

  // Solves for all right-hand sides together (mixed precision, FP64 residual
  // per column). Returns the number of FP32 block applies plus FP64 products.
  int SolveBatched(const std::vector<Vec>& B, std::vector<Vec>& X, double tol = 1e-8, int max_outer = 20,
                   int inner = 100) {
    check(ls_op_enable_f32(op), "ls_op_enable_f32");
    const int nrhs = (int)B.size();
    std::vector<std::complex<double>> flatB((size_t)N * nrhs), flatX((size_t)N * nrhs);
    for (int j = 0; j < nrhs; ++j) std::copy(B[j].begin(), B[j].end(), flatB.begin() + (size_t)j * N);
    int nmv = 0;
    std::vector<double> rr(nrhs);
    check(ls_gmres_mixed_batched(op, nrhs, reinterpret_cast<const double*>(flatB.data()), max_outer, inner, tol,
                                 reinterpret_cast<double*>(flatX.data()), &nmv, rr.data()),
          "ls_gmres_mixed_batched");
    X.assign(nrhs, Vec(N));
    for (int j = 0; j < nrhs; ++j) std::copy(flatX.begin() + (size_t)j * N, flatX.begin() + (size_t)(j + 1) * N, X[j].begin());
    return nmv;
  }
};

// Writes v as the reference's result files do (GMRES/GMRES.cpp:391-397):
// one "(re,im)" per line, six significant digits.
inline void WriteResult(const std::string& path, const Vec& v) {
  check(ls_write_result(path.c_str(), (int)v.size(), reinterpret_cast<const double*>(v.data())), "ls_write_result");
}

// The learned preconditioner (include/ls_fno.h): a spectral neural operator
// read from a weights file ("LSFNO001", five int32: grid, modes, layers,
// proj_width, dtype 0 = float32 / 1 = float16, then the parameters), used
// as initial guess and right preconditioner of the mixed-precision flexible
// GMRES. No counterpart in the reference, whose GMRES is unpreconditioned.
class LearnedPreconditioner {
 public:
  ls_fno* net = nullptr;

  LearnedPreconditioner(const std::string& path, int device = 0) {
    std::ifstream f(path, std::ios::binary);
    char magic[8];
    int32_t hdr[5];
    if (!f.read(magic, 8) || std::memcmp(magic, "LSFNO001", 8) != 0 ||
        !f.read(reinterpret_cast<char*>(hdr), sizeof hdr))
      throw Error(LS_E_INVALID, path + ": not a network weights file");
    ls_fno_config c{hdr[0], hdr[1], hdr[2], hdr[3]};
    check(ls_fno_create(&c, device, 0, &net), "ls_fno_create");
    long long n = 0;
    check(ls_fno_num_params(net, &n), "ls_fno_num_params");
    std::vector<float> p((size_t)n);
    if (hdr[4] == 1) {
      std::vector<uint16_t> h((size_t)n);
      if (!f.read(reinterpret_cast<char*>(h.data()), (std::streamsize)(2 * n))) throw Error(LS_E_INVALID, path + ": short");
      for (long long i = 0; i < n; ++i) p[(size_t)i] = half_to_float(h[(size_t)i]);
    } else if (!f.read(reinterpret_cast<char*>(p.data()), (std::streamsize)(4 * n))) {
      throw Error(LS_E_INVALID, path + ": short");
    }
    check(ls_fno_set_params(net, p.data()), "ls_fno_set_params");
  }
  LearnedPreconditioner(const LearnedPreconditioner&) = delete;
  LearnedPreconditioner& operator=(const LearnedPreconditioner&) = delete;
  ~LearnedPreconditioner() { ls_fno_destroy(net); }

  // Solves S x = b to the FP64 relative residual tol (flags: LS_NN_GUESS,
  // LS_NN_PRECOND); returns the solver's report.
  ls_nn_report Solve(class DFMM* S, const Vec& b, Vec& x, double tol = 1e-8,
                     int flags = LS_NN_GUESS | LS_NN_PRECOND, int max_outer = 20, int inner = 400);

  // IEEE 754 binary16 -> binary32.
  static float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    int e = (h >> 10) & 0x1f;
    uint32_t m = h & 0x3ffu, bits;
    if (e == 0x1f) {
      bits = sign | 0x7f800000u | (m << 13);
    } else if (e != 0) {
      bits = sign | ((uint32_t)(e - 15 + 127) << 23) | (m << 13);
    } else if (m == 0) {
      bits = sign;
    } else {  // subnormal: normalise
      e = -14;
      while (!(m & 0x400u)) {
        m <<= 1;
        --e;
      }
      m &= 0x3ffu;
      bits = sign | ((uint32_t)(e + 127) << 23) | (m << 13);
    }
    float out;
    std::memcpy(&out, &bits, sizeof out);
    return out;
  }
};

inline ls_nn_report LearnedPreconditioner::Solve(DFMM* S, const Vec& b, Vec& x, double tol, int flags, int max_outer,
                                                 int inner) {
  check(ls_op_enable_f32(S->op), "ls_op_enable_f32");
  x.resize(b.size());
  ls_nn_report rep{};
  const ls_status s = ls_fgmres_nn(S->op, net, reinterpret_cast<const double*>(b.data()), flags, max_outer, inner,
                                   tol, reinterpret_cast<double*>(x.data()), nullptr, &rep);
  if (s != LS_OK && s != LS_E_NOT_CONVERGED) check(s, "ls_fgmres_nn");
  return rep;
}

// Fixed-m GMRES with `restart` cycles, x0 = 0 (GMRES/GMRES.cpp:307-319).
inline void RestartedGMRES(int restart, DFMM* S, int m, const inputsToDFMM&, const Vec& b, Vec& solution) {
  solution.resize(b.size());
  check(ls_gmres_restarted(S->op, reinterpret_cast<const double*>(b.data()), m, restart,
                           reinterpret_cast<double*>(solution.data())),
        "ls_gmres_restarted");
}

class classGMRES {
 public:
  // Tolerance-stopped GMRES (GMRES_Hybrid/include/gmres.hpp:54): fills x,
  // the final residual estimate, the iteration count and the history.
  void gmres(DFMM* M, const Vec& b, int maxIterations, double threshold, Vec& x, double& error, int& noOfIterations,
             std::vector<double>& e) {
    x.resize(b.size());
    e.assign(maxIterations + 1, 0.0);
    double rel = 0.0;
    const ls_status s = ls_gmres(M->op, reinterpret_cast<const double*>(b.data()), maxIterations, threshold,
                                 reinterpret_cast<double*>(x.data()), e.data(), &noOfIterations, &rel);
    if (s != LS_OK && s != LS_E_NOT_CONVERGED) check(s, "ls_gmres");
    e.resize(noOfIterations + 1);
    error = e.empty() ? rel : e.back();
  }
};

}  // namespace ls
