// Reference-style driver through the C++ facade: the same steps as
// GMRES/GMRES.cpp main (build the operator, b = RHS, GMRES, report the
// residual of the solution with one more matvec, write the solution as a
// result file), then ten incidence directions solved together, the
// double-float kernels behind the same product, the density interpolated
// at other points, and (given a weights file) the solve with the learned
// preconditioner. Prints one JSON line.
//
//   gmres_driver <nLevelsUniform> <kappa> <TOL_POW> <Qchoice> [result file] [network weights]
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "ls_dafmm.hpp"

int main(int argc, char** argv) {
  ls::inputsToDFMM in;
  ls::userkernel k;
  in.nLevelsUniform = argc > 1 ? std::atoi(argv[1]) : 4;
  k.kappa = argc > 2 ? std::atof(argv[2]) : 10.0;
  in.TOL_POW = argc > 3 ? std::atoi(argv[3]) : 8;
  k.Qchoice = argc > 4 ? std::atoi(argv[4]) : 0;
  try {
    ls::DFMM S(in, k);
    auto t0 = std::chrono::steady_clock::now();
    S.FMMTreeInitialisation();
    auto t1 = std::chrono::steady_clock::now();
    ls::Vec b = S.RHS(), x, Ax;
    ls::classGMRES G;
    double err = 0.0;
    int it = 0;
    std::vector<double> hist;
    G.gmres(&S, b, 400, 1e-10, x, err, it, hist);
    auto t2 = std::chrono::steady_clock::now();
    S.MatVecProduct(x, Ax);
    double rn = 0.0, bn = 0.0;
    for (size_t i = 0; i < b.size(); ++i) {
      rn += std::norm(b[i] - Ax[i]);
      bn += std::norm(b[i]);
    }
    ls::Vec xr;
    ls::RestartedGMRES(2, &S, 10, in, b, xr);
    double dx = 0.0, xn = 0.0;
    for (size_t i = 0; i < x.size(); ++i) {
      dx += std::norm(x[i] - xr[i]);
      xn += std::norm(x[i]);
    }
    // Several incidence directions at once, each checked with one FP64 product.
    std::vector<double> thetas;
    for (int m = 0; m < 10; ++m) thetas.push_back(2.0 * 3.141592653589793 * m / 10.0);
    std::vector<ls::Vec> Bs = S.RHSAngles(thetas), Xs;
    const int nmv = S.SolveBatched(Bs, Xs, 1e-8);
    double worst = 0.0;
    for (size_t j = 0; j < Bs.size(); ++j) {
      ls::Vec Ax2;
      S.MatVecProduct(Xs[j], Ax2);
      double rj = 0.0, bj = 0.0;
      for (int i = 0; i < S.N; ++i) {
        rj += std::norm(Bs[j][i] - Ax2[i]);
        bj += std::norm(Bs[j][i]);
      }
      worst = std::max(worst, std::sqrt(rj / bj));
    }
    // The double-float kernels behind MatVecProduct.
    S.setF64Kernels(LS_F64_DOUBLE_FLOAT);
    ls::Vec Axd;
    S.MatVecProduct(x, Axd);
    S.setF64Kernels(LS_F64_NATIVE);
    double dd = 0.0, an = 0.0;
    for (int i = 0; i < S.N; ++i) {
      dd += std::norm(Axd[i] - Ax[i]);
      an += std::norm(Ax[i]);
    }
    // The solution as the reference writes it (result/Phi_<restart>_<m>).
    if (argc > 5) ls::WriteResult(argv[5], x);
    // Interpolation at other points reproduces a field in the leaves' basis
    // span (total degree < degreeOfBases) exactly.
    ls::Vec poly(S.N);
    auto f = [](double px, double py) { return std::complex<double>(px * px * py - 0.5 * py, px * py * py + 0.25); };
    for (int i = 0; i < S.N; ++i) poly[i] = f(S.gridPoints[i].x, S.gridPoints[i].y);
    std::vector<ls::pts2D> pts;
    for (int i = 0; i < 100; ++i) pts.push_back({-0.99 + 0.0199 * i, 0.73 - 0.0147 * i});
    const ls::Vec at = S.Interpolate(pts, poly);
    double ie = 0.0;
    for (size_t i = 0; i < pts.size(); ++i) ie = std::max(ie, std::abs(at[i] - f(pts[i].x, pts[i].y)));
    // The learned preconditioner, when a weights file is given.
    double nn_res = -1.0;
    int nn_applies = -1;
    if (argc > 6) {
      ls::LearnedPreconditioner P(argv[6]);
      ls::Vec xn, Axn;
      const ls_nn_report rep = P.Solve(&S, b, xn, 1e-8);
      S.MatVecProduct(xn, Axn);
      double r2 = 0.0;
      for (int i = 0; i < S.N; ++i) r2 += std::norm(b[i] - Axn[i]);
      nn_res = std::sqrt(r2 / bn);
      nn_applies = rep.n_precond;
    }
    std::printf("{\"N\": %d, \"iters\": %d, \"estimate\": %.3e, \"residual\": %.3e, \"restarted_vs_tol\": %.3e, "
                "\"batched_max_residual\": %.3e, \"batched_applies\": %d, \"double_float_vs_native\": %.3e, "
                "\"interpolation_error\": %.3e, \"nn_residual\": %.3e, \"nn_network_applies\": %d, "
                "\"assemble_s\": %.3f, \"gmres_s\": %.4f}\n",
                S.N, it, err, std::sqrt(rn / bn), std::sqrt(dx / xn), worst, nmv, std::sqrt(dd / an), ie, nn_res,
                nn_applies, std::chrono::duration<double>(t1 - t0).count(),
                std::chrono::duration<double>(t2 - t1).count());
  } catch (const ls::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
    return 1;
  }
  return 0;
}
