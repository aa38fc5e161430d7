// Reference-style driver through the C++ facade: the same steps as
// GMRES/GMRES.cpp main (build the operator, b = RHS, GMRES, report the
// residual of the solution with one more matvec). Prints one JSON line.
//
//   gmres_driver <nLevelsUniform> <kappa> <TOL_POW> <Qchoice>
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
    std::printf("{\"N\": %d, \"iters\": %d, \"estimate\": %.3e, \"residual\": %.3e, \"restarted_vs_tol\": %.3e, "
                "\"assemble_s\": %.3f, \"gmres_s\": %.4f}\n",
                S.N, it, err, std::sqrt(rn / bn), std::sqrt(dx / xn),
                std::chrono::duration<double>(t1 - t0).count(), std::chrono::duration<double>(t2 - t1).count());
  } catch (const ls::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
    return 1;
  }
  return 0;
}
