/*
 * ORACLE - TEST INFRASTRUCTURE ONLY.
 *
 * C interface of the CPU restatement of the reference DAFMM + GMRES path
 * (vaishna77/Lippmann_Schwinger_Solver, directory GMRES/). Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load
 * this library, and only as the checker or as the CPU baseline; the
 * product never links, loads or calls it.
 *
 * Parity status: pinned to the reference's own printed output. The
 * reference needs Eigen and Boost.Math, which are absent, so it cannot be
 * compiled and run here, and it ships no golden vectors or known-answer
 * tests. Its README (GMRES/Readme.md:43-60, 103-113) publishes the assembly
 * log of its default adaptive run: tree depth, level_LFR, number of points,
 * boxes per level and the largest NCA rank per level and direction. The
 * adaptive-tree restatement (ls_oracle_adaptive.cpp) reproduces all of
 * them, and on a uniform tree it reproduces this oracle's skeletons point
 * for point (tests/test_oracle_pinned.py). The numerical pieces are checked
 * independently: Bessel functions and Gauss-Legendre rules against
 * scipy/numpy, quadrature against scipy integration, the DAFMM matvec
 * against the dense getMatrixEntry2 operator (tests/test_oracle_*.py).
 */
#ifndef LS_ORACLE_H
#define LS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAX_BUMPS 8

/* Mirrors the positional arguments of GMRES/GMRES.cpp:321-333 (main) plus
 * the switches that the reference hard-codes (findPhi, the 6-digit text
 * round trip of the precomputations) and the seeded Gaussian-bump contrast. */
typedef struct {
  int nCones_LFR;
  int nChebNodes;
  int yes2DFMM;
  int TOL_POW;
  int degreeOfBases;
  int nLevelsUniform;
  int Qchoice;             /* 0..5 = reference contrasts; 6 = Gaussian bumps */
  int findPhi;             /* 1: LS operator I + k^2 q G; 0: bare G (scattered field) */
  int reference_rounding;  /* 1: round M and near blocks to 6 significant digits */
  int n_bumps;
  double L;
  double kappa;
  double bump_cx[ORA_MAX_BUMPS];
  double bump_cy[ORA_MAX_BUMPS];
  double bump_a[ORA_MAX_BUMPS];
  double bump_w[ORA_MAX_BUMPS];
} ora_cfg;

void* ora_create(const ora_cfg* cfg, char* err, int errlen);
void ora_destroy(void* h);
int ora_N(void* h);
int ora_nlevels(void* h);
int ora_level_lfr(void* h);
int ora_rank(void* h);
void ora_points(void* h, double* xy);
void ora_contrast(void* h, double* q);
void ora_rhs(void* h, double* b);
void ora_get_M(void* h, double* M);
void ora_get_near(void* h, double* B);
long ora_skeleton_dump(void* h, int* buf, long cap);
void ora_matvec(void* h, const double* x, double* y);
void ora_dense_matvec(void* h, const double* x, double* y);
int ora_gmres(void* h, const double* b, int max_iter, double tol, double* x,
              double* hist, int* iters);
int ora_gmres_restarted(void* h, const double* b, int m, int restarts, double* x);
void ora_set_threads(int n);
/* Stand-alone helpers exposed for unit tests of the restated math. */
void ora_gauss_legendre(int n, double* nodes, double* weights);
void ora_bessel_jy(int n, double x, double* j, double* y);
/* J_0..J_nmax, Y_0..Y_nmax by the recurrences of the far-field Hankel series. */
void ora_bessel_jy_orders(int nmax, double x, double* j, double* y);
void ora_colpiv_solve(int m, int n, const double* A, const double* b, double* x);

/* Adaptive tree (ls_oracle_adaptive.cpp): builds the contrast-adapted tree,
 * its 2:1 level restriction, interaction lists and NCA skeletons, and
 * reports the per-level statistics the reference prints while assembling.
 * head = {nLevels, level_LFR, N, records}; 7 ints per record. */
int ora_adaptive_report(const ora_cfg* cfg, int treeAdaptivity, int* head, int* rec, int cap);
/* Skeleton node sets of the same build (treeAdaptivity < 0: uniform tree of
 * nLevelsUniform levels); j, k, cone, then four length-prefixed lists. */
long ora_adaptive_skeletons(const ora_cfg* cfg, int treeAdaptivity, int* buf, long cap);
/* Far-field Bessel orders of the adaptive restatement: 1 = one library call
 * per order (the reference's pattern), 0 (default) = the recurrence shared
 * with the uniform oracle and the library. */
void ora_adaptive_set_per_order_bessel(int on);

#ifdef __cplusplus
}
#endif
#endif
