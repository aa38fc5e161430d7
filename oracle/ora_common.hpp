// ORACLE - TEST INFRASTRUCTURE ONLY.
//
// Pieces shared by the uniform-tree oracle (ls_oracle.cpp) and the
// adaptive-tree oracle (ls_oracle_adaptive.cpp): complex dense algebra,
// pivoted QR, Bessel functions, Gauss-Legendre rules, the 6-digit text
// round trip, adaptive quadrature, the contrast plugin and the pivoted
// cross approximation of the reference. Parity unpinned at the vector
// level (see ls_oracle.h).
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "ls_oracle.h"

namespace ora {


using cd = std::complex<double>;
const double PI = 3.1415926535897932384;  // GMRES/ACA.hpp:14
const cd I(0.0, 1.0);                       // GMRES/ACA.hpp:10

struct Pt { double x, y; };
struct Pair { int x, y; };

// ---------------------------------------------------------------------------
// Dense complex matrix, column major.
struct CMat {
  int r = 0, c = 0;
  std::vector<cd> a;
  CMat() {}
  CMat(int rr, int cc) : r(rr), c(cc), a((size_t)rr * cc, cd(0.0, 0.0)) {}
  cd& operator()(int i, int j) { return a[(size_t)j * r + i]; }
  const cd& operator()(int i, int j) const { return a[(size_t)j * r + i]; }
};

// y += A * x (sequential column order).
inline void gemv_acc(const CMat& A, const cd* x, cd* y) {
  for (int j = 0; j < A.c; ++j) {
    const cd xj = x[j];
    const cd* col = &A.a[(size_t)j * A.r];
    for (int i = 0; i < A.r; ++i) y[i] += col[i] * xj;
  }
}

inline double vnorm(const std::vector<cd>& v) {
  double s = 0.0;
  for (const cd& z : v) s += std::norm(z);
  return std::sqrt(s);
}

// ---------------------------------------------------------------------------
// Householder QR with column pivoting (LAPACK xGEQP3 style with norm
// downdating), standing in for Eigen::ColPivHouseholderQR used at
// GMRES/G_FMM2DTree.hpp:2135, 2346, 3379, 3536 (Atilde) and
// GMRES/GMRES.cpp:299 (least squares). solve() returns the basic solution
// on the numerically nonzero pivots, the rest set to zero.
struct ColPivQR {
  int m = 0, n = 0, nzp = 0;
  CMat qr;
  std::vector<cd> tau;
  std::vector<int> perm;  // perm[k] = original column placed at position k

  void compute(const CMat& A) {
    m = A.r; n = A.c;
    qr = A;
    const int size = std::min(m, n);
    tau.assign(size, cd(0.0, 0.0));
    perm.resize(n);
    for (int j = 0; j < n; ++j) perm[j] = j;
    std::vector<double> nu(n), nd(n);
    double maxn = 0.0;
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int i = 0; i < m; ++i) s += std::norm(qr(i, j));
      nu[j] = nd[j] = std::sqrt(s);
      maxn = std::max(maxn, nu[j]);
    }
    const double eps = std::numeric_limits<double>::epsilon();
    const double thr_helper = (maxn * eps) * (maxn * eps) / double(std::max(m, 1));
    const double downdate_thr = std::sqrt(eps);
    nzp = size;
    std::vector<cd> tmp(n);
    for (int k = 0; k < size; ++k) {
      int p = k;
      for (int j = k + 1; j < n; ++j) if (nu[j] > nu[p]) p = j;
      if (nzp == size && nu[p] * nu[p] < thr_helper * double(m - k)) nzp = k;
      if (p != k) {
        for (int i = 0; i < m; ++i) std::swap(qr(i, k), qr(i, p));
        std::swap(nu[k], nu[p]);
        std::swap(nd[k], nd[p]);
        std::swap(perm[k], perm[p]);
      }
      // Reflector for qr(k:m, k): H = I - tau v v^H with v = [1; ess].
      cd c0 = qr(k, k);
      double tail = 0.0;
      for (int i = k + 1; i < m; ++i) tail += std::norm(qr(i, k));
      double beta;
      const double tiny = std::numeric_limits<double>::min();
      if (tail <= tiny && c0.imag() * c0.imag() <= tiny) {
        tau[k] = cd(0.0, 0.0);
        beta = c0.real();
        for (int i = k + 1; i < m; ++i) qr(i, k) = cd(0.0, 0.0);
      } else {
        beta = std::sqrt(std::norm(c0) + tail);
        if (c0.real() >= 0.0) beta = -beta;
        const cd d = c0 - beta;
        for (int i = k + 1; i < m; ++i) qr(i, k) = qr(i, k) / d;
        tau[k] = std::conj((beta - c0) / beta);
      }
      qr(k, k) = cd(beta, 0.0);
      // Apply H to the trailing columns.
      if (tau[k] != cd(0.0, 0.0)) {
        for (int j = k + 1; j < n; ++j) {
          cd t = qr(k, j);
          for (int i = k + 1; i < m; ++i) t += std::conj(qr(i, k)) * qr(i, j);
          tmp[j] = t;
        }
        for (int j = k + 1; j < n; ++j) {
          qr(k, j) -= tau[k] * tmp[j];
          for (int i = k + 1; i < m; ++i) qr(i, j) -= (tau[k] * qr(i, k)) * tmp[j];
        }
      }
      // Column-norm downdating (LAPACK working note 176).
      for (int j = k + 1; j < n; ++j) {
        if (nu[j] != 0.0) {
          double t = std::abs(qr(k, j)) / nu[j];
          t = (1.0 + t) * (1.0 - t);
          if (t < 0.0) t = 0.0;
          const double ratio = nu[j] / nd[j];
          const double t2 = t * ratio * ratio;
          if (t2 <= downdate_thr) {
            double s = 0.0;
            for (int i = k + 1; i < m; ++i) s += std::norm(qr(i, j));
            nd[j] = std::sqrt(s);
            nu[j] = nd[j];
          } else {
            nu[j] *= std::sqrt(t);
          }
        }
      }
    }
  }

  // x (length n) = argmin |A x - b| on the nonzero pivots.
  void solve(const cd* b, cd* x) const {
    std::vector<cd> c(b, b + m);
    for (int k = 0; k < nzp; ++k) {
      if (tau[k] == cd(0.0, 0.0)) continue;
      cd t = c[k];
      for (int i = k + 1; i < m; ++i) t += std::conj(qr(i, k)) * c[i];
      t *= tau[k];
      c[k] -= t;
      for (int i = k + 1; i < m; ++i) c[i] -= qr(i, k) * t;
    }
    for (int i = nzp - 1; i >= 0; --i) {
      cd s = c[i];
      for (int j = i + 1; j < nzp; ++j) s -= qr(i, j) * c[j];
      c[i] = s / qr(i, i);
    }
    for (int j = 0; j < n; ++j) x[j] = cd(0.0, 0.0);
    for (int k = 0; k < nzp; ++k) x[perm[k]] = c[k];
  }
};

// ---------------------------------------------------------------------------
// Special functions.

// GMRES/G_FMM2DTree.hpp:73-100: J_n, Y_n with the reflection rule for n < 0.
inline double besselJ(int n, double x) {
  if (n >= 0) return std::cyl_bessel_j(double(n), x);
  double t = std::cyl_bessel_j(double(-n), x);
  return ((-n) % 2 == 0) ? t : -t;
}
inline double besselY(int n, double x) {
  if (n >= 0) return std::cyl_neumann(double(n), x);
  double t = std::cyl_neumann(double(-n), x);
  return ((-n) % 2 == 0) ? t : -t;
}

// J_n(x) and Y_n(x) for n = 0 .. nmax (nmax <= 62) for the far-field
// Hankel series, from four library calls instead of one per order:
// J_0, J_1, Y_0, Y_1 from libstdc++; Y_n by forward recurrence (Y is the
// dominant solution); J_n by forward recurrence when x > nmax (below the
// turning point the recurrence is stable), else by Miller's backward
// recurrence from order 2((max(nmax, x) + 20 + sqrt(60 max)) / 2), scaled to
// whichever of J_0, J_1 is larger in magnitude (they never vanish
// together). Against libstdc++'s per-order values for x in [0.3, 250],
// n <= 15: J within 5e-14 and Y within 1e-13 of max_n |.|. Both this oracle
// and the library's assembler use exactly these operations.
inline void bessel_jy_orders(int nmax, double x, double* J, double* Y) {
  const double j0 = std::cyl_bessel_j(0.0, x), j1 = std::cyl_bessel_j(1.0, x);
  Y[0] = std::cyl_neumann(0.0, x);
  if (nmax >= 1) Y[1] = std::cyl_neumann(1.0, x);
  for (int n = 1; n < nmax; ++n) Y[n + 1] = (2.0 * n / x) * Y[n] - Y[n - 1];
  J[0] = j0;
  if (nmax >= 1) J[1] = j1;
  if (x > nmax) {
    for (int n = 1; n < nmax; ++n) J[n + 1] = (2.0 * n / x) * J[n] - J[n - 1];
    return;
  }
  const int base = nmax > (int)x ? nmax : (int)x;
  const int m = 2 * ((base + 20 + (int)std::sqrt(60.0 * base)) / 2);
  double F[64];
  double fp = 0.0, f = 1.0;
  for (int j = m; j > 0; --j) {
    const double fm = (2.0 * j / x) * f - fp;
    fp = f;
    f = fm;
    if (std::fabs(f) > 1e10) {
      f *= 1e-10;
      fp *= 1e-10;
      for (int i = j + 1; i <= nmax; ++i) F[i] *= 1e-10;
    }
    if (j <= nmax) F[j] = fp;
  }
  F[0] = f;
  const double s = (std::fabs(j0) >= std::fabs(j1) || nmax < 1) ? j0 / F[0] : j1 / F[1];
  for (int i = 0; i <= nmax; ++i) J[i] = F[i] * s;
}

// GMRES/G_FMM2DTree.hpp:670-672 (and FarFieldInteraction.hpp:96-98).
inline double chebT(double x, int n) { return std::cos(n * std::acos(x)); }

// Gauss-Legendre rule of order n on [-1, 1], computed by Newton iteration on
// P_n in long double. Nodes are stored in the interleaved order of the
// reference's table (GMRES/Gauss_Legendre_Nodes_and_Weights.hpp:17):
// pairs (-t_i, +t_i) from the centre outwards (a zero node first when n is
// odd).
inline void gauss_legendre(int n, std::vector<double>& nodes, std::vector<double>& weights) {
  std::vector<long double> t, w;
  for (int i = 1; i <= n; ++i) {
    long double x = std::cos(PI * (i - 0.25L) / (n + 0.5L));
    long double dp = 0.0L;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1.0L, p1 = x;
      for (int k = 2; k <= n; ++k) {
        long double p2 = ((2.0L * k - 1.0L) * x * p1 - (k - 1.0L) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = n * (x * p1 - p0) / (x * x - 1.0L);
      long double dx = p1 / dp;
      x -= dx;
      if (std::fabs((double)dx) < 1e-30) break;
    }
    {
      long double p0 = 1.0L, p1 = x;
      for (int k = 2; k <= n; ++k) {
        long double p2 = ((2.0L * k - 1.0L) * x * p1 - (k - 1.0L) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = n * (x * p1 - p0) / (x * x - 1.0L);
    }
    t.push_back(x);
    w.push_back(2.0L / ((1.0L - x * x) * dp * dp));
  }
  // t is descending from near +1; collect the non-negative roots ascending.
  std::vector<std::pair<long double, long double>> pos;
  for (int i = 0; i < n; ++i) if (t[i] >= 0.0L) pos.push_back({t[i], w[i]});
  std::sort(pos.begin(), pos.end());
  nodes.clear(); weights.clear();
  for (auto& pw : pos) {
    if (pw.first == 0.0L || std::fabs((double)pw.first) < 1e-300) {
      nodes.push_back(0.0); weights.push_back((double)pw.second);
    } else {
      nodes.push_back(-(double)pw.first); weights.push_back((double)pw.second);
      nodes.push_back((double)pw.first);  weights.push_back((double)pw.second);
    }
  }
}

// Rounds to 6 significant digits the way the reference's text round trip
// does: Eigen's operator<< at the default stream precision (printf %g with
// 6 digits) followed by operator>> (GMRES/G_FMM2DTree.hpp:1264-1270,
// 1304-1315, 1868-1950).
inline double round6(double v) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.6g", v);
  return std::strtod(buf, nullptr);
}
inline cd round6(cd v) { return cd(round6(v.real()), round6(v.imag())); }

// ---------------------------------------------------------------------------
// Adaptive 2-D Gauss-Legendre quadrature, GMRES/domain2D.hpp:7-138: each
// panel is integrated with a 10x10 rule; a panel whose four children
// reproduce its value within epsilon (absolute) becomes a leaf and
// contributes its own (parent) value.
template <class F>
inline cd adaptive_quad(const F& f, const std::vector<double>& gn, const std::vector<double>& gw,
                        double eps) {
  struct Panel { double xc, yc, xr, yr; cd val; };
  const int nn = (int)gn.size();
  auto integrate = [&](Panel& p) {
    cd s(0.0, 0.0);
    for (int m = 0; m < nn; ++m) {
      const double px = p.xc + p.xr * gn[m];
      for (int q = 0; q < nn; ++q) {
        const double py = p.yc + p.yr * gn[q];
        s += gw[m] * gw[q] * f(px, py);
      }
    }
    s *= (p.xr * p.yr);
    p.val = s;
  };
  Panel root{0.0, 0.0, 1.0, 1.0, cd(0.0, 0.0)};
  integrate(root);
  cd total(0.0, 0.0);
  // Depth-first recursion in the reference's child order (0,1,2,3).
  std::vector<Panel> stack;
  stack.push_back(root);
  // Explicit stack that reproduces the recursive visiting order: children
  // are pushed in reverse so that child 0 is refined first.
  while (!stack.empty()) {
    Panel p = stack.back();
    stack.pop_back();
    const double xr = 0.5 * p.xr, yr = 0.5 * p.yr;
    Panel ch[4] = {{p.xc - xr, p.yc - yr, xr, yr, cd()}, {p.xc + xr, p.yc - yr, xr, yr, cd()},
                   {p.xc + xr, p.yc + yr, xr, yr, cd()}, {p.xc - xr, p.yc + yr, xr, yr, cd()}};
    for (int l = 0; l < 4; ++l) integrate(ch[l]);
    cd err = p.val;
    for (int l = 0; l < 4; ++l) err -= ch[l].val;
    if (std::abs(err) < eps) {
      total += p.val;
    } else {
      for (int l = 3; l >= 0; --l) stack.push_back(ch[l]);
    }
  }
  return total;
}


// --- contrast plugin (GMRES/GMRES.cpp:5-117) ---
// --- contrast (GMRES/GMRES.cpp:5-117) ---
inline double contrast_value(const ora_cfg& cfg, Pt r) {
  switch (cfg.Qchoice) {
    case 0: { double R2 = r.x * r.x + r.y * r.y; return 1.5 * std::exp(-160.0 * R2); }
    case 1: {
      static const double cxs[20] = {-1.17182014706864, -0.861066625441127, -1.14533939124057,
        -0.856639124568525, -0.620066350133170, -0.457064031294315, -0.482782006538245,
        -0.635070123186999, 0.108594058866164, -0.0315722590552472, -0.177274727610547,
        0.0342987980936911, 0.369662097773613, 0.591444264226524, 0.401225715100565,
        0.666822699314234, 1.10327781188617, 0.827519268441487, 0.873411278211136, 1.09482906183464};
      static const double cys[20] = {-0.361066625441127, 0.0719520938231629, 0.354660608759432,
        1.14336087543147, -1.12006635013317, -0.457064031294315, 0.364929876813001,
        0.802261227250738, -0.394084977497864, -0.0315722590552472, 0.322725272389453,
        1.03429879809369, -1.13033790222639, 0.0137164199764117, 0.401225715100565,
        1.16682269931423, -0.345187707108795, -0.172480731558513, 0.373411278211136, 1.09482906183464};
      double q = 0.0, a = 0.0013;
      for (int i = 0; i < 20; ++i) {
        double R2 = (r.x - cxs[i]) * (r.x - cxs[i]) + (r.y - cys[i]) * (r.y - cys[i]);
        q += 1.5 * std::exp(-R2 / a);
      }
      return q;
    }
    case 2: {
      double C = 0.4987;
      double psi = 1.0 - (r.x - 0.15 * (1 - r.x * r.x)) * (r.x - 0.15 * (1 - r.x * r.x)) -
                   C * (1.0 + 0.3 * r.x) * (1.0 + 0.3 * r.x) * r.y * r.y;
      static const double aa[5] = {0.45, 0.195, 0.51, 0.195, 0.63};
      static const double xx[5] = {0.8, 0.54, -0.14, -0.5, 0.18};
      static const double yy[5] = {0.0, -0.28, 0.7, -0.01, 0.8};
      if (psi <= 0.05) return 0.0;
      double g = 0.0;
      for (int i = 0; i < 5; ++i) {
        double t = (r.x - xx[i]) * (r.x - xx[i]) + (r.y - yy[i]) * (r.y - yy[i]);
        g += aa[i] * std::exp(-t / 0.01);
      }
      return -1.5 * (psi - 0.05) - g * std::cos(0.9 * r.y);
    }
    case 3: { double R2 = r.x * r.x + r.y * r.y; return 0.5 * std::erfc(5.0 * (R2 - 1.0)); }
    case 4: {
      double R = std::sqrt(r.x * r.x + r.y * r.y);
      double th = std::atan2(r.y, r.x);
      return (1.0 - std::pow(std::sin(0.5 * th), 500)) * std::exp(-2000 * (0.1 - R * R) * (0.1 - R * R));
    }
    case 5: {
      double R = std::sqrt(r.x * r.x + r.y * r.y);
      return 4 * (r.y - 0.1) * (1.0 - std::erf(25.0 * (R - 0.3)));
    }
    default: {  // seeded Gaussian bumps: sum_k a_k exp(-|x - c_k|^2 / w_k^2)
      double q = 0.0;
      for (int k = 0; k < cfg.n_bumps; ++k) {
        double dx = r.x - cfg.bump_cx[k], dy = r.y - cfg.bump_cy[k];
        double R2 = dx * dx + dy * dy;
        q += cfg.bump_a[k] * std::exp(-R2 / (cfg.bump_w[k] * cfg.bump_w[k]));
      }
      return q;
    }
  }
}


// --- NCA: ACA_only_nodes, GMRES/ACA.hpp:253-481 ---
inline int argmax_abs(const std::vector<cd>& v, const std::set<int>& allowed) {
  // An empty set yields index 0: the reference dereferences begin() of an
  // empty std::set there, which reads the set's element count (0) with
  // libstdc++; the ACA loop then ends on rank == min(rows, cols).
  if (allowed.empty()) return 0;
  auto it = allowed.begin();
  int idx = *it;
  double mx = std::abs(v[idx]);
  for (; it != allowed.end(); ++it)
    if (std::abs(v[*it]) > mx) { idx = *it; mx = std::abs(v[idx]); }
  return idx;
}
inline cd dotc(const std::vector<cd>& a, const std::vector<cd>& b) {  // a^H b
  cd s(0.0, 0.0);
  for (size_t i = 0; i < a.size(); ++i) s += std::conj(a[i]) * b[i];
  return s;
}
// Returns rank; row_bases / col_bases index rows / cols; Ar = K(pivot rows, cols).
template <class E>
int aca_nodes(const std::vector<int>& rows, const std::vector<int>& cols, double eps, std::vector<int>& rb,
            std::vector<int>& cb, CMat* Ar, const E& entry) {
  const int N1 = (int)rows.size(), N2 = (int)cols.size();
  const int mn = std::min(N1, N2);
  int rank_ = 0;
  std::set<int> rrem, crem;
  for (int l = 0; l < N1; ++l) rrem.insert(l);
  for (int l = 0; l < N2; ++l) crem.insert(l);
  std::vector<std::vector<cd>> U, V, Arows;
  std::vector<cd> row(N2), col(N1), u, v;
  auto getRow = [&](int ri) { std::vector<cd> r(N2); for (int k = 0; k < N2; ++k) r[k] = entry(rows[ri], cols[k]); return r; };
  auto getCol = [&](int ci) { std::vector<cd> c(N1); for (int k = 0; k < N1; ++k) c[k] = entry(rows[k], cols[ci]); return c; };
  int ri = 0, ci = 0;
  if (N1 < N2) {
    int l;
    for (l = 0; l < N1; ++l) {
      ri = l;
      row = getRow(ri);
      ci = argmax_abs(row, crem);
      if (std::abs(row[ci]) > eps * std::pow(10, -1.0 * 0)) break;
    }
    if (l == N1) return 0;
    v.resize(N2);
    for (int s = 0; s < N2; ++s) v[s] = row[s] / row[ci];
    rb.push_back(ri); cb.push_back(ci);
    col = getCol(ci);
    u = col;
    U.push_back(u); V.push_back(v); Arows.push_back(row);
    crem.erase(ci); rrem.erase(ri);
    rank_ = 1;
    double normS = 0.0, prev = 1000.0;
    ri = argmax_abs(col, rrem);
    while (std::abs(row[ci]) > eps * std::pow(10, -1.0 * 0) && std::abs(col[ri]) > eps &&
           std::abs(prev - normS) >= eps * prev && rank_ < mn) {
      rb.push_back(ri);
      row = getRow(ri);
      std::vector<cd> row_temp = row;
      for (int l2 = 0; l2 < rank_; ++l2)
        for (int s = 0; s < (int)V[l2].size(); ++s) row[s] -= U[l2][ri] * V[l2][s];
      ci = argmax_abs(row, crem);
      cb.push_back(ci);
      for (int s = 0; s < (int)row.size(); ++s) v[s] = row[s] / row[ci];
      col = getCol(ci);
      for (int l2 = 0; l2 < rank_; ++l2)
        for (int s = 0; s < (int)U[l2].size(); ++s) col[s] -= V[l2][ci] * U[l2][s];
      u = col;
      if (vnorm(u) < 1e-8 || vnorm(v) < 1e-8) { rb.pop_back(); cb.pop_back(); break; }
      U.push_back(u); V.push_back(v); Arows.push_back(row_temp);
      ++rank_;
      crem.erase(ci); rrem.erase(ri);
      if (rank_ != 2) prev = normS;
      normS = std::pow(normS, 2) + std::pow(vnorm(u) * vnorm(v), 2);
      for (int l2 = 0; l2 < rank_; ++l2) normS += 2 * std::abs(dotc(U[l2], u) * dotc(V[l2], v));
      normS = std::sqrt(normS);
      ri = argmax_abs(col, rrem);
    }
  } else {
    int l;
    for (l = 0; l < N2; ++l) {
      ci = l;
      col = getCol(ci);
      ri = argmax_abs(col, rrem);
      if (std::abs(col[ri]) > eps * std::pow(10, -1.0 * 0)) break;
    }
    if (l == N2) return 0;
    cb.push_back(ci);
    v.resize(N1);
    for (int s = 0; s < N1; ++s) v[s] = col[s] / col[ri];
    rb.push_back(ri);
    row = getRow(ri);
    u = row;
    U.push_back(u); V.push_back(v); Arows.push_back(row);
    rank_ = 1;
    rrem.erase(ri); crem.erase(ci);
    double normS = 0.0, prev = 1000.0;
    ci = argmax_abs(row, crem);
    while (std::abs(row[ci]) > eps * std::pow(10, -1.0 * 0) && std::abs(col[ri]) > eps &&
           std::abs(prev - normS) >= eps * prev && rank_ < mn) {
      cb.push_back(ci);
      col = getCol(ci);
      for (int l2 = 0; l2 < rank_; ++l2)
        for (int s = 0; s < (int)V[l2].size(); ++s) col[s] -= U[l2][ci] * V[l2][s];
      ri = argmax_abs(col, rrem);
      rb.push_back(ri);
      for (int s = 0; s < (int)col.size(); ++s) v[s] = col[s] / col[ri];
      row = getRow(ri);
      std::vector<cd> row_temp = row;
      for (int l2 = 0; l2 < rank_; ++l2)
        for (int s = 0; s < (int)U[l2].size(); ++s) row[s] -= V[l2][ri] * U[l2][s];
      u = row;
      if (vnorm(u) < 1e-8 || vnorm(v) < 1e-8) { cb.pop_back(); rb.pop_back(); break; }
      U.push_back(u); V.push_back(v); Arows.push_back(row_temp);
      ++rank_;
      rrem.erase(ri); crem.erase(ci);
      if (rank_ != 2) prev = normS;
      normS = std::pow(normS, 2) + std::pow(vnorm(u) * vnorm(v), 2);
      for (int l2 = 0; l2 < rank_; ++l2) normS += 2 * std::abs(dotc(U[l2], u) * dotc(V[l2], v));
      normS = std::sqrt(normS);
      ci = argmax_abs(row, crem);
    }
  }
  if (Ar) {
    *Ar = CMat(rank_, N2);
    for (int a = 0; a < rank_; ++a)
      for (int b = 0; b < N2; ++b) (*Ar)(a, b) = Arows[a][b];
  }
  return rank_;
}



// ---------------------------------------------------------------------------
// GMRES and RestartedGMRES, GMRES/GMRES.cpp:257-319: m Arnoldi steps with
// modified Gram-Schmidt (H(i,j) = V_i^H W_j), early exit when
// |H(j+1,j)| < 1e-8, least squares by column-pivoted QR, x = x0 + V y;
// `restarts` cycles, each from the previous solution (x0 = 0 first).
template <class MV>
inline void restarted_gmres(int N, MV&& matvec, const cd* b, int m, int restarts, cd* x) {
  std::vector<cd> x0(N, cd(0.0, 0.0)), out(N);
  for (int rs = 0; rs < restarts; ++rs) {
    int mm = m;
    matvec(x0.data(), out.data());
    std::vector<cd> r0(N);
    for (int i = 0; i < N; ++i) r0[i] = b[i] - out[i];
    double beta = 0.0;
    for (int i = 0; i < N; ++i) beta += std::norm(r0[i]);
    beta = std::sqrt(beta);
    std::vector<std::vector<cd>> V(1, std::vector<cd>(N));
    for (int i = 0; i < N; ++i) V[0][i] = r0[i] / beta;
    CMat Hm(m + 1, m);
    std::vector<cd> w(N);
    for (int j = 0; j < m; ++j) {
      matvec(V[j].data(), w.data());
      for (int i = 0; i <= j; ++i) {
        cd s(0.0, 0.0);
        for (int t = 0; t < N; ++t) s += std::conj(V[i][t]) * w[t];
        Hm(i, j) = s;
        for (int t = 0; t < N; ++t) w[t] -= s * V[i][t];
      }
      double wn = 0.0;
      for (int t = 0; t < N; ++t) wn += std::norm(w[t]);
      Hm(j + 1, j) = std::sqrt(wn);
      if (std::abs(Hm(j + 1, j)) < 1e-8) { mm = j + 1; break; }
      V.push_back(std::vector<cd>(N));
      for (int t = 0; t < N; ++t) V[j + 1][t] = w[t] / Hm(j + 1, j);
    }
    CMat Hs(mm + 1, mm);
    for (int a = 0; a <= mm; ++a) for (int c = 0; c < mm; ++c) Hs(a, c) = Hm(a, c);
    std::vector<cd> be1(mm + 1, cd(0.0, 0.0)), ym(mm);
    be1[0] = beta;
    ColPivQR qr;
    qr.compute(Hs);
    qr.solve(be1.data(), ym.data());
    for (int t = 0; t < N; ++t) {
      cd s = x0[t];
      for (int c = 0; c < mm; ++c) s += V[c][t] * ym[c];
      x[t] = s;
    }
    for (int t = 0; t < N; ++t) x0[t] = x[t];
  }
}

}  // namespace ora
