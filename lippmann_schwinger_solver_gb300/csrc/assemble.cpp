// Host assembler of the DAFMM operator for a uniform quadtree.
//
// Builds, in this order, the pieces that the reference computes in
// DFMM::FMMTreeInitialisation (GMRES/GMRES.cpp:161-199):
//   * tree geometry, level_LFR and cones      G_FMM2DTree.hpp:293-328, 917-941, 1952-1974
//   * interaction lists (LFR and per cone)    G_FMM2DTree.hpp:1356-1498
//   * Chebyshev basis Q, Q^+, far moments M   FarFieldInteraction.hpp:115-160
//   * colleague near blocks                   NearFieldInteraction1.hpp:260-290, G_FMM2DTree.hpp:1773-1830
//   * NCA skeletons (ACA_only_nodes)          ACA.hpp:253-481, G_FMM2DTree.hpp:2062-2385, 3232-3571
//   * user check points                       G_FMM2DTree.hpp:3146-3230
//   * block fills                             G_FMM2DTree.hpp:2502, 2653, 2824, 3573-3880, 3944-4206
// and then lays the operator out for the GPU: every phase of the matvec
// becomes a list of gather-GEMV items over two flat buffers (skeleton
// charges and skeleton potentials). The per-box QR solves of the reference
// (Atilde^{-1}) are folded into the blocks: upward T = Atilde^{-1} Ar,
// downward W = L2L Atilde^{-1}, so the device never solves a system.
//
// Kernel entries, quadrature integrands and the ACA updates use the same
// floating-point expression order as the reference source (and the file
// is compiled with -ffp-contract=off), so skeleton choices are
// reproducible across hosts.

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include <omp.h>

#include "ls_internal.h"

namespace lsg {
namespace {

constexpr double kPi = 3.1415926535897932384;
const cd kI(0.0, 1.0);
constexpr int kSeries = 15;                 // FarFieldInteraction.hpp:55
constexpr double kQuadEps = 1e-7;           // FarFieldInteraction.hpp:37, NearFieldInteraction1.hpp:199
constexpr int kQuadOrder = 10;              // 10x10 Gauss-Legendre per panel
constexpr int kMaxChebOrder = 15;           // basis orders: degreeOfBases <= 10 (checked with nChebNodes <= 8)

// ---------------------------------------------------------------- special functions
// J_n(x), Y_n(x) for n = 0 .. nmax (nmax < 64) for the far-field Hankel
// series, from four library calls instead of one per order: J_0, J_1, Y_0,
// Y_1 from libstdc++; Y_n by forward recurrence (Y is the dominant
// solution); J_n by forward recurrence when x > nmax (stable below the
// turning point), else by Miller's backward recurrence from order
// 2((max(nmax, x) + 20 + sqrt(60 max)) / 2), scaled to whichever of J_0, J_1
// is larger in magnitude (they never vanish together). Against libstdc++'s
// per-order values for x in [0.3, 250], n <= 15: J within 5e-14 and Y
// within 1e-13 of max_n |.|. The CPU oracle performs exactly the same
// operations, so the two assemblers still pick the same skeletons.
void bessel_jy_orders(int nmax, double x, double* J, double* Y) {
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

double bes_j(int n, double x) {
  if (n >= 0) return std::cyl_bessel_j(double(n), x);
  const double t = std::cyl_bessel_j(double(-n), x);
  return ((-n) % 2 == 0) ? t : -t;
}
double bes_y(int n, double x) {
  if (n >= 0) return std::cyl_neumann(double(n), x);
  const double t = std::cyl_neumann(double(-n), x);
  return ((-n) % 2 == 0) ? t : -t;
}
double cheb_t(double x, int n) { return std::cos(n * std::acos(x)); }

// Gauss-Legendre nodes by Newton iteration on P_n in extended precision,
// ordered as pairs (-t, +t) from the centre outwards.
void gl_rule(int n, std::vector<double>& x, std::vector<double>& w) {
  std::vector<std::pair<long double, long double>> pos;
  for (int i = 1; i <= n; ++i) {
    long double t = std::cos(kPi * (i - 0.25L) / (n + 0.5L));
    long double d = 0.0L;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1.0L, p1 = t;
      for (int k = 2; k <= n; ++k) {
        const long double p2 = ((2.0L * k - 1.0L) * t * p1 - (k - 1.0L) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      d = n * (t * p1 - p0) / (t * t - 1.0L);
      const long double dt = p1 / d;
      t -= dt;
      if (std::fabs((double)dt) < 1e-30) break;
    }
    long double p0 = 1.0L, p1 = t;
    for (int k = 2; k <= n; ++k) {
      const long double p2 = ((2.0L * k - 1.0L) * t * p1 - (k - 1.0L) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    d = n * (t * p1 - p0) / (t * t - 1.0L);
    if (t >= 0.0L) pos.push_back({t, 2.0L / ((1.0L - t * t) * d * d)});
  }
  std::sort(pos.begin(), pos.end());
  x.clear();
  w.clear();
  for (auto& p : pos) {
    if (std::fabs((double)p.first) < 1e-300) {
      x.push_back(0.0);
      w.push_back((double)p.second);
    } else {
      x.push_back(-(double)p.first);
      w.push_back((double)p.second);
      x.push_back((double)p.first);
      w.push_back((double)p.second);
    }
  }
}

// 6-significant-digit round trip of the reference's text cache.
double round6(double v) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.6g", v);
  return std::strtod(buf, nullptr);
}

// Adaptive quadrature on [-1,1]^2 (domain2D.hpp:46-138): a panel whose four
// children reproduce its 10x10 value within eps becomes a leaf and
// contributes its own value; leaves are summed in depth-first order.
template <class F>
cd quad2d(const F& f, const std::vector<double>& gx, const std::vector<double>& gw) {
  struct P { double xc, yc, xr, yr; cd v; };
  const int n = (int)gx.size();
  auto integ = [&](P& p) {
    cd s(0.0, 0.0);
    for (int a = 0; a < n; ++a) {
      const double x = p.xc + p.xr * gx[a];
      for (int b = 0; b < n; ++b) {
        const double y = p.yc + p.yr * gx[b];
        s += gw[a] * gw[b] * f(x, y);
      }
    }
    s *= (p.xr * p.yr);
    p.v = s;
  };
  P root{0.0, 0.0, 1.0, 1.0, cd()};
  integ(root);
  cd total(0.0, 0.0);
  std::vector<P> todo{root};
  while (!todo.empty()) {
    P p = todo.back();
    todo.pop_back();
    const double hx = 0.5 * p.xr, hy = 0.5 * p.yr;
    P c[4] = {{p.xc - hx, p.yc - hy, hx, hy, cd()}, {p.xc + hx, p.yc - hy, hx, hy, cd()},
              {p.xc + hx, p.yc + hy, hx, hy, cd()}, {p.xc - hx, p.yc + hy, hx, hy, cd()}};
    for (auto& q : c) integ(q);
    cd e = p.v;
    for (auto& q : c) e -= q.v;
    if (std::abs(e) < kQuadEps) total += p.v;
    else for (int l = 3; l >= 0; --l) todo.push_back(c[l]);
  }
  return total;
}

thread_local int t_assembly_device = -1;
// Device for the precomputation quadratures of an assembly with cfg: its GPU
// when cfg asks for it (and there is one), else none.
int quadrature_device(const ls_config& cfg) { return cfg.precompute_on_gpu ? t_assembly_device : -1; }

// ---------------------------------------------------------------- precomputation cache
// The reference writes M and the near blocks to text files at 6 digits and
// reads them back (writeMToFile / writeNeighborInteractionsForLevel,
// G_FMM2DTree.hpp:1264-1270, 1868-1950), recomputing them on every run.
// Here a record holds the exact values an assembly computed, keyed on every
// input they depend on (the kind of record, kappa, radii and offsets as
// bits, Chebyshev nodes, basis degree, rounding, host or GPU integration),
// so an assembly that reads one is the same bit for bit. Files: "LSPC",
// format version, key length and bytes, value count, values (native
// doubles); written to a temporary name and renamed, checked key for key
// on reading (a file that does not match is a miss).
class PrecomputeCache {
 public:
  void set(const char* dir) {
    std::lock_guard<std::mutex> lk(mu_);
    on_ = dir != nullptr;
    dir_ = dir ? dir : "";
    mem_.clear();
    mem_bytes_ = 0;
  }
  bool enabled() {
    std::lock_guard<std::mutex> lk(mu_);
    return on_;
  }
  bool get(const std::string& key, std::vector<cd>& out) {
    std::string dir;
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (!on_) return false;
      auto it = mem_.find(key);
      if (it != mem_.end()) {
        out = it->second;
        ++hits_;
        return true;
      }
      dir = dir_;
    }
    if (!dir.empty() && read_file(dir, key, out)) {
      std::lock_guard<std::mutex> lk(mu_);
      if (mem_bytes_ + out.size() * sizeof(cd) > kMemCap) {
        mem_.clear();
        mem_bytes_ = 0;
      }
      if (!mem_.count(key)) {
        mem_[key] = out;
        mem_bytes_ += out.size() * sizeof(cd);
      }
      ++hits_;
      return true;
    }
    std::lock_guard<std::mutex> lk(mu_);
    ++misses_;
    return false;
  }
  void put(const std::string& key, const std::vector<cd>& v) {
    std::string dir;
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (!on_) return;
      // Records held in memory are capped: past the cap they are dropped
      // (files, when there is a directory, still serve them).
      if (mem_bytes_ + v.size() * sizeof(cd) > kMemCap) {
        mem_.clear();
        mem_bytes_ = 0;
      }
      auto it = mem_.find(key);
      if (it != mem_.end()) mem_bytes_ -= it->second.size() * sizeof(cd);
      mem_[key] = v;
      mem_bytes_ += v.size() * sizeof(cd);
      dir = dir_;
    }
    if (!dir.empty()) write_file(dir, key, v);
  }
  void stats(long long& h, long long& m) {
    std::lock_guard<std::mutex> lk(mu_);
    h = hits_;
    m = misses_;
  }

 private:
  static constexpr uint32_t kVersion = 1;
  static constexpr size_t kMemCap = size_t(2) << 30;  // bytes of records held in memory
  static std::string path(const std::string& dir, const std::string& key) {
    uint64_t h = 1469598103934665603ULL;  // FNV-1a
    for (unsigned char c : key) h = (h ^ c) * 1099511628211ULL;
    char name[40];
    std::snprintf(name, sizeof(name), "/%016llx.lspc", (unsigned long long)h);
    return dir + name;
  }
  static bool read_file(const std::string& dir, const std::string& key, std::vector<cd>& out) {
    FILE* f = std::fopen(path(dir, key).c_str(), "rb");
    if (!f) return false;
    char magic[4];
    uint32_t ver = 0;
    uint64_t klen = 0, n = 0;
    bool ok = std::fread(magic, 1, 4, f) == 4 && std::memcmp(magic, "LSPC", 4) == 0 &&
              std::fread(&ver, sizeof(ver), 1, f) == 1 && ver == kVersion && std::fread(&klen, sizeof(klen), 1, f) == 1 &&
              klen == key.size();
    std::string k;
    if (ok) {
      k.resize(klen);
      ok = std::fread(&k[0], 1, klen, f) == klen && k == key && std::fread(&n, sizeof(n), 1, f) == 1 &&
           n <= (uint64_t(1) << 32);
    }
    if (ok) {
      std::vector<cd> v((size_t)n);
      ok = std::fread(v.data(), sizeof(cd), (size_t)n, f) == n && std::fgetc(f) == EOF;
      if (ok) out.swap(v);
    }
    std::fclose(f);
    return ok;
  }
  static void write_file(const std::string& dir, const std::string& key, const std::vector<cd>& v) {
    const std::string final_path = path(dir, key);
    char suffix[64];
    std::snprintf(suffix, sizeof(suffix), ".tmp%llu", (unsigned long long)std::hash<std::thread::id>()(
                                                          std::this_thread::get_id()));
    const std::string tmp = final_path + suffix;
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;
    const uint32_t ver = kVersion;
    const uint64_t klen = key.size(), n = v.size();
    const bool ok = std::fwrite("LSPC", 1, 4, f) == 4 && std::fwrite(&ver, sizeof(ver), 1, f) == 1 &&
                    std::fwrite(&klen, sizeof(klen), 1, f) == 1 && std::fwrite(key.data(), 1, klen, f) == klen &&
                    std::fwrite(&n, sizeof(n), 1, f) == 1 && std::fwrite(v.data(), sizeof(cd), n, f) == n;
    if (std::fclose(f) == 0 && ok)
      std::rename(tmp.c_str(), final_path.c_str());
    else
      std::remove(tmp.c_str());
  }
  std::mutex mu_;
  bool on_ = false;
  std::string dir_;
  std::map<std::string, std::vector<cd>> mem_;
  size_t mem_bytes_ = 0;
  long long hits_ = 0, misses_ = 0;
};
PrecomputeCache g_pcache;

// Key of a precomputation record: its kind, then doubles (as bits) and ints.
std::string pc_key(const char* kind, std::initializer_list<double> ds, std::initializer_list<int> is) {
  std::string k(kind);
  k.push_back('\0');
  for (double d : ds) k.append(reinterpret_cast<const char*>(&d), sizeof(double));
  for (int i : is) k.append(reinterpret_cast<const char*>(&i), sizeof(int));
  return k;
}
// Largest far-field sum table tabulated for far_on_gpu (host and device copies).
constexpr size_t kFarTableMaxBytes = size_t(4) << 30;
// Rank capacity of a GPU NCA block (its scratch holds this many pivot
// vectors); the host redoes the rare block that passes it.
constexpr int kNcaRankCap = 48;

// ---------------------------------------------------------------- small dense QR
// Column-pivoted Householder QR (xGEQP3 with norm downdating); solve()
// returns the basic least-squares solution on the nonzero pivots.
struct PivQR {
  int m = 0, n = 0, nz = 0;
  std::vector<cd> a;  // column major m x n
  std::vector<cd> tau;
  std::vector<int> perm;
  cd& at(int i, int j) { return a[(size_t)j * m + i]; }
  const cd& at(int i, int j) const { return a[(size_t)j * m + i]; }

  void factor(int rows, int cols, const std::vector<cd>& colmajor) {
    m = rows;
    n = cols;
    a = colmajor;
    const int sz = std::min(m, n);
    tau.assign(sz, cd(0.0, 0.0));
    perm.resize(n);
    for (int j = 0; j < n; ++j) perm[j] = j;
    std::vector<double> upd(n), dir(n);
    double big = 0.0;
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int i = 0; i < m; ++i) s += std::norm(at(i, j));
      upd[j] = dir[j] = std::sqrt(s);
      big = std::max(big, upd[j]);
    }
    const double eps = std::numeric_limits<double>::epsilon();
    const double helper = (big * eps) * (big * eps) / double(std::max(m, 1));
    const double dthr = std::sqrt(eps);
    nz = sz;
    std::vector<cd> t(n);
    for (int k = 0; k < sz; ++k) {
      int p = k;
      for (int j = k + 1; j < n; ++j)
        if (upd[j] > upd[p]) p = j;
      if (nz == sz && upd[p] * upd[p] < helper * double(m - k)) nz = k;
      if (p != k) {
        for (int i = 0; i < m; ++i) std::swap(at(i, k), at(i, p));
        std::swap(upd[k], upd[p]);
        std::swap(dir[k], dir[p]);
        std::swap(perm[k], perm[p]);
      }
      const cd c0 = at(k, k);
      double tail = 0.0;
      for (int i = k + 1; i < m; ++i) tail += std::norm(at(i, k));
      double beta;
      const double tiny = std::numeric_limits<double>::min();
      if (tail <= tiny && c0.imag() * c0.imag() <= tiny) {
        tau[k] = cd(0.0, 0.0);
        beta = c0.real();
        for (int i = k + 1; i < m; ++i) at(i, k) = cd(0.0, 0.0);
      } else {
        beta = std::sqrt(std::norm(c0) + tail);
        if (c0.real() >= 0.0) beta = -beta;
        const cd d = c0 - beta;
        for (int i = k + 1; i < m; ++i) at(i, k) = at(i, k) / d;
        tau[k] = std::conj((beta - c0) / beta);
      }
      at(k, k) = cd(beta, 0.0);
      if (tau[k] != cd(0.0, 0.0)) {
        for (int j = k + 1; j < n; ++j) {
          cd s = at(k, j);
          for (int i = k + 1; i < m; ++i) s += std::conj(at(i, k)) * at(i, j);
          t[j] = s;
        }
        for (int j = k + 1; j < n; ++j) {
          at(k, j) -= tau[k] * t[j];
          for (int i = k + 1; i < m; ++i) at(i, j) -= (tau[k] * at(i, k)) * t[j];
        }
      }
      for (int j = k + 1; j < n; ++j) {
        if (upd[j] != 0.0) {
          double r = std::abs(at(k, j)) / upd[j];
          r = (1.0 + r) * (1.0 - r);
          if (r < 0.0) r = 0.0;
          const double q = upd[j] / dir[j];
          if (r * q * q <= dthr) {
            double s = 0.0;
            for (int i = k + 1; i < m; ++i) s += std::norm(at(i, j));
            dir[j] = std::sqrt(s);
            upd[j] = dir[j];
          } else {
            upd[j] *= std::sqrt(r);
          }
        }
      }
    }
  }

  void solve(const cd* b, cd* x) const {
    std::vector<cd> c(b, b + m);
    for (int k = 0; k < nz; ++k) {
      if (tau[k] == cd(0.0, 0.0)) continue;
      cd s = c[k];
      for (int i = k + 1; i < m; ++i) s += std::conj(at(i, k)) * c[i];
      s *= tau[k];
      c[k] -= s;
      for (int i = k + 1; i < m; ++i) c[i] -= at(i, k) * s;
    }
    for (int i = nz - 1; i >= 0; --i) {
      cd s = c[i];
      for (int j = i + 1; j < nz; ++j) s -= at(i, j) * c[j];
      c[i] = s / at(i, i);
    }
    for (int j = 0; j < n; ++j) x[j] = cd(0.0, 0.0);
    for (int k = 0; k < nz; ++k) x[perm[k]] = c[k];
  }
};

// ---------------------------------------------------------------- contrast plugin
double contrast_fn(const ls_config& c, double x, double y) {
  switch (c.Qchoice) {
    case 0: {
      const double R2 = x * x + y * y;
      return 1.5 * std::exp(-160.0 * R2);
    }
    case 1: {
      static const double cx[20] = {-1.17182014706864, -0.861066625441127, -1.14533939124057,
        -0.856639124568525, -0.620066350133170, -0.457064031294315, -0.482782006538245,
        -0.635070123186999, 0.108594058866164, -0.0315722590552472, -0.177274727610547,
        0.0342987980936911, 0.369662097773613, 0.591444264226524, 0.401225715100565,
        0.666822699314234, 1.10327781188617, 0.827519268441487, 0.873411278211136, 1.09482906183464};
      static const double cy[20] = {-0.361066625441127, 0.0719520938231629, 0.354660608759432,
        1.14336087543147, -1.12006635013317, -0.457064031294315, 0.364929876813001,
        0.802261227250738, -0.394084977497864, -0.0315722590552472, 0.322725272389453,
        1.03429879809369, -1.13033790222639, 0.0137164199764117, 0.401225715100565,
        1.16682269931423, -0.345187707108795, -0.172480731558513, 0.373411278211136, 1.09482906183464};
      double q = 0.0;
      const double a = 0.0013;
      for (int i = 0; i < 20; ++i) {
        const double R2 = (x - cx[i]) * (x - cx[i]) + (y - cy[i]) * (y - cy[i]);
        q += 1.5 * std::exp(-R2 / a);
      }
      return q;
    }
    case 2: {
      const double C = 0.4987;
      const double psi = 1.0 - (x - 0.15 * (1 - x * x)) * (x - 0.15 * (1 - x * x)) -
                         C * (1.0 + 0.3 * x) * (1.0 + 0.3 * x) * y * y;
      static const double aa[5] = {0.45, 0.195, 0.51, 0.195, 0.63};
      static const double xs[5] = {0.8, 0.54, -0.14, -0.5, 0.18};
      static const double ys[5] = {0.0, -0.28, 0.7, -0.01, 0.8};
      if (psi <= 0.05) return 0.0;
      double g = 0.0;
      for (int i = 0; i < 5; ++i) {
        const double t = (x - xs[i]) * (x - xs[i]) + (y - ys[i]) * (y - ys[i]);
        g += aa[i] * std::exp(-t / 0.01);
      }
      return -1.5 * (psi - 0.05) - g * std::cos(0.9 * y);
    }
    case 3: {
      const double R2 = x * x + y * y;
      return 0.5 * std::erfc(5.0 * (R2 - 1.0));
    }
    case 4: {
      const double R = std::sqrt(x * x + y * y);
      const double th = std::atan2(y, x);
      return (1.0 - std::pow(std::sin(0.5 * th), 500)) * std::exp(-2000 * (0.1 - R * R) * (0.1 - R * R));
    }
    case 5: {
      const double R = std::sqrt(x * x + y * y);
      return 4 * (y - 0.1) * (1.0 - std::erf(25.0 * (R - 0.3)));
    }
    default: {
      double q = 0.0;
      for (int k = 0; k < c.n_bumps; ++k) {
        const double dx = x - c.bump_cx[k], dy = y - c.bump_cy[k];
        const double R2 = dx * dx + dy * dy;
        q += c.bump_a[k] * std::exp(-R2 / (c.bump_w[k] * c.bump_w[k]));
      }
      return q;
    }
  }
}

// ---------------------------------------------------------------- Hankel table
// Far-field sums shared by every task of one assembly. The far-field entry
// K(i, j) is a scaling of sum_n M[j mod rank][n] h_n, where the Hankel
// vector h of target i about leaf(j) is a function of the two doubles
// (px - lx, py - ly) alone and M is the same for every leaf. So the table is
// keyed on the bit patterns of that relative position and stores, per key,
// the sums for all `rank` source nodes of a leaf: a hit returns exactly what
// the caller would have computed, and skeletons and blocks do not depend on
// which thread filled a slot first. On a uniform tree the leaf centres are
// dyadic and a Chebyshev node's offset from its leaf centre rounds the same
// way in every box of one binade, so few distinct keys occur: at level 5
// (kappa 40) 178 thousand, where per-task caches computed 7.4 million Hankel
// vectors and every entry its own 31-term sum.
using HankelVec = std::array<cd, 2 * kSeries + 1>;

class HankelTable {
 public:
  struct Key {
    uint64_t x, y;
    bool operator==(const Key& o) const { return x == o.x && y == o.y; }
  };
  static Key key(double rx, double ry) {
    Key k;
    std::memcpy(&k.x, &rx, sizeof(double));
    std::memcpy(&k.y, &ry, sizeof(double));
    return k;
  }
  static uint64_t hash(const Key& k) {
    uint64_t h = k.x * 0x9E3779B97F4A7C15ULL ^ (k.y + 0xC2B2AE3D27D4EB4FULL + (k.x << 6) + (k.x >> 2));
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ULL;
    return h ^ (h >> 29);
  }
  // Stored record for `k`, or nullptr.
  const cd* find(const Key& k) {
    const uint64_t h = hash(k);
    Shard& sh = shards_[h >> (64 - kShardBits)];
    std::lock_guard<std::mutex> lk(sh.mu);
    if (sh.keys.empty()) return nullptr;
    for (size_t p = h & sh.mask;; p = (p + 1) & sh.mask) {
      if (sh.keys[p].x == kEmpty) return nullptr;
      if (sh.keys[p] == k) return sh.vals[p];
    }
  }
  // Records hold `w` complex values; set before the first insert.
  void set_width(int w) { width_ = (size_t)w; }
  // Stores the record `v` under `k` unless the table is full; returns the
  // stored record (a concurrent insert of the same key keeps the first,
  // bit-identical one) or nullptr when full. Pointers stay valid until clear().
  const cd* insert(const Key& k, const cd* v) {
    const uint64_t h = hash(k);
    Shard& sh = shards_[h >> (64 - kShardBits)];
    std::lock_guard<std::mutex> lk(sh.mu);
    if (sh.keys.empty()) sh.rehash(1024);
    size_t p = h & sh.mask;
    for (;; p = (p + 1) & sh.mask) {
      if (sh.keys[p].x == kEmpty) break;
      if (sh.keys[p] == k) return sh.vals[p];
    }
    if (size_.load(std::memory_order_relaxed) >= cap_) return nullptr;
    cd* rec = sh.alloc(width_);
    std::copy(v, v + width_, rec);
    sh.keys[p] = k;
    sh.vals[p] = rec;
    ++sh.used;
    size_.fetch_add(1, std::memory_order_relaxed);
    if (2 * sh.used > sh.mask) sh.rehash(2 * (sh.mask + 1));
    return rec;
  }
  void clear() {
    for (Shard& sh : shards_) {
      std::vector<Key>().swap(sh.keys);
      std::vector<const cd*>().swap(sh.vals);
      std::vector<std::unique_ptr<cd[]>>().swap(sh.chunks);
      sh.chunk_cap = 0;
      sh.chunk_left = 0;
      sh.used = 0;
      sh.mask = 0;
    }
    size_.store(0);
  }

 private:
  // The bits of a relative position: never a NaN, so all-ones marks a free slot.
  static constexpr uint64_t kEmpty = ~0ULL;
  static constexpr int kShardBits = 8;
  // At most 4 million records (about 2.4 GB of host memory at 36 nodes per
  // leaf) unless LS_HANKEL_TABLE_CAP gives another count; beyond it the tasks
  // keep what they compute to themselves (same values, computed more than
  // once).
  static size_t cap_from_env() {
    const char* v = std::getenv("LS_HANKEL_TABLE_CAP");
    char* end = nullptr;
    const long long c = v ? std::strtoll(v, &end, 10) : -1;
    return (v && end != v && *end == '\0' && c >= 0) ? (size_t)c : (size_t(1) << 22);
  }
  // Open addressing with linear probing; records live in chunks (64 records
  // at first, doubling up to 4096, so small tables stay small), and a rehash
  // moves keys and pointers but never a record.
  struct Shard {
    std::mutex mu;
    std::vector<Key> keys;
    std::vector<const cd*> vals;
    std::vector<std::unique_ptr<cd[]>> chunks;
    size_t chunk_cap = 0, chunk_left = 0, used = 0, mask = 0;
    cd* alloc(size_t w) {
      if (chunk_left == 0) {
        chunk_cap = chunk_cap == 0 ? 64 : std::min<size_t>(2 * chunk_cap, 4096);
        chunks.emplace_back(new cd[chunk_cap * w]);
        chunk_left = chunk_cap;
      }
      return chunks.back().get() + (chunk_cap - chunk_left--) * w;
    }
    void rehash(size_t cap) {
      std::vector<Key> nk(cap, Key{kEmpty, kEmpty});
      std::vector<const cd*> nv(cap, nullptr);
      for (size_t q = 0; q < keys.size(); ++q) {
        if (keys[q].x == kEmpty) continue;
        size_t p = hash(keys[q]) & (cap - 1);
        while (nk[p].x != kEmpty) p = (p + 1) & (cap - 1);
        nk[p] = keys[q];
        nv[p] = vals[q];
      }
      keys.swap(nk);
      vals.swap(nv);
      mask = cap - 1;
    }
  };
  Shard shards_[1 << kShardBits];
  std::atomic<size_t> size_{0};
  const size_t cap_ = cap_from_env();
  size_t width_ = 0;
};

// Recently used table records of one thread, direct-mapped and lock-free,
// in front of the shared table: neighbouring boxes see the same relative
// positions (translation invariance), so a thread meets the same keys task
// after task. Entries carry the id of the assembly that stored them; a
// record pointer is only returned to that assembly, whose table is alive.
struct ThreadRecent {
  static constexpr int kBits = 15;
  struct Slot {
    HankelTable::Key k;
    const cd* v;
    uint64_t owner;
  };
  std::vector<Slot> slots = std::vector<Slot>(size_t(1) << kBits, Slot{{0, 0}, nullptr, 0});
  Slot& at(const HankelTable::Key& k) { return slots[HankelTable::hash(k) & ((size_t(1) << kBits) - 1)]; }
};
thread_local ThreadRecent t_recent;
std::atomic<uint64_t> g_assembly_id{0};

// ---------------------------------------------------------------- the builder
struct Node {
  bool out_active = false, in_active = false;
  std::vector<int> out_charge, out_check, in_charge, in_check, user_check;
  std::vector<cd> Ar;  // rank_out x K, row major (pivot rows of the outgoing NCA)
  std::vector<int> IL; // source boxes at the same level
  // derived during packing
  std::vector<int> fidx;   // gather indices of f_out in the charge buffer
  long long own_charge = -1;
  long long pot_off = -1;
  bool pot_nonzero = false;
};

class Builder {
 public:
  explicit Builder(const ls_config& c) : cfg(c) {}
  ~Builder() { gpu_far_close(gfar); }
  Builder(const Builder&) = delete;
  Builder& operator=(const Builder&) = delete;
  bool run(HostOperator& op, std::string& err);

 private:
  ls_config cfg;
  int nL = 0, rank = 0, nb = 0, level_LFR = 2, N = 0;
  double kappa = 0.0, L = 1.0;
  std::vector<double> radius;         // boxRadius per level (0..10)
  std::vector<int> nCones;
  std::vector<double> aperture;
  std::vector<std::vector<double>> cx, cy;  // box centres per level
  std::vector<double> gx_, gy_;       // grid points
  std::vector<double> kq_;            // kappa*kappa*q at grid points (entry scaling)
  std::vector<double> cheb1;
  std::vector<std::pair<int, int>> bases;
  std::vector<double> gln, glw;
  std::vector<cd> Mleaf;              // (2S+1) x rank, column major
  std::vector<cd> near;               // 9 x rank x rank, row major
  std::vector<cd> nearVt;             // 9 x rank x nb, row major (factor of near)
  std::vector<cd> nearE;              // 9 x rank x rank, rounding residual of near
  std::vector<double> Qpinv;          // nb x rank, row major
  std::vector<std::vector<std::vector<int>>> nbrs;  // [level][box] same-level neighbours
  std::vector<std::vector<Node>> nodes;             // [level][node]
  mutable HankelTable htab;                         // shared by NCA and block fills
  const uint64_t id = ++g_assembly_id;              // tags thread-local table entries
  // far_on_gpu: the far-field sums of every distinct relative position
  // (FarTables); a target's record about a leaf is dense_rec(i, leaf).
  FarTables ft;
  struct FreeDeleter {
    void operator()(cd* p) const { std::free(p); }
  };
  std::unique_ptr<cd[], FreeDeleter> dS;
  bool dense = false;
  int dny = 0;
  GpuFar* gfar = nullptr;
  const cd* dense_rec(int i, int leaf) const {
    const int xi = ft.xid[(size_t)ft.xrow[i] * ft.ncol + ft.lcol[leaf]];
    const int yi = ft.yid[(size_t)ft.yrow[i] * ft.ncol + ft.lrow[leaf]];
    return dS.get() + ((size_t)xi * dny + yi) * rank;
  }

  bool is_lfr(int j) const { return j >= level_LFR; }
  int nodes_at(int j) const { return is_lfr(j) ? (1 << (2 * j)) : (1 << (2 * j)) * nCones[j]; }
  Node& lfr(int j, int k) { return nodes[j][k]; }
  Node& cone(int j, int k, int c) { return nodes[j][(size_t)k * nCones[j] + c]; }
  // Node through which box (j,k) exposes its data to direction `c` of a
  // parent/IL relation: LFR boxes have one node, HFR boxes one per cone.
  Node& child_node(int jchild, int kchild, int parent_cone) {
    return is_lfr(jchild) ? lfr(jchild, kchild) : cone(jchild, kchild, parent_cone / 2);
  }

  // Far-field Hankel vector h_n = (J_n + i Y_n) e^{i n theta}, n = -15..15,
  // of a target at (rx, ry) from a leaf centre (G_FMM2DTree.hpp:603-658).
  void hankel_rel(double rx, double ry, cd* h) const {
    const double th = std::atan2(ry, rx);
    const double R2 = ry * ry + rx * rx;
    const double R = kappa * std::sqrt(R2);
    double J[kSeries + 1], Y[kSeries + 1];
    bessel_jy_orders(kSeries, R, J, Y);
    for (int n = -kSeries; n <= kSeries; ++n) {
      const int a = n < 0 ? -n : n;
      const double sg = (n < 0 && (a % 2 == 1)) ? -1.0 : 1.0;
      const double jn = sg == 1.0 ? J[a] : -J[a];
      const double yn = sg == 1.0 ? Y[a] : -Y[a];
      h[n + kSeries] = (jn + kI * yn) * std::exp(kI * double(n) * th);
    }
  }
  // Far-field sums of a target at (rx, ry) from a leaf centre for all `rank`
  // source nodes of the leaf: out[idx] = sum_n M[idx][n] h_n, in real
  // arithmetic with the operand order of the complex product,
  // (a + ib)(c + id) = (ac - bd) + i(ad + bc), so each sum equals the
  // std::complex one bit for bit without its per-product NaN checks.
  void key_sums(double rx, double ry, cd* out) const {
    HankelVec h;
    hankel_rel(rx, ry, h.data());
    constexpr int nS = 2 * kSeries + 1;
    for (int idx = 0; idx < rank; ++idx) {
      const cd* m = &Mleaf[(size_t)idx * nS];
      double sr = 0.0, si = 0.0;
      for (int n = 0; n < nS; ++n) {
        const double a = m[n].real(), b = m[n].imag(), c = h[n].real(), d = h[n].imag();
        sr += a * c - b * d;
        si += a * d + b * c;
      }
      out[idx] = cd(sr, si);
    }
  }
  // Per-task cache of the far-field sums of target i about leaf(j), over the
  // shared table: open addressing on the key i * 2^20 + leaf (-1 marks a
  // free slot).
  struct HCache {
    const Builder* b;
    std::vector<long long> keys;
    std::vector<const cd*> vals;
    size_t used = 0;
    std::deque<std::vector<cd>> own;  // records the full table did not take
    long long last_key = -1;    // rows and columns visit a leaf's points in runs
    const cd* last = nullptr;
    static size_t slot(long long key, size_t mask) {
      uint64_t h = (uint64_t)key * 0x9E3779B97F4A7C15ULL;
      return (size_t)(h ^ (h >> 32)) & mask;
    }
    void grow() {
      const size_t cap = keys.empty() ? 4096 : 2 * keys.size();
      std::vector<long long> nk(cap, -1);
      std::vector<const cd*> nv(cap, nullptr);
      for (size_t q = 0; q < keys.size(); ++q) {
        if (keys[q] < 0) continue;
        size_t p = slot(keys[q], cap - 1);
        while (nk[p] >= 0) p = (p + 1) & (cap - 1);
        nk[p] = keys[q];
        nv[p] = vals[q];
      }
      keys.swap(nk);
      vals.swap(nv);
    }
    const cd* get(int i, int leaf) {
      if (b->dense) return b->dense_rec(i, leaf);
      const long long key = (long long)i * 1048576LL + leaf;
      if (key == last_key) return last;
      last_key = key;
      if (2 * (used + 1) > keys.size()) grow();
      const size_t mask = keys.size() - 1;
      size_t p = slot(key, mask);
      for (; keys[p] >= 0; p = (p + 1) & mask)
        if (keys[p] == key) return last = vals[p];
      const double rx = b->gx_[i] - b->cx[b->nL][leaf], ry = b->gy_[i] - b->cy[b->nL][leaf];
      const HankelTable::Key k = HankelTable::key(rx, ry);
      ThreadRecent::Slot& rs = t_recent.at(k);
      const cd* h = (rs.owner == b->id && rs.k == k) ? rs.v : b->htab.find(k);
      bool shared = h != nullptr;  // a table record, alive until the assembly ends
      if (!h) {
        std::vector<cd> v((size_t)b->rank);
        b->key_sums(rx, ry, v.data());
        h = b->htab.insert(k, v.data());
        shared = h != nullptr;
        if (!h) {
          own.push_back(std::move(v));
          h = own.back().data();
        }
      }
      if (shared) rs = {k, h, b->id};
      keys[p] = key;
      vals[p] = h;
      ++used;
      return last = h;
    }
  };
  // K(i, j) from its far-field sum.
  cd scale(int i, int j, cd s) const {
    s *= kI / 4.0;
    if (cfg.findPhi) {
      s *= kq_[i];
      if (i == j) s += 1.0;
    }
    return s;
  }
  cd entry(int i, int j, HCache& hc) const { return scale(i, j, hc.get(i, j / rank)[j % rank]); }
  // Row-major block K(rows, cols).
  void fill(const std::vector<int>& rows, const std::vector<int>& cols, HCache& hc, cd* out, int ld) const {
    for (size_t a = 0; a < rows.size(); ++a)
      for (size_t b = 0; b < cols.size(); ++b) out[a * ld + b] = entry(rows[a], cols[b], hc);
  }
  std::vector<cd> block_colmajor(const std::vector<int>& rows, const std::vector<int>& cols, HCache& hc) const {
    std::vector<cd> A(rows.size() * cols.size());
    for (size_t b = 0; b < cols.size(); ++b)
      for (size_t a = 0; a < rows.size(); ++a) A[b * rows.size() + a] = entry(rows[a], cols[b], hc);
    return A;
  }

  int aca(const std::vector<int>& rows, const std::vector<int>& cols, double eps, std::vector<int>& rb,
          std::vector<int>& cb, std::vector<cd>* Ar, HCache& hc) const;

  // One NCA block: out (outgoing) has the far checks as rows and the
  // box's own charges as columns, in the box's own checks as rows and the
  // far charges as columns.
  struct NcaJob {
    Node* nd = nullptr;
    bool out = false;
    std::vector<int> rows, cols, rb, cb;
    int rank = 0;
  };

  void geometry();
  void precompute();
  void interaction_lists();
  void far_tables();
  void fill_tiles_host(GemvPhase& ph, const std::vector<FillTile>& fl, const std::vector<int>& rowpts,
                       const std::vector<int>& colpts);
  void run_nca(std::vector<NcaJob>& jobs);
  void nca_level_lfr(int j);
  void nca_level_hfr(int j);
  void user_checks();
  void pack(HostOperator& op);
};

// First index of the largest |v| among the unused ones (strict >, so ties
// go to the lowest index, ACA.hpp:153-166). With every index used the
// reference dereferences begin() of an empty std::set, which reads the
// set's element count (0) with libstdc++: index 0, after which the ACA loop
// ends on rank == min(rows, cols).
//
// |v| is std::abs (hypot), which is costly, so a first pass finds the
// largest re^2 + im^2 = Q. Both forms are within a few ulps of the true
// magnitude: every index whose |v| equals the largest one has
// re^2 + im^2 >= Q (1 - 1e-12), and every other index has a strictly
// smaller |v|. The rule above, run on those candidates alone, therefore
// picks the same index as a scan of all of them. That bound needs the
// squares to carry full relative precision: below |v| ~ 1e-145 they are
// subnormal (or zero), so when Q < 1e-290 every unused index goes through
// hypot.
static int argmax_remaining(const std::vector<cd>& v, const std::vector<char>& used) {
  const int n = (int)v.size();
  double Q = -1.0;
  for (int i = 0; i < n; ++i) {
    if (used[i]) continue;
    const double q = v[i].real() * v[i].real() + v[i].imag() * v[i].imag();
    if (q > Q) Q = q;
  }
  if (Q < 0.0) return 0;  // every index used
  const double cut = Q < 1e-290 ? -1.0 : Q * (1.0 - 1e-12);
  int idx = -1;
  double mx = 0.0;
  for (int i = 0; i < n; ++i) {
    if (used[i]) continue;
    const double q = v[i].real() * v[i].real() + v[i].imag() * v[i].imag();
    if (!(q >= cut)) continue;
    if (idx < 0) { idx = i; mx = std::abs(v[i]); continue; }
    if (std::abs(v[i]) > mx) { idx = i; mx = std::abs(v[idx]); }
  }
  return idx < 0 ? 0 : idx;
}
static double norm2(const std::vector<cd>& v) {
  double s = 0.0;
  for (const cd& z : v) s += std::norm(z);
  return std::sqrt(s);
}
// sum_i conj(a_i) b_i. conj(x + iy) (c + id) = (xc - (-y)d) + i(xd + (-y)c),
// and p - (-q) is the same IEEE operation as p + q, so the real form below
// equals the std::complex one bit for bit, without its NaN checks.
static cd cdot(const std::vector<cd>& a, const std::vector<cd>& b) {
  double sr = 0.0, si = 0.0;
  for (size_t i = 0; i < a.size(); ++i) {
    const double x = a[i].real(), y = a[i].imag(), c = b[i].real(), d = b[i].imag();
    sr += x * c + y * d;
    si += x * d - y * c;
  }
  return cd(sr, si);
}
// v[s] -= f * w[s] for all s, with the operand order of the complex product
// (a + ib)(c + id) = (ac - bd) + i(ad + bc): equal to the std::complex
// update bit for bit.
static void sub_scaled(std::vector<cd>& v, cd f, const std::vector<cd>& w) {
  const double a = f.real(), b = f.imag();
  for (size_t s = 0; s < w.size(); ++s) {
    const double c = w[s].real(), d = w[s].imag();
    v[s] = cd(v[s].real() - (a * c - b * d), v[s].imag() - (a * d + b * c));
  }
}

// Partially pivoted cross approximation that keeps only the pivots
// (ACA_only_nodes, ACA.hpp:253-481). Row-first when there are fewer rows
// than columns, column-first otherwise; ties go to the lowest index.
// ACA_only_nodes (GMRES/ACA.hpp:253-481) over a rows x cols block given by
// its row and column fetchers: pivot search, rank-1 updates, the norm
// estimate and the stopping rules in the reference's order. Returns the
// rank; rb / cb get the pivot rows / columns and Ar (if given) the pivot
// rows of the block, row major rank x n2.
template <class GetRow, class GetCol>
static int aca_core(int n1, int n2, double eps, std::vector<int>& rb, std::vector<int>& cb, std::vector<cd>* Ar,
                    GetRow get_row, GetCol get_col) {
  const int mn = std::min(n1, n2);
  std::vector<char> rused(n1, 0), cused(n2, 0);
  std::vector<std::vector<cd>> U, V, piv_rows;
  std::vector<cd> row(n2), col(n1), u, v;
  int rk = 0, ri = 0, ci = 0;
  const double thr = eps * std::pow(10, -1.0 * 0);
  if (n1 < n2) {
    int l = 0;
    for (; l < n1; ++l) {
      ri = l;
      row = get_row(ri);
      ci = argmax_remaining(row, cused);
      if (std::abs(row[ci]) > thr) break;
    }
    if (l == n1) return 0;
    v.resize(n2);
    for (int s = 0; s < n2; ++s) v[s] = row[s] / row[ci];
    rb.push_back(ri);
    cb.push_back(ci);
    col = get_col(ci);
    u = col;
    U.push_back(u); V.push_back(v); piv_rows.push_back(row);
    cused[ci] = 1; rused[ri] = 1;
    rk = 1;
    double nS = 0.0, prev = 1000.0;
    ri = argmax_remaining(col, rused);
    while (std::abs(row[ci]) > thr && std::abs(col[ri]) > eps && std::abs(prev - nS) >= eps * prev && rk < mn) {
      rb.push_back(ri);
      row = get_row(ri);
      const std::vector<cd> raw = row;
      for (int a = 0; a < rk; ++a) sub_scaled(row, U[a][ri], V[a]);
      ci = argmax_remaining(row, cused);
      cb.push_back(ci);
      for (size_t s = 0; s < row.size(); ++s) v[s] = row[s] / row[ci];
      col = get_col(ci);
      for (int a = 0; a < rk; ++a) sub_scaled(col, V[a][ci], U[a]);
      u = col;
      if (norm2(u) < 1e-8 || norm2(v) < 1e-8) { rb.pop_back(); cb.pop_back(); break; }
      U.push_back(u); V.push_back(v); piv_rows.push_back(raw);
      ++rk;
      cused[ci] = 1; rused[ri] = 1;
      if (rk != 2) prev = nS;
      nS = std::pow(nS, 2) + std::pow(norm2(u) * norm2(v), 2);
      for (int a = 0; a < rk; ++a) nS += 2 * std::abs(cdot(U[a], u) * cdot(V[a], v));
      nS = std::sqrt(nS);
      ri = argmax_remaining(col, rused);
    }
  } else {
    int l = 0;
    for (; l < n2; ++l) {
      ci = l;
      col = get_col(ci);
      ri = argmax_remaining(col, rused);
      if (std::abs(col[ri]) > thr) break;
    }
    if (l == n2) return 0;
    cb.push_back(ci);
    v.resize(n1);
    for (int s = 0; s < n1; ++s) v[s] = col[s] / col[ri];
    rb.push_back(ri);
    row = get_row(ri);
    u = row;
    U.push_back(u); V.push_back(v); piv_rows.push_back(row);
    rk = 1;
    rused[ri] = 1; cused[ci] = 1;
    double nS = 0.0, prev = 1000.0;
    ci = argmax_remaining(row, cused);
    while (std::abs(row[ci]) > thr && std::abs(col[ri]) > eps && std::abs(prev - nS) >= eps * prev && rk < mn) {
      cb.push_back(ci);
      col = get_col(ci);
      for (int a = 0; a < rk; ++a) sub_scaled(col, U[a][ci], V[a]);
      ri = argmax_remaining(col, rused);
      rb.push_back(ri);
      for (size_t s = 0; s < col.size(); ++s) v[s] = col[s] / col[ri];
      row = get_row(ri);
      const std::vector<cd> raw = row;
      for (int a = 0; a < rk; ++a) sub_scaled(row, V[a][ri], U[a]);
      u = row;
      if (norm2(u) < 1e-8 || norm2(v) < 1e-8) { cb.pop_back(); rb.pop_back(); break; }
      U.push_back(u); V.push_back(v); piv_rows.push_back(raw);
      ++rk;
      rused[ri] = 1; cused[ci] = 1;
      if (rk != 2) prev = nS;
      nS = std::pow(nS, 2) + std::pow(norm2(u) * norm2(v), 2);
      for (int a = 0; a < rk; ++a) nS += 2 * std::abs(cdot(U[a], u) * cdot(V[a], v));
      nS = std::sqrt(nS);
      ci = argmax_remaining(row, cused);
    }
  }
  if (Ar) {
    Ar->assign((size_t)rk * n2, cd(0.0, 0.0));
    for (int a = 0; a < rk; ++a)
      for (int b = 0; b < n2; ++b) (*Ar)[(size_t)a * n2 + b] = piv_rows[a][b];
  }
  return rk;
}


int Builder::aca(const std::vector<int>& rows, const std::vector<int>& cols, double eps, std::vector<int>& rb,
                 std::vector<int>& cb, std::vector<cd>* Ar, HCache& hc) const {
  const int n1 = (int)rows.size(), n2 = (int)cols.size();
  auto get_row = [&](int r) { std::vector<cd> o(n2); for (int k = 0; k < n2; ++k) o[k] = entry(rows[r], cols[k], hc); return o; };
  // Columns in one source leaf share the far-field records of every row:
  // keep them per leaf, indexed by row position.
  std::vector<std::pair<int, std::vector<const cd*>>> col_leaf;
  auto get_col = [&](int c) {
    std::vector<cd> o(n1);
    const int j = cols[c], leaf = j / rank, node = j % rank;
    std::vector<const cd*>* P = nullptr;
    for (auto& e : col_leaf)
      if (e.first == leaf) P = &e.second;
    if (!P) {
      col_leaf.emplace_back(leaf, std::vector<const cd*>(n1, nullptr));
      P = &col_leaf.back().second;
    }
    for (int k = 0; k < n1; ++k) {
      const cd*& h = (*P)[k];
      if (!h) h = hc.get(rows[k], leaf);
      o[k] = scale(rows[k], j, h[node]);
    }
    return o;
  };
  return aca_core(n1, n2, eps, rb, cb, Ar, get_row, get_col);
}

void Builder::geometry() {
  kappa = cfg.kappa;
  L = cfg.L;
  const int n1 = cfg.nChebNodes;
  rank = n1 * n1;
  nb = cfg.degreeOfBases * (cfg.degreeOfBases + 1) / 2;
  nL = cfg.nLevelsUniform;
  if (cfg.yes2DFMM == 1) {
    if (kappa == 0) level_LFR = 2;
    else level_LFR = (int)std::floor(std::log(kappa * L / 0.35) / std::log(2.0));
    if (level_LFR < 2) level_LFR = 2;
  } else {
    level_LFR = 2;
  }
  if (level_LFR >= nL) level_LFR = nL - 1;
  radius.push_back(L);
  for (int j = 1; j <= 10; ++j) radius.push_back(radius[j - 1] / 2.0);
  cx.assign(nL + 1, {});
  cy.assign(nL + 1, {});
  cx[0] = {0.0};
  cy[0] = {0.0};
  std::vector<double> rr(1, L);
  for (int j = 0; j < nL; ++j) {
    const size_t nbx = cx[j].size();
    cx[j + 1].resize(nbx * 4);
    cy[j + 1].resize(nbx * 4);
    const double h = 0.5 * radius[j];
    // Child 0 (-,-), 1 (+,-), 2 (+,+), 3 (-,+); index 4k + c.
    for (size_t k = 0; k < nbx; ++k) {
      cx[j + 1][4 * k + 0] = cx[j][k] - h; cy[j + 1][4 * k + 0] = cy[j][k] - h;
      cx[j + 1][4 * k + 1] = cx[j][k] + h; cy[j + 1][4 * k + 1] = cy[j][k] - h;
      cx[j + 1][4 * k + 2] = cx[j][k] + h; cy[j + 1][4 * k + 2] = cy[j][k] + h;
      cx[j + 1][4 * k + 3] = cx[j][k] - h; cy[j + 1][4 * k + 3] = cy[j][k] + h;
    }
  }
  nCones.push_back((int)(cfg.nCones_LFR * std::pow(2.0, level_LFR - 1)));
  aperture.push_back(2 * kPi / nCones[0]);
  for (int j = 1; j <= level_LFR - 1; ++j) {
    nCones.push_back((int)(nCones[j - 1] / 2.0));
    aperture.push_back(aperture[j - 1] * 2.0);
  }
  for (int k = 0; k < n1; ++k) cheb1.push_back(-std::cos((k + 0.5) / n1 * kPi));
  const int nleaf = 1 << (2 * nL);
  N = nleaf * rank;
  gx_.resize(N);
  gy_.resize(N);
  for (int t = 0; t < nleaf; ++t)
    for (int r = 0; r < n1; ++r)
      for (int c = 0; c < n1; ++c) {
        const int i = t * rank + r * n1 + c;
        gx_[i] = radius[nL] * cheb1[c] + cx[nL][t];
        gy_[i] = radius[nL] * cheb1[r] + cy[nL][t];
      }
  kq_.resize(N);
  for (int i = 0; i < N; ++i) kq_[i] = kappa * kappa * (contrast_fn(cfg, gx_[i], gy_[i]));
  for (int d = 0; d < cfg.degreeOfBases; ++d)
    for (int a = 0; a < d + 1; ++a) bases.push_back({a, d - a});
  gl_rule(kQuadOrder, gln, glw);
}

void Builder::precompute() {
  // Q (rank x nb) at the standard nodes and Q^+ from its QR.
  std::vector<cd> Q((size_t)rank * nb);
  const int n1 = cfg.nChebNodes;
  for (int l = 0; l < nb; ++l)
    for (int i = 0; i < rank; ++i) {
      const double xs = cheb1[i % n1], ys = cheb1[i / n1];
      Q[(size_t)l * rank + i] = cd(cheb_t(xs, bases[l].first) * cheb_t(ys, bases[l].second), 0.0);
    }
  PivQR qr;
  qr.factor(rank, nb, Q);
  std::vector<double> Qp((size_t)nb * rank);  // Qp[l * rank + i]
  {
    std::vector<cd> e(rank), s(nb);
    for (int i = 0; i < rank; ++i) {
      std::fill(e.begin(), e.end(), cd(0.0, 0.0));
      e[i] = 1.0;
      qr.solve(e.data(), s.data());
      for (int l = 0; l < nb; ++l) Qp[(size_t)l * rank + i] = s[l].real();
    }
  }
  const int nS = 2 * kSeries + 1;
  const double rj = radius[nL];
  // A cached record of this leaf size: M, then the near blocks, their
  // factors and rounding residuals.
  const size_t nM = (size_t)nS * rank, nB = (size_t)9 * rank * rank, nV = (size_t)9 * rank * nb;
  auto key = [&](int gpu) {
    return pc_key("uniform-leaf", {kappa, rj}, {cfg.nChebNodes, cfg.degreeOfBases, cfg.reference_rounding, gpu, kSeries});
  };
  {
    std::vector<cd> rec;
    if (g_pcache.get(key(quadrature_device(cfg) >= 0), rec) && rec.size() == nM + 2 * nB + nV) {
      Mleaf.assign(rec.begin(), rec.begin() + nM);
      near.assign(rec.begin() + nM, rec.begin() + nM + nB);
      nearVt.assign(rec.begin() + nM + nB, rec.begin() + nM + nB + nV);
      nearE.assign(rec.begin() + nM + nB + nV, rec.end());
      Qpinv = Qp;
      return;
    }
  }
  static const double ncx[9] = {-2, 0, 2, 2, 2, 0, -2, -2, 0};
  static const double ncy[9] = {-2, -2, -2, 0, 2, 2, 2, 0, 0};
  const double rA = radius[nL], rB = radius[nL];
  // The quadratures below (far moments, then near integrals) run on the
  // operator's GPU when it has one; otherwise, or if that fails, on the host.
  std::vector<QuadTask> tasks;
  tasks.reserve((size_t)nS * nb + (size_t)9 * rank * nb);
  for (int t = 0; t < nS * nb; ++t)
    tasks.push_back({0.0, 0.0, kappa * rj, bases[t % nb].first, bases[t % nb].second, t / nb - kSeries, 1});
  for (int t = 0; t < 9 * rank; ++t) {
    const int q = t / rank, i = t % rank;
    const double Xx = (rA * cheb1[i % n1] + 0.0 - ncx[q] * rA) / rB, Xy = (rA * cheb1[i / n1] + 0.0 - ncy[q] * rA) / rB;
    for (int l = 0; l < nb; ++l) tasks.push_back({Xx, Xy, kappa * rB, bases[l].first, bases[l].second, 0, 0});
  }
  std::vector<cd> qv;
  const bool on_gpu = gpu_quadrature(quadrature_device(cfg), tasks, gln, glw, qv);
  // Far moments C (2S+1) x nb, then M = C Q^+ rounded like the text cache.
  std::vector<cd> C((size_t)nS * nb);
  if (on_gpu)
    for (int t = 0; t < nS * nb; ++t) C[t] = rj * rj * qv[t];
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < (on_gpu ? 0 : nS * nb); ++t) {
    const int n = t / nb - kSeries, l = t % nb;
    const int a = bases[l].first, b = bases[l].second;
    auto f = [&](double x, double y) -> cd {
      const double R2 = x * x + y * y;
      const double nx = std::sqrt(R2);
      const double arg = kappa * rj * nx;
      const double th = std::atan2(y, x);
      return bes_j(n, arg) * std::exp(-kI * double(n) * th) * cheb_t(x, a) * cheb_t(y, b);
    };
    C[(size_t)(n + kSeries) * nb + l] = rj * rj * quad2d(f, gln, glw);
  }
  Mleaf.assign((size_t)nS * rank, cd(0.0, 0.0));
  for (int n = 0; n < nS; ++n)
    for (int i = 0; i < rank; ++i) {
      cd s(0.0, 0.0);
      for (int l = 0; l < nb; ++l) s += C[(size_t)n * nb + l] * Qp[(size_t)l * rank + i];
      if (cfg.reference_rounding) s = cd(round6(s.real()), round6(s.imag()));
      Mleaf[(size_t)i * nS + n] = s;
    }
  // Colleague near blocks: V(i,l) = int H0(k r |X_i - P|) T_a T_b dP, then
  // V (i r^2 / 4) Q^+.
  std::vector<cd> V((size_t)9 * rank * nb);
  if (on_gpu)
    for (size_t t = 0; t < V.size(); ++t) V[t] = qv[(size_t)nS * nb + t];
  int max_order = 0;
  for (const auto& ab : bases) max_order = std::max(max_order, std::max(ab.first, ab.second));
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < (on_gpu ? 0 : 9 * rank); ++t) {
    const int q = t / rank, i = t % rank;
    const double bx = ncx[q] * rA, by = ncy[q] * rA;
    const double ax = rA * cheb1[i % n1] + 0.0, ay = rA * cheb1[i / n1] + 0.0;
    const double Xx = (ax - bx) / rB, Xy = (ay - by) / rB;
    // Per quadrature point: H0 and the Chebyshev values of every order the
    // bases use, computed once and shared by all bases of this target.
    struct PointVals {
      cd H;
      double tx[kMaxChebOrder + 1], ty[kMaxChebOrder + 1];
    };
    std::unordered_map<unsigned long long, PointVals> memo;
    auto key = [](double a, double b) {
      unsigned long long ka, kb;
      std::memcpy(&ka, &a, 8);
      std::memcpy(&kb, &b, 8);
      return ka * 0x9E3779B97F4A7C15ULL ^ (kb + 0x632BE59BD9B4E019ULL + (ka << 6) + (ka >> 2));
    };
    for (int l = 0; l < nb; ++l) {
      const int a = bases[l].first, b = bases[l].second;
      auto f = [&](double x, double y) -> cd {
        const unsigned long long kk = key(x, y);
        auto it = memo.find(kk);
        if (it == memo.end()) {
          PointVals pv;
          const double R2 = (Xx - x) * (Xx - x) + (Xy - y) * (Xy - y);
          const double R = std::sqrt(R2);
          const double arg = kappa * rB * R;
          pv.H = bes_j(0, arg) + kI * bes_y(0, arg);
          for (int o = 0; o <= max_order; ++o) {
            pv.tx[o] = cheb_t(x, o);
            pv.ty[o] = cheb_t(y, o);
          }
          it = memo.emplace(kk, pv).first;
        }
        const PointVals& pv = it->second;
        return pv.H * pv.tx[a] * pv.ty[b];
      };
      V[((size_t)q * rank + i) * nb + l] = quad2d(f, gln, glw);
    }
  }
  near.assign((size_t)9 * rank * rank, cd(0.0, 0.0));
  // Factored form for the device: B_q = Vt_q Q^+ + E_q, with Vt_q = V_q (i r^2/4)
  // (rank x nb) and E_q the residual of the 6-digit rounding (0 without it).
  nearVt.assign((size_t)9 * rank * nb, cd(0.0, 0.0));
  nearE.assign((size_t)9 * rank * rank, cd(0.0, 0.0));
  Qpinv = Qp;
  for (int q = 0; q < 9; ++q)
    for (int i = 0; i < rank; ++i) {
      for (int l = 0; l < nb; ++l)
        nearVt[((size_t)q * rank + i) * nb + l] = V[((size_t)q * rank + i) * nb + l] * kI * rB * rB / 4.0;
      for (int c = 0; c < rank; ++c) {
        cd s(0.0, 0.0);
        for (int l = 0; l < nb; ++l) {
          const cd vt = V[((size_t)q * rank + i) * nb + l] * kI * rB * rB / 4.0;
          s += vt * Qp[(size_t)l * rank + c];
        }
        const cd exact = s;
        if (cfg.reference_rounding) s = cd(round6(s.real()), round6(s.imag()));
        near[((size_t)q * rank + i) * rank + c] = s;
        nearE[((size_t)q * rank + i) * rank + c] = s - exact;
      }
    }
  if (g_pcache.enabled()) {
    std::vector<cd> rec;
    rec.reserve(nM + 2 * nB + nV);
    rec.insert(rec.end(), Mleaf.begin(), Mleaf.end());
    rec.insert(rec.end(), near.begin(), near.end());
    rec.insert(rec.end(), nearVt.begin(), nearVt.end());
    rec.insert(rec.end(), nearE.begin(), nearE.end());
    g_pcache.put(key(on_gpu ? 1 : 0), rec);
  }
}

// Interaction lists of the children of every box (assign_Child_Interaction,
// G_FMM2DTree.hpp:1356-1461). In a uniform tree every neighbour is a
// same-level box, so lists hold box indices of the same level.
void Builder::interaction_lists() {
  const double epsR = std::pow(10, -8);
  nbrs.assign(nL + 1, {});
  nodes.assign(nL + 1, {});
  for (int j = 2; j <= nL; ++j) nodes[j].assign(nodes_at(j), Node());
  nbrs[1].assign(4, {0, 1, 2, 3});
  for (int j = 1; j <= nL - 1; ++j) {
    const int J = j + 1;
    nbrs[J].assign((size_t)1 << (2 * J), {});
#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < (1 << (2 * j)); ++k) {
      for (int c = 0; c < 4; ++c) {
        const int A = 4 * k + c;
        for (int pn : nbrs[j][k]) {
          for (int nc = 0; nc < 4; ++nc) {
            const int B = 4 * pn + nc;
            const double dx = std::fabs(cx[J][A] - cx[J][B]), dy = std::fabs(cy[J][A] - cy[J][B]);
            if (J >= level_LFR) {
              const double lim = 3.0 * radius[J] + radius[J] - epsR;
              if (dx >= lim || dy >= lim) lfr(J, A).IL.push_back(B);
              else nbrs[J][A].push_back(B);
            } else {
              const double limx = kappa * radius[J] * radius[J] + radius[J] + radius[J] - epsR;
              const double limy = kappa * radius[J] * radius[J] + radius[J] - epsR;
              if (dx >= limx || dy >= limy) {
                double arg = std::atan2(cy[J][A] - cy[J][B], cx[J][A] - cx[J][B]);
                arg = std::fmod(arg + 2 * kPi + kPi, 2 * kPi);
                const int cn = int(arg / aperture[J]);
                cone(J, A, cn).IL.push_back(B);
              } else {
                nbrs[J][A].push_back(B);
              }
            }
          }
        }
      }
    }
  }
}

// Cone of source box `src` (level j) that points at box `dst`
// (G_FMM2DTree.hpp:2524-2526, 3335-3337, 3863-3865).
static inline int cone_towards(const std::vector<double>& cxj, const std::vector<double>& cyj, int dst, int src,
                               double ap) {
  const double arg = std::atan2(cyj[dst] - cyj[src], cxj[dst] - cxj[src]);
  const double a = std::fmod(arg + 2 * kPi, 2 * kPi);
  return int(a / ap);
}

// Tables for far_on_gpu (see FarTables). Leaf centres of one column share
// their x bits (every box of a column is reached by the same halvings), so
// fl(gx_i - cx_leaf) is a function of (x node of i, column of i's leaf,
// column of the leaf). The sums are tabulated on the operator's GPU, or on
// the host cores when the operator has no device; a GPU that cannot do it
// leaves the assembly on the default path. Every record the host reads
// here is key_sums of the same (rx, ry) bits that the default path keys its
// cache on, so a host-tabulated assembly is the default one bit for bit.
void Builder::far_tables() {
  dense = false;
  if (!cfg.far_on_gpu || !(kappa > 0.0)) return;
  const int n1 = cfg.nChebNodes, nleaf = 1 << (2 * nL), ncol = 1 << nL;
  std::vector<double> xs(cx[nL]), ys(cy[nL]);
  std::sort(xs.begin(), xs.end());
  std::sort(ys.begin(), ys.end());
  xs.erase(std::unique(xs.begin(), xs.end()), xs.end());
  ys.erase(std::unique(ys.begin(), ys.end()), ys.end());
  if ((int)xs.size() != ncol || (int)ys.size() != ncol) return;
  FarTables t;
  t.rank = rank;
  t.ncol = ncol;
  t.findPhi = cfg.findPhi;
  t.kappa = kappa;
  t.lcol.resize(nleaf);
  t.lrow.resize(nleaf);
  for (int l = 0; l < nleaf; ++l) {
    t.lcol[l] = (int)(std::lower_bound(xs.begin(), xs.end(), cx[nL][l]) - xs.begin());
    t.lrow[l] = (int)(std::lower_bound(ys.begin(), ys.end(), cy[nL][l]) - ys.begin());
  }
  // Coordinates of each (node, column) row, checked bit for bit against
  // every point of the row.
  std::vector<double> gxr((size_t)n1 * ncol), gyr((size_t)n1 * ncol);
  std::vector<char> seenx(gxr.size(), 0), seeny(gyr.size(), 0);
  t.xrow.resize(N);
  t.yrow.resize(N);
  for (int i = 0; i < N; ++i) {
    const int l = i / rank, c = (i % rank) % n1, r = (i % rank) / n1;
    const int xr = c * ncol + t.lcol[l], yr = r * ncol + t.lrow[l];
    t.xrow[i] = xr;
    t.yrow[i] = yr;
    for (int axis = 0; axis < 2; ++axis) {
      std::vector<double>& g = axis ? gyr : gxr;
      std::vector<char>& seen = axis ? seeny : seenx;
      const int row = axis ? yr : xr;
      const double v = axis ? gy_[i] : gx_[i];
      if (!seen[row]) {
        g[row] = v;
        seen[row] = 1;
      } else if (std::memcmp(&g[row], &v, sizeof(double)) != 0) {
        return;
      }
    }
  }
  auto distinct = [&](const std::vector<double>& g, const std::vector<double>& cs, std::vector<double>& u,
                      std::vector<int>& id) {
    std::unordered_map<uint64_t, int> at;
    id.resize(g.size() * cs.size());
    for (size_t row = 0; row < g.size(); ++row)
      for (size_t lc = 0; lc < cs.size(); ++lc) {
        const double v = g[row] - cs[lc];
        uint64_t bits;
        std::memcpy(&bits, &v, sizeof(double));
        auto it = at.find(bits);
        if (it == at.end()) {
          it = at.emplace(bits, (int)u.size()).first;
          u.push_back(v);
        }
        id[row * cs.size() + lc] = it->second;
      }
  };
  distinct(gxr, xs, t.ux, t.xid);
  distinct(gyr, ys, t.uy, t.yid);
  const size_t nkeys = t.ux.size() * t.uy.size();
  if (nkeys * rank * sizeof(cd) > kFarTableMaxBytes) return;
  t.kq = kq_;
  t.M = Mleaf;
  ft = std::move(t);
  dny = (int)ft.uy.size();
  // The host copy, allocated without a serial fill and first touched by
  // all threads (its pages then spread over the threads that read them).
  const size_t nrec = nkeys * rank;
  dS.reset(static_cast<cd*>(std::malloc(nrec * sizeof(cd))));
  if (!dS) return;
  cd* S = dS.get();
#pragma omp parallel for schedule(static)
  for (long long key = 0; key < (long long)nkeys; ++key)
    for (int r = 0; r < rank; ++r) S[(size_t)key * rank + r] = cd(0.0, 0.0);
  const int device = t_assembly_device;
  if (device >= 0) {
    gfar = gpu_far_open(device, ft, S);
    if (!gfar) {
      dS.reset();
      return;
    }
  } else {
#pragma omp parallel for schedule(dynamic, 256)
    for (long long key = 0; key < (long long)nkeys; ++key) {
      const double rx = ft.ux[key / dny], ry = ft.uy[key % dny];
      if (rx == 0.0 && ry == 0.0) continue;  // coincident points: never a far-field pair
      key_sums(rx, ry, S + (size_t)key * rank);
    }
  }
  dense = true;
}

// Fills the tiles described by fl from the far-field table on the host
// (far_on_gpu = 3 without a device, or when the device fill failed): the
// entries the device fill writes, and the values the default packing
// writes for the same blocks.
void Builder::fill_tiles_host(GemvPhase& ph, const std::vector<FillTile>& fl, const std::vector<int>& rowpts,
                              const std::vector<int>& colpts) {
  ph.A.resize((size_t)ph.dev_A_elems);
  ph.dev_A_elems = 0;
#pragma omp parallel for schedule(dynamic, 64)
  for (size_t t = 0; t < fl.size(); ++t) {
    const FillTile& f = fl[t];
    HCache hc{this, {}};
    const int S = 1 << f.log2s, R = kTileLanes >> f.log2s;
    for (int q = 0; q < f.qmax; ++q)
      for (int lane = 0; lane < kTileLanes; ++lane) {
        const int sl = lane / R, r = lane % R, k = q * S + sl;
        cplx v{0.0, 0.0};
        if (r < f.rows && k < f.K) {
          const cd e = entry(rowpts[(size_t)(f.row_off + r)], colpts[(size_t)(f.col_off + k)], hc);
          v = cplx{e.real(), e.imag()};
        }
        ph.A[(size_t)(f.a_off + (long long)q * kTileLanes + lane)] = v;
      }
  }
}

// The NCA of a batch of blocks (ACA_only_nodes per block). With far_on_gpu
// >= 2 the blocks run on the GPU, and the host keeps only those the GPU
// marked (rank capacity) or could not run; the outgoing blocks' pivot rows
// (Ar) of GPU results are filled from the table. Then the results go to
// their nodes: an empty side leaves the node inactive with its own list
// passed through.
void Builder::run_nca(std::vector<NcaJob>& jobs) {
  const double tol = std::pow(10, -1.0 * cfg.TOL_POW);
  const int nj = (int)jobs.size();
  std::vector<char> on_gpu(nj, 0);
  if (gfar && cfg.far_on_gpu >= 2) {
    std::vector<NcaTask> tasks;
    std::vector<int> which, idx;
    int piv_off = 0;
    long long idx_len = 0;
    for (int t = 0; t < nj; ++t) {
      const NcaJob& jb = jobs[t];
      if (jb.rows.empty() || jb.cols.empty()) continue;
      NcaTask tk;
      tk.idx_off = idx_len;
      tk.n1 = (int)jb.rows.size();
      tk.n2 = (int)jb.cols.size();
      tk.R = std::min(std::min(tk.n1, tk.n2), kNcaRankCap);
      tk.out_off = piv_off;
      piv_off += 2 * tk.R;
      idx_len += (long long)tk.n1 + tk.n2;
      tasks.push_back(tk);
      which.push_back(t);
    }
    // Every block's rows then columns, copied in parallel to its offset.
    idx.resize((size_t)idx_len);
#pragma omp parallel for schedule(dynamic, 64)
    for (int u = 0; u < (int)tasks.size(); ++u) {
      const NcaJob& jb = jobs[which[u]];
      int* dst = idx.data() + tasks[u].idx_off;
      std::copy(jb.rows.begin(), jb.rows.end(), dst);
      std::copy(jb.cols.begin(), jb.cols.end(), dst + jb.rows.size());
    }
    std::vector<int> ranks, piv, status;
    if (!tasks.empty() && gpu_far_nca(gfar, tasks, idx, tol, ranks, piv, status)) {
      for (size_t u = 0; u < tasks.size(); ++u) {
        if (status[u] != 0) continue;
        NcaJob& jb = jobs[which[u]];
        const NcaTask& tk = tasks[u];
        jb.rank = ranks[u];
        jb.rb.assign(piv.begin() + tk.out_off, piv.begin() + tk.out_off + jb.rank);
        jb.cb.assign(piv.begin() + tk.out_off + tk.R, piv.begin() + tk.out_off + tk.R + jb.rank);
        on_gpu[which[u]] = 1;
      }
    }
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < nj; ++t) {
    NcaJob& jb = jobs[t];
    if (jb.rows.empty() || jb.cols.empty()) continue;
    HCache hc{this, {}};
    if (!on_gpu[t]) {
      jb.rank = aca(jb.rows, jb.cols, tol, jb.rb, jb.cb, jb.out ? &jb.nd->Ar : nullptr, hc);
    } else if (jb.out && jb.rank > 0) {
      std::vector<int> prow(jb.rank);
      for (int a = 0; a < jb.rank; ++a) prow[a] = jb.rows[jb.rb[a]];
      jb.nd->Ar.assign((size_t)jb.rank * jb.cols.size(), cd(0.0, 0.0));
      fill(prow, jb.cols, hc, jb.nd->Ar.data(), (int)jb.cols.size());
    }
  }
  for (NcaJob& jb : jobs) {
    Node& nd = *jb.nd;
    const bool active = !jb.rows.empty() && !jb.cols.empty();
    if (jb.out) {
      nd.out_active = active;
      if (!active) {
        nd.out_charge = jb.cols;
      } else if (jb.rank > 0) {
        for (int r : jb.rb) nd.out_check.push_back(jb.rows[r]);
        for (int c : jb.cb) nd.out_charge.push_back(jb.cols[c]);
      }
    } else {
      nd.in_active = active;
      if (!active) {
        nd.in_check = jb.rows;
      } else if (jb.rank > 0) {
        for (int r : jb.rb) nd.in_check.push_back(jb.rows[r]);
        for (int c : jb.cb) nd.in_charge.push_back(jb.cols[c]);
      }
    }
  }
}

// NCA of the LFR level j (G_FMM2DTree.hpp:2062-2386): the outgoing block of
// a box pairs the far checks (its interaction list's, leaves: all their
// points; else their children's incoming checks) with its own charges
// (leaves: its points; else its children's outgoing charges); the incoming
// block pairs its own checks with the far charges.
void Builder::nca_level_lfr(int j) {
  const int nbx = 1 << (2 * j);
  const bool leaf = (j == nL);
  std::vector<NcaJob> jobs(2 * (size_t)nbx);
#pragma omp parallel for schedule(dynamic, 16)
  for (int t = 0; t < 2 * nbx; ++t) {
    const int k = t % nbx;
    NcaJob& jb = jobs[t];
    jb.out = t < nbx;
    jb.nd = &lfr(j, k);
    std::vector<int>& own = jb.out ? jb.cols : jb.rows;
    std::vector<int>& far = jb.out ? jb.rows : jb.cols;
    if (leaf) {
      for (int i = 0; i < rank; ++i) own.push_back(k * rank + i);
    } else {
      for (int c = 0; c < 4; ++c) {
        const Node& ch = lfr(j + 1, 4 * k + c);
        const auto& v = jb.out ? ch.out_charge : ch.in_check;
        own.insert(own.end(), v.begin(), v.end());
      }
    }
    for (int b : jb.nd->IL) {
      if (leaf) {
        for (int i = 0; i < rank; ++i) far.push_back(b * rank + i);
      } else {
        for (int c = 0; c < 4; ++c) {
          const Node& ch = lfr(j + 1, 4 * b + c);
          const auto& v = jb.out ? ch.in_check : ch.out_charge;
          far.insert(far.end(), v.begin(), v.end());
        }
      }
    }
  }
  run_nca(jobs);
}

// NCA of the HFR level j (G_FMM2DTree.hpp:3232-3571), per box and cone:
// own charges / checks from the children's nodes for that cone, far ones
// from the interaction list's boxes through the cone that faces this box.
void Builder::nca_level_hfr(int j) {
  const int nbx = 1 << (2 * j), nc = nCones[j];
  auto gather = [&](int jj, int kk, int cn, bool charges, std::vector<int>& dst) {
    for (int c = 0; c < 4; ++c) {
      Node& ch = child_node(jj + 1, 4 * kk + c, cn);
      const auto& v = charges ? ch.out_charge : ch.in_check;
      dst.insert(dst.end(), v.begin(), v.end());
    }
  };
  const int nn = nbx * nc;
  std::vector<NcaJob> jobs(2 * (size_t)nn);
#pragma omp parallel for schedule(dynamic, 16)
  for (int t = 0; t < 2 * nn; ++t) {
    const int u = t % nn, k = u / nc, cn = u % nc;
    NcaJob& jb = jobs[t];
    jb.out = t < nn;
    jb.nd = &cone(j, k, cn);
    std::vector<int>& own = jb.out ? jb.cols : jb.rows;
    std::vector<int>& far = jb.out ? jb.rows : jb.cols;
    gather(j, k, cn, jb.out, own);
    for (int b : jb.nd->IL) gather(j, b, cone_towards(cx[j], cy[j], k, b, aperture[j]), !jb.out, far);
  }
  run_nca(jobs);
}

void Builder::user_checks() {
  for (int j = nL; j >= level_LFR; --j)
    for (int k = 0; k < (1 << (2 * j)); ++k) {
      Node& nd = lfr(j, k);
      if (j == nL) {
        nd.user_check.clear();
        for (int i = 0; i < rank; ++i) nd.user_check.push_back(k * rank + i);
      } else if (nd.in_active) {
        nd.user_check = nd.in_check;
      } else {
        for (int c = 0; c < 4; ++c) { const auto& v = lfr(j + 1, 4 * k + c).user_check; nd.user_check.insert(nd.user_check.end(), v.begin(), v.end()); }
      }
    }
  for (int j = level_LFR - 1; j >= 2; --j)
    for (int k = 0; k < (1 << (2 * j)); ++k)
      for (int cn = 0; cn < nCones[j]; ++cn) {
        Node& nd = cone(j, k, cn);
        if (nd.in_active) nd.user_check = nd.in_check;
        else for (int c = 0; c < 4; ++c) { const auto& v = child_node(j + 1, 4 * k + c, cn).user_check; nd.user_check.insert(nd.user_check.end(), v.begin(), v.end()); }
      }
}

// Appends a row-major block (rows x K) with its gather list to a phase.
// Hands blocks to a phase for packing, in the order t = 0..n-1: get(t)
// gives block t (A: rows x K, row major; idx: at least K gather indices;
// its first row writes output element `out`); rows or K = 0 skips it. The
// phase takes the two vectors over (a move, no copy) and records one row
// per block row.
struct BlockView {
  std::vector<cd>* A;
  int rows, K;
  std::vector<int>* idx;
  int out;
  // A == nullptr: the block is filled from the far-field table, row r from
  // target point (*rowpts)[r] against the source points *colpts.
  std::vector<int>* rowpts = nullptr;
  std::vector<int>* colpts = nullptr;
};
template <class Get>
static void stage_blocks(GemvPhase& ph, int n, Get get) {
  for (int t = 0; t < n; ++t) {
    const BlockView v = get(t);
    if (v.rows <= 0 || v.K <= 0) continue;
    ph.stageIdx.push_back(std::move(*v.idx));
    const int* ix = ph.stageIdx.back().data();
    if (v.A) {
      ph.stageA.push_back(std::move(*v.A));
      const cd* a = ph.stageA.back().data();
      for (int r = 0; r < v.rows; ++r) ph.rows.push_back({a + (size_t)r * v.K, v.K, ix, v.out + r});
    } else {
      ph.stageCols.push_back(std::move(*v.colpts));
      const int* cp = ph.stageCols.back().data();
      for (int r = 0; r < v.rows; ++r) ph.rows.push_back({nullptr, v.K, ix, v.out + r, (*v.rowpts)[r], cp});
    }
    ph.nnz += (long long)v.rows * v.K;
  }
}

// Packs the staged blocks into warp tiles (see GemvTile). A tile holds R
// rows of ONE block, R a power of two, so its rows share their gather list
// and the tile stores one index per column slice and step (S = 32 / R per
// step) instead of one per element. A block of r rows is cut into tiles of
// R = 16, 8, ... rows (largest first) so that no rows are padded, except
// that R never drops below r_min: slices must keep at least 4 columns
// (R >= 128 / K), and the last tile of a block pads up to r_min. r_max
// (at most 8) keeps at least ~7,300 tiles per phase (one wave of 48 warps
// on each of 152 SMs): fewer, longer warps leave too few loads in flight to
// cover HBM latency, more and shorter ones spend their time in the slice
// combination (measured on GB300: 96 warps per SM was 3-8% slower, 32 and
// 24 slower again, rows up to 16 slower for FP32 and double-float). Blocks
// go longest first (stable, so neighbouring blocks keep their order).
static int pow2_ceil(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Tile knobs of one phase kind ("UP", "M2L", "DOWN"): the largest rows per
// tile (1, 2, 4 or 8) and the warps per SM that the tile count aims at.
// Defaults 8 and 48; the environment variable LS_TILE_<kind> = "rows,warps"
// overrides them (set by lippmann_schwinger_solver_gb300.autotune, which
// times the candidates on the GPU).
struct TileKnobs {
  int rows = 8;
  int warps = 48;
};

static TileKnobs tile_knobs(const char* kind) {
  TileKnobs k;
  const std::string name = std::string("LS_TILE_") + kind;
  const char* v = std::getenv(name.c_str());
  int r = 0, w = 0;
  if (v && std::sscanf(v, "%d,%d", &r, &w) == 2 && (r == 1 || r == 2 || r == 4 || r == 8) && w >= 1 && w <= 1024) {
    k.rows = r;
    k.warps = w;
  }
  return k;
}

// Rows staged without values (table blocks) leave ph.A empty: the tiles
// are described in *fill (row points in *frows, each block's source points
// once in *fcols) and ph.dev_A_elems holds their size, for a fill from the
// far-field table on the device or on the host.
static void finalize(GemvPhase& ph, const char* kind, std::vector<FillTile>* fill = nullptr,
                     std::vector<int>* frows = nullptr, std::vector<int>* fcols = nullptr) {
  struct Block { size_t r0; int rows, K; };
  std::vector<Block> blocks;
  for (size_t r = 0; r < ph.rows.size();) {
    size_t e = r + 1;
    while (e < ph.rows.size() && ph.rows[e].idx == ph.rows[r].idx) ++e;
    blocks.push_back({r, (int)(e - r), ph.rows[r].K});
    r = e;
  }
  std::stable_sort(blocks.begin(), blocks.end(), [](const Block& a, const Block& b) { return a.K > b.K; });
  const TileKnobs kn = tile_knobs(kind);
  const long long want_tiles = 152LL * kn.warps;
  int r_max = kn.rows;
  while (r_max > 1 && (long long)ph.rows.size() < want_tiles * r_max) r_max >>= 1;
  struct T { size_t r0; int rows, S, qmax, K; long long off, ioff; int row_base; };
  std::vector<T> tl;
  long long total = 0, total_idx = 0;
  int total_rows = 0;
  ph.blk_tile0.clear();
  ph.blk_rows.clear();
  ph.blk_K.clear();
  for (const Block& b : blocks) {
    ph.blk_tile0.push_back((int)tl.size());
    ph.blk_rows.push_back(b.rows);
    ph.blk_K.push_back(b.K);
    const int r_min = std::min(kTileLanes, pow2_ceil((128 + b.K - 1) / b.K));
    const int rcap = std::max(r_max, r_min);
    for (int done = 0; done < b.rows;) {
      const int rem = b.rows - done;
      int R = 1;
      while (R * 2 <= std::min(rem, rcap)) R *= 2;
      R = std::max(R, r_min);
      const int rows = std::min(R, rem);
      const int S = kTileLanes / R;
      const int qmax = (b.K + S - 1) / S;
      tl.push_back({b.r0 + (size_t)done, rows, S, qmax, b.K, total, total_idx, total_rows});
      total += (long long)qmax * kTileLanes;
      total_idx += (long long)qmax * S;
      total_rows += rows;
      done += rows;
    }
  }
  ph.blk_tile0.push_back((int)tl.size());
  const bool table = !ph.rows.empty() && ph.rows[0].a == nullptr;
  if (table) {
    fill->clear();
    frows->clear();
    fcols->clear();
    const int* last_cols = nullptr;
    long long col_off = 0;
    for (const T& d : tl) {
      const GemvPhase::Row& first = ph.rows[d.r0];
      if (first.cpt != last_cols) {
        col_off = (long long)fcols->size();
        fcols->insert(fcols->end(), first.cpt, first.cpt + d.K);
        last_cols = first.cpt;
      }
      int log2s = 0;
      while ((1 << log2s) < d.S) ++log2s;
      fill->push_back({d.off, (long long)frows->size(), col_off, d.qmax, d.rows, log2s, d.K});
      for (int r = 0; r < d.rows; ++r) frows->push_back(ph.rows[d.r0 + r].pt);
    }
    ph.dev_A_elems = total;
  } else {
    ph.A.resize((size_t)total);  // uninitialised: each tile zeroes and fills its own range below
  }
  ph.idx.assign((size_t)total_idx, 0);
  ph.out.assign(ph.rows.size(), 0);
  ph.klen.assign(tl.size() * kTileLanes, 0);
  // Tiles own disjoint ranges of A, idx, klen and out: fill them in parallel.
  ph.tiles.assign(tl.size(), GemvTile{});
#pragma omp parallel for schedule(dynamic, 64)
  for (size_t t = 0; t < tl.size(); ++t) {
    const T& d = tl[t];
    const int R = kTileLanes / d.S;
    int log2s = 0;
    while ((1 << log2s) < d.S) ++log2s;
    const GemvPhase::Row& first = ph.rows[d.r0];
    if (!table)
      std::fill(ph.A.begin() + d.off, ph.A.begin() + d.off + (long long)d.qmax * kTileLanes, cplx{0.0, 0.0});
    for (int q = 0; q < d.qmax; ++q)
      for (int sl = 0; sl < d.S; ++sl) {
        const int k = q * d.S + sl;
        if (k < d.K) ph.idx[(size_t)(d.ioff + (long long)q * d.S + sl)] = first.idx[k];
      }
    for (int r = 0; r < d.rows; ++r) {
      const GemvPhase::Row& row = ph.rows[d.r0 + r];
      ph.out[(size_t)d.row_base + r] = row.out;
      for (int sl = 0; sl < d.S; ++sl) {
        const int lane = sl * R + r;
        int q = 0;
        for (int k = sl; k < row.K; k += d.S, ++q)
          if (!table) ph.A[(size_t)(d.off + (long long)q * kTileLanes + lane)] = cplx{row.a[k].real(), row.a[k].imag()};
        ph.klen[t * kTileLanes + lane] = q;
      }
    }
    ph.tiles[t] = {d.off, d.ioff, d.qmax, d.rows, log2s, (int)(t * kTileLanes), d.row_base};
  }
  std::vector<std::vector<cd>>().swap(ph.stageA);
  std::vector<std::vector<int>>().swap(ph.stageIdx);
  std::vector<std::vector<int>>().swap(ph.stageCols);
  std::vector<GemvPhase::Row>().swap(ph.rows);
}

void Builder::pack(HostOperator& op) {
  const int nleaf = 1 << (2 * nL);
  // ---- charge buffer: x, then own skeleton charges level by level.
  long long S = N;
  for (int j = nL; j >= 2; --j) {
    for (auto& nd : nodes[j])
      if (nd.out_active && !nd.out_charge.empty()) { nd.own_charge = S; S += (long long)nd.out_charge.size(); }
  }
  // f_out gather lists, bottom up.
  for (int j = nL; j >= 2; --j) {
    const int nbx = 1 << (2 * j);
    const int ncn = is_lfr(j) ? 1 : nCones[j];
    for (int k = 0; k < nbx; ++k)
      for (int cn = 0; cn < ncn; ++cn) {
        Node& nd = is_lfr(j) ? lfr(j, k) : cone(j, k, cn);
        nd.fidx.clear();
        if (nd.out_active) {
          for (long long s = 0; s < (long long)nd.out_charge.size(); ++s) nd.fidx.push_back((int)(nd.own_charge + s));
        } else if (j == nL) {
          for (int i = 0; i < rank; ++i) nd.fidx.push_back(k * rank + i);
        } else {
          for (int c = 0; c < 4; ++c) {
            const auto& v = child_node(j + 1, 4 * k + c, cn).fidx;
            nd.fidx.insert(nd.fidx.end(), v.begin(), v.end());
          }
        }
      }
  }
  // ---- which potentials can be nonzero: a node's potential is nonzero
  // when it has an M2L term with at least one source charge, or when a
  // parent with a nonzero potential passes something down (top down).
  for (int j = 2; j <= nL; ++j) {
    const int nn = (int)nodes[j].size();
    for (int t = 0; t < nn; ++t) {
      Node& X = nodes[j][t];
      X.pot_nonzero = false;
      if (X.user_check.empty()) continue;
      const int k = is_lfr(j) ? t : t / nCones[j];
      if (X.in_active) {
        for (int b : X.IL) {
          const Node& src = is_lfr(j) ? lfr(j, b) : cone(j, b, cone_towards(cx[j], cy[j], k, b, aperture[j]));
          if (!src.out_charge.empty()) { X.pot_nonzero = true; break; }
        }
      }
      if (X.pot_nonzero || j == 2) continue;
      const int cc = is_lfr(j) ? 0 : t % nCones[j];
      const int kp = k / 4, jp = j - 1;
      const int npc = is_lfr(jp) ? 1 : nCones[jp];
      for (int pc = 0; pc < npc && !X.pot_nonzero; ++pc) {
        if (!is_lfr(jp) && !is_lfr(j) && pc / 2 != cc) continue;
        const Node& p = is_lfr(jp) ? lfr(jp, kp) : cone(jp, kp, pc);
        if (p.pot_nonzero && (!p.in_active || !p.in_charge.empty())) X.pot_nonzero = true;
      }
    }
  }
  // ---- potential buffer: leaves (N), then every other node whose
  // potential can be nonzero.
  long long P = N;
  for (int k = 0; k < nleaf; ++k) lfr(nL, k).pot_off = (long long)k * rank;
  for (int j = 2; j < nL; ++j)
    for (auto& nd : nodes[j])
      if (nd.pot_nonzero && !nd.user_check.empty()) { nd.pot_off = P; P += (long long)nd.user_check.size(); }
  op.charges_len = S;
  op.pots_len = P;

  // ---- upward pass: T = Atilde^{-1} Ar for every node with a skeleton.
  op.up.clear();
  for (int j = nL; j >= 2; --j) {
    GemvPhase ph;
    const int nn = (int)nodes[j].size();
    std::vector<std::vector<cd>> T(nn);
    std::vector<std::vector<int>> src(nn);
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < nn; ++t) {
      Node& nd = nodes[j][t];
      if (!(nd.out_active && !nd.out_charge.empty())) continue;
      const int k = is_lfr(j) ? t : t / nCones[j];
      const int cn = is_lfr(j) ? 0 : t % nCones[j];
      std::vector<int> s;
      if (j == nL) for (int i = 0; i < rank; ++i) s.push_back(k * rank + i);
      else for (int c = 0; c < 4; ++c) { const auto& v = child_node(j + 1, 4 * k + c, cn).fidx; s.insert(s.end(), v.begin(), v.end()); }
      const int r = (int)nd.out_charge.size(), K = (int)s.size();
      if (K == 0) continue;
      HCache hc{this, {}};
      PivQR qr;
      qr.factor(r, r, block_colmajor(nd.out_check, nd.out_charge, hc));
      std::vector<cd> Tm((size_t)r * K), col(r), sol(r);
      for (int c = 0; c < K; ++c) {
        for (int a = 0; a < r; ++a) col[a] = nd.Ar[(size_t)a * K + c];
        qr.solve(col.data(), sol.data());
        for (int a = 0; a < r; ++a) Tm[(size_t)a * K + c] = sol[a];
      }
      T[t] = std::move(Tm);
      src[t] = std::move(s);
    }
    stage_blocks(ph, nn, [&](int t) {
      if (T[t].empty()) return BlockView{nullptr, 0, 0, nullptr, 0};
      return BlockView{&T[t], (int)nodes[j][t].out_charge.size(), (int)src[t].size(), &src[t],
                       (int)nodes[j][t].own_charge};
    });
    finalize(ph, "UP");
    op.up.push_back(std::move(ph));
  }

  // ---- M2L: one task per node with an incoming interaction list. With
  // far_on_gpu = 3 the blocks keep only their target and source points and
  // their tiles are filled from the far-field table on the device.
  {
    struct Task { std::vector<cd> A; std::vector<int> idx, rowpts, colpts; int rows = 0, K = 0; long long out = 0; };
    const bool by_table = dense && cfg.far_on_gpu >= 3;
    std::vector<std::pair<int, int>> all;
    for (int j = 2; j <= nL; ++j)
      for (int t = 0; t < (int)nodes[j].size(); ++t) all.push_back({j, t});
    std::vector<Task> tasks(all.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (int u = 0; u < (int)all.size(); ++u) {
      const int j = all[u].first, t = all[u].second;
      Node& nd = nodes[j][t];
      if (!nd.in_active || nd.user_check.empty()) continue;
      const int k = is_lfr(j) ? t : t / nCones[j];
      std::vector<const Node*> srcs;
      for (int b : nd.IL) {
        const Node& s = is_lfr(j) ? lfr(j, b) : cone(j, b, cone_towards(cx[j], cy[j], k, b, aperture[j]));
        if (!s.out_charge.empty()) srcs.push_back(&s);
      }
      int K = 0;
      for (const Node* s : srcs) K += (int)s->out_charge.size();
      if (K == 0) continue;
      const int rows = (int)nd.user_check.size();
      HCache hc{this, {}};
      Task& tk = tasks[u];
      if (!by_table) tk.A.resize((size_t)rows * K);
      int c0 = 0;
      for (const Node* s : srcs) {
        if (by_table)
          tk.colpts.insert(tk.colpts.end(), s->out_charge.begin(), s->out_charge.end());
        else
          fill(nd.user_check, s->out_charge, hc, tk.A.data() + c0, K);
        tk.idx.insert(tk.idx.end(), s->fidx.begin(), s->fidx.end());
        c0 += (int)s->out_charge.size();
      }
      if (by_table) tk.rowpts = nd.user_check;
      tk.rows = rows;
      tk.K = K;
      tk.out = nd.pot_off;
    }
    GemvPhase ph;
    op.m2l_rows = 0;
    for (auto& tk : tasks)
      if (tk.K != 0) op.m2l_rows += tk.rows;
    stage_blocks(ph, (int)tasks.size(), [&](int u) {
      Task& tk = tasks[u];
      if (tk.K == 0) return BlockView{nullptr, 0, 0, nullptr, 0};
      if (by_table) return BlockView{nullptr, tk.rows, tk.K, &tk.idx, (int)tk.out, &tk.rowpts, &tk.colpts};
      return BlockView{&tk.A, tk.rows, tk.K, &tk.idx, (int)tk.out};
    });
    if (by_table) {
      std::vector<FillTile> fl;
      std::vector<int> frows, fcols;
      finalize(ph, "M2L", &fl, &frows, &fcols);
      ph.dev_A = gfar ? gpu_far_fill(gfar, fl, frows, fcols, ph.dev_A_elems) : nullptr;
      if (!ph.dev_A) fill_tiles_host(ph, fl, frows, fcols);
    } else {
      finalize(ph, "M2L");
    }
    op.m2l = std::move(ph);
  }

  // ---- downward pass: child pulls W = L2L Atilde^{-1} (or a slice when the
  // parent is a pass-through), parents in cone order.
  op.down.clear();
  for (int j = 2; j < nL; ++j) {
    const int J = j + 1;
    // QR of Atilde^T for every IL-active parent. W = L2L Atilde^{-1} is
    // formed row by row by solving Atilde^T w^T = l^T: the rounding error of
    // each row then lies along left singular vectors of Atilde with small
    // singular values, which the parent's potential (in the range of
    // Atilde) does not excite. An explicit inverse would not have this
    // property and loses ~eps * cond(Atilde) in the product.
    const int np = (int)nodes[j].size();
    std::vector<PivQR> AT(np);
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < np; ++t) {
      Node& p = nodes[j][t];
      if (!(p.in_active && !p.in_charge.empty() && p.pot_nonzero)) continue;
      HCache hc{this, {}};
      const int r = (int)p.in_charge.size();
      const std::vector<cd> A = block_colmajor(p.in_check, p.in_charge, hc);
      std::vector<cd> At((size_t)r * r);
      for (int a = 0; a < r; ++a)
        for (int c = 0; c < r; ++c) At[(size_t)c * r + a] = A[(size_t)a * r + c];  // At(a,c) = A(c,a)
      AT[t].factor(r, r, At);
    }
    const int nch = (int)nodes[J].size();
    struct Task { std::vector<cd> A; std::vector<int> idx; int rows = 0, K = 0; long long out = 0; bool any = false; };
    std::vector<Task> tasks(nch);
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < nch; ++t) {
      Node& X = nodes[J][t];
      const int rows = (int)X.user_check.size();
      if (rows == 0) continue;
      const int kc = is_lfr(J) ? t : t / nCones[J];
      const int cc = is_lfr(J) ? 0 : t % nCones[J];
      const int kp = kc / 4, child = kc % 4;
      std::vector<int> pcones;
      if (is_lfr(j)) pcones.push_back(-1);
      else for (int pc = 0; pc < nCones[j]; ++pc) if (is_lfr(J) || pc / 2 == cc) pcones.push_back(pc);
      HCache hc{this, {}};
      Task& tk = tasks[t];
      std::vector<std::vector<cd>> cols_blocks;  // per term, row-major rows x w
      std::vector<int> widths;
      for (int pc : pcones) {
        const int pt = (pc < 0) ? kp : kp * nCones[j] + pc;
        Node& p = nodes[j][pt];
        if (!p.pot_nonzero) continue;
        if (p.in_active) {
          if (p.in_charge.empty()) continue;
          const int r = (int)p.in_charge.size();
          std::vector<cd> Lb((size_t)rows * r);
          fill(X.user_check, p.in_charge, hc, Lb.data(), r);
          std::vector<cd> W((size_t)rows * r, cd(0.0, 0.0));
          for (int a = 0; a < rows; ++a) AT[pt].solve(&Lb[(size_t)a * r], &W[(size_t)a * r]);
          cols_blocks.push_back(std::move(W));
          widths.push_back(r);
          for (int m = 0; m < r; ++m) tk.idx.push_back((int)(p.pot_off + m));
        } else {
          // Pass-through: slice of the parent's potential for this child.
          int off = 0;
          for (int c = 0; c < child; ++c) off += (int)child_node(J, 4 * kp + c, pc < 0 ? 0 : pc).user_check.size();
          std::vector<cd> Id((size_t)rows * rows, cd(0.0, 0.0));
          for (int a = 0; a < rows; ++a) Id[(size_t)a * rows + a] = 1.0;
          cols_blocks.push_back(std::move(Id));
          widths.push_back(rows);
          for (int m = 0; m < rows; ++m) tk.idx.push_back((int)(p.pot_off + off + m));
        }
      }
      int K = 0;
      for (int w : widths) K += w;
      if (K == 0) continue;
      tk.A.assign((size_t)rows * K, cd(0.0, 0.0));
      int c0 = 0;
      for (size_t b = 0; b < cols_blocks.size(); ++b) {
        for (int a = 0; a < rows; ++a)
          for (int c = 0; c < widths[b]; ++c) tk.A[(size_t)a * K + c0 + c] = cols_blocks[b][(size_t)a * widths[b] + c];
        c0 += widths[b];
      }
      tk.rows = rows;
      tk.K = K;
      tk.out = X.pot_off;
      tk.any = true;
    }
    GemvPhase ph;
    ph.accumulate = 1;
    stage_blocks(ph, nch, [&](int t) {
      Task& tk = tasks[t];
      if (!tk.any) return BlockView{nullptr, 0, 0, nullptr, 0};
      return BlockView{&tk.A, tk.rows, tk.K, &tk.idx, (int)tk.out};
    });
    finalize(ph, "DOWN");
    op.down.push_back(std::move(ph));
  }
}

bool Builder::run(HostOperator& op, std::string& err) {
  const auto t0 = std::chrono::steady_clock::now();
  // Depth 2 would put level_LFR = min(max(., 2), nLevels - 1) below the
  // coarsest far-field level 2, which the level structure does not allow.
  if (cfg.nLevelsUniform < 3 || cfg.nLevelsUniform > 10) { err = "nLevelsUniform must be in [3, 10]"; return false; }
  if (cfg.nChebNodes < 2 || cfg.nChebNodes > 8) { err = "nChebNodes must be in [2, 8]"; return false; }
  if (cfg.degreeOfBases < 1 || cfg.degreeOfBases * (cfg.degreeOfBases + 1) / 2 > cfg.nChebNodes * cfg.nChebNodes) {
    err = "degreeOfBases gives more basis polynomials than nodes"; return false;
  }
  if (!(cfg.L > 0.0) || !(cfg.kappa >= 0.0)) { err = "L must be > 0 and kappa >= 0"; return false; }
  if (cfg.Qchoice < 0 || cfg.Qchoice > 6) { err = "Qchoice must be in [0, 6]"; return false; }
  if (cfg.Qchoice == 6 && (cfg.n_bumps < 1 || cfg.n_bumps > LS_MAX_BUMPS)) { err = "n_bumps must be in [1, 8]"; return false; }
  if (cfg.nCones_LFR < 1 || cfg.TOL_POW < 1 || cfg.TOL_POW > 16) { err = "nCones_LFR >= 1 and TOL_POW in [1, 16] required"; return false; }
  if ((long long)(1LL << (2 * cfg.nLevelsUniform)) * cfg.nChebNodes * cfg.nChebNodes > (1LL << 28)) { err = "problem too large"; return false; }
  auto lap = [t = t0]() mutable {
    const auto now = std::chrono::steady_clock::now();
    const double s = std::chrono::duration<double>(now - t).count();
    t = now;
    return s;
  };
  geometry();
  op.stage_seconds[0] = lap();
  precompute();
  htab.set_width(rank);
  op.stage_seconds[1] = lap();
  interaction_lists();
  op.stage_seconds[2] = lap();
  far_tables();
  for (int j = nL; j >= level_LFR; --j) nca_level_lfr(j);
  for (int j = level_LFR - 1; j >= 2; --j) nca_level_hfr(j);
  op.stage_seconds[3] = lap();
  user_checks();
  op.stage_seconds[4] = lap();
  pack(op);
  htab.clear();
  gpu_far_close(gfar);
  gfar = nullptr;
  dense = false;
  dS.reset();
  op.stage_seconds[5] = lap();
  // Operator-level data for the near field and the C ABI.
  op.cfg = cfg;
  op.N = N;
  op.n_leaves = 1 << (2 * nL);
  op.rank = rank;
  op.n_levels = nL;
  op.level_LFR = level_LFR;
  op.n_bases = nb;
  op.px = gx_;
  op.py = gy_;
  op.q.resize(N);
  for (int i = 0; i < N; ++i) op.q[i] = contrast_fn(cfg, gx_[i], gy_[i]);
  op.kq = kq_;
  op.nearB = near;
  op.nearVt = nearVt;
  op.nearE = nearE;
  op.Qpinv = Qpinv;
  op.M.assign((size_t)rank * (2 * kSeries + 1), cd());
  for (size_t i = 0; i < op.M.size(); ++i) op.M[i] = Mleaf[i];
  // Colleague table of the leaves (getNeighbors, G_FMM2DTree.hpp:1567-1601):
  // slot n <-> offset of N_centers[n] / 2 in box units.
  static const int ox[9] = {-1, 0, 1, 1, 1, 0, -1, -1, 0};
  static const int oy[9] = {-1, -1, -1, 0, 1, 1, 1, 0, 0};
  const int nleaf = op.n_leaves;
  op.colleague.assign((size_t)nleaf * 9, -1);
  {
    // grid coordinates of each leaf from its centre
    const double w = 2.0 * radius[nL];
    std::unordered_map<long long, int> at;
    auto gidx = [&](double x, double y) { return std::llround((x + L) / w - 0.5) * 4194304LL + std::llround((y + L) / w - 0.5); };
    for (int t = 0; t < nleaf; ++t) at[gidx(cx[nL][t], cy[nL][t])] = t;
    for (int t = 0; t < nleaf; ++t) {
      const long long gxi = std::llround((cx[nL][t] + L) / w - 0.5), gyi = std::llround((cy[nL][t] + L) / w - 0.5);
      for (int q = 0; q < 9; ++q) {
        auto it = at.find((gxi + ox[q]) * 4194304LL + (gyi + oy[q]));
        if (it != at.end()) op.colleague[(size_t)t * 9 + q] = it->second;
      }
    }
  }
  // Skeleton dump (same record format as the CPU oracle).
  op.skeleton_dump.clear();
  int mr = 0;
  auto put = [&](int v) { op.skeleton_dump.push_back(v); };
  auto putv = [&](const std::vector<int>& v) { put((int)v.size()); for (int x : v) put(x); };
  for (int j = 2; j <= nL; ++j)
    for (int k = 0; k < (1 << (2 * j)); ++k) {
      const int ncn = is_lfr(j) ? 1 : nCones[j];
      for (int cn = 0; cn < ncn; ++cn) {
        const Node& nd = is_lfr(j) ? lfr(j, k) : cone(j, k, cn);
        put(j); put(k); put(is_lfr(j) ? -1 : cn); put(nd.out_active); put(nd.in_active);
        putv(nd.out_charge); putv(nd.out_check); putv(nd.in_charge); putv(nd.in_check); putv(nd.user_check);
        if (nd.out_active) mr = std::max(mr, (int)nd.out_charge.size());
        if (nd.in_active) mr = std::max(mr, (int)nd.in_charge.size());
      }
    }
  op.max_rank = mr;
  op.assemble_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return true;
}

#include "assemble_adaptive.h"

}  // namespace

bool assemble(const ls_config& cfg, HostOperator& op, std::string& err) {
  try {
    if (cfg.tree_adaptive) {
      AdaptiveBuilder b(cfg);
      return b.run(op, err);
    }
    Builder b(cfg);
    return b.run(op, err);
  } catch (const std::bad_alloc&) {
    err = "host allocation failed during assembly";
    return false;
  } catch (const std::exception& e) {
    err = std::string("assembly failed: ") + e.what();
    return false;
  }
}

double contrast_at(const ls_config& cfg, double x, double y) { return contrast_fn(cfg, x, y); }

void set_assembly_device(int device) { t_assembly_device = device; }

void precompute_cache_set(const char* dir) { g_pcache.set(dir); }
void precompute_cache_stats(long long& hits, long long& misses) { g_pcache.stats(hits, misses); }

// The GPU quadrature (csrc/quadrature.cu) replaces this stub in the library;
// a host-only build keeps it and integrates on the host.
__attribute__((weak)) GpuFar* gpu_far_open(int, const FarTables&, cd*) { return nullptr; }
__attribute__((weak)) bool gpu_far_nca(GpuFar*, const std::vector<NcaTask>&, const std::vector<int>&, double,
                                       std::vector<int>&, std::vector<int>&, std::vector<int>&) {
  return false;
}
__attribute__((weak)) void gpu_far_close(GpuFar*) {}
__attribute__((weak)) void* gpu_far_fill(GpuFar*, const std::vector<FillTile>&, const std::vector<int>&,
                                         const std::vector<int>&, long long) {
  return nullptr;
}
__attribute__((weak)) void gpu_far_free(void*) {}
__attribute__((weak)) bool gpu_quadrature(int, const std::vector<QuadTask>&, const std::vector<double>&,
                                          const std::vector<double>&, std::vector<cd>&) {
  return false;
}

}  // namespace lsg
