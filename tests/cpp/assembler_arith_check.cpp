// Checks that the assembler's fast forms of three ACA building blocks give
// exactly the results of their plain forms: the pivot search (hypot only
// near the largest squared magnitude) against a full hypot scan, and the
// real-arithmetic inner product and rank-1 update against std::complex.
// Compiled against the assembler source itself so that the functions under
// test are the ones the library runs. Exit status 0 = all equal.
#include "../../lippmann_schwinger_solver_gb300/csrc/assemble.cpp"

#include <cstdint>
#include <cstdio>
#include <random>

namespace {

using cd = std::complex<double>;

int full_scan(const std::vector<cd>& v, const std::vector<char>& used) {
  int idx = -1;
  double mx = 0.0;
  for (int i = 0; i < (int)v.size(); ++i) {
    if (used[i]) continue;
    if (idx < 0) { idx = i; mx = std::abs(v[i]); continue; }
    if (std::abs(v[i]) > mx) { idx = i; mx = std::abs(v[idx]); }
  }
  return idx < 0 ? 0 : idx;
}

cd plain_cdot(const std::vector<cd>& a, const std::vector<cd>& b) {
  cd s(0.0, 0.0);
  for (size_t i = 0; i < a.size(); ++i) s += std::conj(a[i]) * b[i];
  return s;
}

bool same_bits(double a, double b) {
  uint64_t x, y;
  std::memcpy(&x, &a, 8);
  std::memcpy(&y, &b, 8);
  return x == y;
}
bool same_bits(const cd& a, const cd& b) { return same_bits(a.real(), b.real()) && same_bits(a.imag(), b.imag()); }

}  // namespace

int main() {
  std::mt19937_64 g(20261203);
  std::uniform_real_distribution<double> u(-1.0, 1.0), ph(0.0, 6.283185307179586);
  long long bad_pivot = 0, bad_dot = 0, bad_update = 0;
  for (int t = 0; t < 200000; ++t) {
    const int n = 1 + (int)(g() % 64);
    std::vector<cd> v(n);
    std::vector<char> used(n);
    const double R = std::exp(20.0 * u(g));
    for (int i = 0; i < n; ++i) {
      used[i] = (g() % 4) == 0;
      switch (t % 8) {
        case 0: v[i] = cd(u(g), u(g)); break;
        case 1: v[i] = std::polar(R, ph(g)); break;  // equal magnitudes, many phases
        case 2: v[i] = std::polar(R * (1.0 + 1e-16 * (double)(g() % 7)), ph(g)); break;
        case 3: { const double x = u(g); v[i] = (g() % 2) ? cd(x, 0.0) : cd(0.0, std::nextafter(x, 2.0)); } break;
        case 4: v[i] = (g() % 3 == 0) ? cd(0.0, 0.0) : cd(std::nextafter(R, 0.0) * ((g() % 2) ? 1.0 : -1.0), 0.0); break;
        case 5: v[i] = cd((g() % 2) ? -0.0 : 0.0, (g() % 2) ? -0.0 : u(g) * 1e-300); break;  // zeros and tiny values
        case 6: v[i] = std::polar(1e-160 * (1.0 + 1e-7 * (double)(g() % 5)), ph(g)); break;  // subnormal squares
        default: v[i] = std::polar(std::exp(-345.0 - 15.0 * std::fabs(u(g))), ph(g)); break;  // squares near underflow

      }
    }
    if (lsg::argmax_remaining(v, used) != full_scan(v, used)) ++bad_pivot;
    std::vector<cd> w(n);
    for (int i = 0; i < n; ++i) w[i] = (t % 8 == 5) ? cd(-0.0, u(g)) : cd(u(g) * R, u(g));
    if (!same_bits(lsg::cdot(v, w), plain_cdot(v, w))) ++bad_dot;
    const cd f(u(g), (t % 3 == 0) ? -0.0 : u(g));
    std::vector<cd> a = v, b = v;
    lsg::sub_scaled(a, f, w);
    for (int i = 0; i < n; ++i) b[i] -= f * w[i];
    for (int i = 0; i < n; ++i)
      if (!same_bits(a[i], b[i])) { ++bad_update; break; }
  }
  std::printf("pivot mismatches %lld, inner-product mismatches %lld, update mismatches %lld\n", bad_pivot, bad_dot,
              bad_update);
  return (bad_pivot || bad_dot || bad_update) ? 1 : 0;
}
