// Runs an assembled operator's packed gather-GEMV program (the phases the
// device kernels execute) on the host, touching exactly the words the
// device's gemv_tiles_kernel reads and writes, after checking that every
// one of them lies inside its buffer:
//   - a tile's A, idx, lane-length and output ranges lie inside the phase;
//   - every gather index lies inside the source buffer, every output row
//     inside the destination buffer;
//   - no output row is written twice in one phase (the kernel's
//     read-modify-write of an accumulating phase is not atomic);
//   - a phase that reads and writes the same buffer never reads a row it
//     writes (its tiles run concurrently).
// Compiled against the assembler source itself (host code only).
//
// usage: packed_program_check <ls_config bytes> <x: N complex128> <y out> [--far-only]
// --far-only: y is the far part alone (the leaf potentials after the upward,
// M2L and downward phases), for uniform trees, whose near field is not a
// packed phase.
// Exit status: 0 = all checks passed and y written; 2 = bad arguments;
// 3 = assembly failed; 4 = a check failed (reason on stderr).
#include "../../lippmann_schwinger_solver_gb300/csrc/assemble.cpp"

#include <cstdio>

namespace {

using lsg::cd;
using lsg::GemvPhase;

bool fail(const char* phase, const char* what, long long a, long long b) {
  std::fprintf(stderr, "%s: %s (%lld, %lld)\n", phase, what, a, b);
  return false;
}

bool run_phase(const GemvPhase& ph, const std::vector<cd>& src, std::vector<cd>& dst, bool in_place,
               const char* name) {
  const int L = lsg::kTileLanes;
  std::vector<char> written(dst.size(), 0), read(src.size(), 0);
  std::vector<std::pair<int, cd>> result;
  for (size_t t = 0; t < ph.tiles.size(); ++t) {
    const lsg::GemvTile& T = ph.tiles[t];
    if (T.log2s < 0 || T.log2s > 5) return fail(name, "log2s", (long long)t, T.log2s);
    const int S = 1 << T.log2s, R = L >> T.log2s;
    if (T.rows < 1 || T.rows > R) return fail(name, "rows", (long long)t, T.rows);
    if (T.a_off < 0 || T.a_off + (long long)T.qmax * L > (long long)ph.A.size())
      return fail(name, "A range", (long long)t, T.a_off);
    if (T.i_off < 0 || T.i_off + (long long)T.qmax * S > (long long)ph.idx.size())
      return fail(name, "idx range", (long long)t, T.i_off);
    if (T.lane_base < 0 || T.lane_base + L > (long long)ph.klen.size())
      return fail(name, "lane range", (long long)t, T.lane_base);
    if (T.row_base < 0 || T.row_base + T.rows > (long long)ph.out.size())
      return fail(name, "out range", (long long)t, T.row_base);
    std::vector<cd> lane_sum(L);
    for (int lane = 0; lane < L; ++lane) {
      const int ql = ph.klen[T.lane_base + lane];
      if (ql < 0 || ql > T.qmax) return fail(name, "lane length", (long long)t, ql);
      const int sl = lane / R;
      cd s(0.0, 0.0);
      for (int q = 0; q < ql; ++q) {
        const int i = ph.idx[T.i_off + (long long)S * q + sl];
        if (i < 0 || i >= (long long)src.size()) return fail(name, "gather index", (long long)t, i);
        read[i] = 1;
        const lsg::cplx a = ph.A[T.a_off + (long long)L * q + lane];
        s += cd(a.re, a.im) * src[i];
      }
      lane_sum[lane] = s;
    }
    for (int r = 0; r < T.rows; ++r) {
      cd v(0.0, 0.0);
      for (int sl = 0; sl < S; ++sl) v += lane_sum[sl * R + r];
      const int o = ph.out[T.row_base + r];
      if (o < 0 || o >= (long long)dst.size()) return fail(name, "output row", (long long)t, o);
      if (written[o]) return fail(name, "output row written twice", (long long)t, o);
      written[o] = 1;
      result.emplace_back(o, v);
    }
  }
  if (in_place)
    for (size_t i = 0; i < dst.size(); ++i)
      if (written[i] && read[i]) return fail(name, "row both read and written", (long long)i, 0);
  for (auto& [o, v] : result) dst[o] = ph.accumulate ? dst[o] + v : v;
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4 && argc != 5) return 2;
  const bool far_only = argc == 5 && std::string(argv[4]) == "--far-only";
  if (argc == 5 && !far_only) return 2;
  ls_config cfg;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  const size_t got = std::fread(&cfg, 1, sizeof(cfg), f);
  const int extra = std::fgetc(f);
  std::fclose(f);
  if (got != sizeof(cfg) || extra != EOF) {
    std::fprintf(stderr, "config: %zu bytes, expected %zu\n", got, sizeof(cfg));
    return 2;
  }
  lsg::HostOperator h;
  std::string err;
  if (!lsg::assemble(cfg, h, err)) {
    std::fprintf(stderr, "assemble: %s\n", err.c_str());
    return 3;
  }
  if (!h.generic_near && !far_only) {
    std::fprintf(stderr, "the operator has no generic near phase\n");
    return 4;
  }
  const int N = h.N;
  std::vector<cd> x(N);
  f = std::fopen(argv[2], "rb");
  if (!f || std::fread(x.data(), sizeof(cd), N, f) != (size_t)N) return 2;
  std::fclose(f);
  std::vector<cd> S(h.charges_len, cd(0.0, 0.0)), P(h.pots_len, cd(0.0, 0.0));
  for (int i = 0; i < N; ++i) S[i] = x[i];
  for (auto& ph : h.up)
    if (!run_phase(ph, S, S, true, "up")) return 4;
  if (!run_phase(h.m2l, S, P, false, "m2l")) return 4;
  for (auto& ph : h.down)
    if (!run_phase(ph, P, P, true, "down")) return 4;
  if (!far_only && !run_phase(h.nearph, S, P, false, "near")) return 4;
  f = std::fopen(argv[3], "wb");
  if (!f || std::fwrite(P.data(), sizeof(cd), N, f) != (size_t)N) return 2;
  std::fclose(f);
  std::printf("N %d charges %lld potentials %lld phases up %zu down %zu\n", N, h.charges_len, h.pots_len,
              h.up.size(), h.down.size());
  return 0;
}
