// Internal types shared by the host assembler (assemble.cpp), the device
// runtime (matvec.cu, gmres.cu) and the C ABI (capi.cpp).
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ls_dafmm.h"

namespace lsg {

using cd = std::complex<double>;

// One warp-sized unit of a gather-GEMV phase:
//   dst[out_off + r] (=|+=) sum_k A[r, k] * src[idx[idx_off + k]],  r < nr.
// Blocks with K >= kColsThreshold are stored row major (lanes stride over
// K); narrower blocks are stored column major (one lane per row).
struct GemvItem {
  long long a_off;   // element offset of row 0 of this item in A
  int idx_off;       // offset of the gather list in idx
  int K;             // columns
  int nr;            // rows handled by this item
  int out_off;       // output element offset
  int lda;           // row-major: K; column-major: total rows of the block
  int layout;        // 0 = row major (lanes over K), 1 = column major (lane per row)
};

constexpr int kRowsPerItem = 12;   // rows per warp item in the row-major kernel
constexpr int kColsThreshold = 64; // K below this uses the lane-per-row kernel

// A phase (or one tree level of a phase) in device-ready form.
struct GemvPhase {
  std::vector<cd> A;            // concatenated blocks
  std::vector<int> idx;         // gather indices into the source buffer
  std::vector<GemvItem> items;
  int accumulate = 0;           // 0: overwrite, 1: accumulate into dst
  long long entries() const { return (long long)A.size(); }
};

// Host-side intermediate representation of an assembled operator.
struct HostOperator {
  ls_config cfg;
  int N = 0, n_leaves = 0, rank = 0, n_levels = 0, level_LFR = 2, n_bases = 0;
  std::vector<double> px, py, q;     // grid points and contrast
  std::vector<int> colleague;        // n_leaves x 9, -1 = none
  std::vector<cd> nearB;             // 9 x rank x rank, row major
  std::vector<cd> M;                 // rank x 31 (leaf level), row major
  std::vector<double> kq;            // kappa^2 q at the grid points
  long long charges_len = 0;         // x (N) + skeleton charges
  long long pots_len = 0;            // leaf potentials (N) + skeleton potentials
  std::vector<GemvPhase> up;         // M2M, leaves first, then coarser levels
  GemvPhase m2l;                     // all levels in one launch
  long long m2l_rows = 0;            // potential rows written by M2L
  std::vector<GemvPhase> down;       // L2L, coarse to fine
  std::vector<int> skeleton_dump;
  int max_rank = 0;
  double assemble_seconds = 0.0;
};

// assemble.cpp
bool assemble(const ls_config& cfg, HostOperator& op, std::string& err);

// Thread-local last error message used by the C ABI.
void set_error(const std::string& msg);

}  // namespace lsg
