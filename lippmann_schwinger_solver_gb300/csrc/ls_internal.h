// Internal types shared by the host assembler (assemble.cpp), the device
// runtime (matvec.cu, gmres.cu) and the C ABI (capi.cpp).
#pragma once

#include <complex>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/ls_dafmm.h"

namespace lsg {

using cd = std::complex<double>;

// A complex double as two plain doubles, and a vector of them whose
// elements are left uninitialised on resize: the packed operator (hundreds
// of MB) is then first touched by the threads that fill it, in parallel,
// instead of zeroed by one thread (std::complex always zero-initialises).
struct cplx {
  double re, im;
};
template <class T>
struct NoInitAllocator {
  using value_type = T;
  NoInitAllocator() = default;
  template <class U>
  NoInitAllocator(const NoInitAllocator<U>&) noexcept {}
  T* allocate(size_t n) { return std::allocator<T>().allocate(n); }
  void deallocate(T* p, size_t n) noexcept { std::allocator<T>().deallocate(p, n); }
  template <class U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
  template <class U>
  bool operator==(const NoInitAllocator<U>&) const noexcept {
    return true;
  }
  template <class U>
  bool operator!=(const NoInitAllocator<U>&) const noexcept {
    return false;
  }
};
using PackedBlocks = std::vector<cplx, NoInitAllocator<cplx>>;

// One warp tile of a gather-GEMV phase: R = 32 / S rows of one block, each
// split into S interleaved column slices, so lane l = s * R + r sums the
// columns k = q * S + s of row r. Element (q, l) sits at a_off + 32 q + l in
// A: every warp load is one contiguous line. The rows of a tile share their
// gather list, stored once per slice and step: column k = q * S + s of the
// tile gathers src[idx[i_off + q * S + s]]. After the loop the S slice sums
// are combined with shuffles and the lanes of slice 0 write:
//   dst[out[row_base + r]] (=|+=) sum_k A(r, k) * src[idx(k)]
struct GemvTile {
  long long a_off;  // first element of the tile in A
  long long i_off;  // first gather index of the tile in idx
  int qmax;         // steps of the longest lane
  int rows;         // rows in the tile (<= R)
  int log2s;        // S = 1 << log2s column slices per row
  int lane_base;    // offset of the tile's 32 lane lengths in qlen
  int row_base;     // offset of the tile's rows in out
  int pad;
};

constexpr int kTileLanes = 32;

// A phase (or one tree level of a phase) in device-ready form.
struct GemvPhase {
  PackedBlocks A;               // tiles, column interleaved (zero padded)
  std::vector<int> idx;         // gather indices, one per tile, step and slice
  std::vector<int> out;         // output element of each row
  std::vector<int> klen;        // steps of each lane (32 per tile)
  std::vector<GemvTile> tiles;
  int accumulate = 0;           // 0: overwrite, 1: accumulate into dst
  long long nnz = 0;            // true (unpadded) block entries
  // Block structure of the tiles: block b is tiles [blk_tile0[b],
  // blk_tile0[b + 1]) with blk_rows[b] rows and blk_K[b] columns; its rows
  // are consecutive in `out` from the first tile's row_base and its gather
  // list is the first tile's idx range (column k at i_off + k). Read by the
  // tensor-core form of the phase (batched_tc.cu).
  std::vector<int> blk_tile0, blk_rows, blk_K;
  // Staging before packing: the phase owns its blocks (row major) and their
  // gather lists until they are packed; one record per block row points
  // into them.
  // A row staged without values (a == nullptr) is filled from the far-field
  // table: its target point pt against the block's source points cpt[0, K).
  struct Row {
    const cd* a;
    int K;
    const int* idx;
    int out;
    int pt = -1;
    const int* cpt = nullptr;
  };
  std::vector<std::vector<cd>> stageA;
  std::vector<std::vector<int>> stageIdx, stageCols;
  std::vector<Row> rows;
  // The tiles filled on the device (far_on_gpu = 3, M2L): A stays empty on
  // the host and dev_A (dev_A_elems complex doubles, cudaMalloc'd on the
  // operator's device) holds them until the device upload adopts it.
  void* dev_A = nullptr;
  long long dev_A_elems = 0;
  long long entries() const { return nnz; }
};

// Host-side intermediate representation of an assembled operator.
struct HostOperator {
  ls_config cfg;
  int N = 0, n_leaves = 0, rank = 0, n_levels = 0, level_LFR = 2, n_bases = 0;
  std::vector<double> px, py, q;     // grid points and contrast
  std::vector<int> colleague;        // n_leaves x 9, -1 = none
  std::vector<cd> nearB;             // 9 x rank x rank, row major
  std::vector<cd> nearVt;            // 9 x rank x n_bases: B_q = Vt_q Q^+ + E_q
  std::vector<cd> nearE;             // 9 x rank x rank: residual of the 6-digit rounding
  std::vector<double> Qpinv;         // n_bases x rank: Q^+
  std::vector<cd> M;                 // rank x 31 (leaf level), row major
  std::vector<double> kq;            // kappa^2 q at the grid points
  long long charges_len = 0;         // x (N) + skeleton charges
  long long pots_len = 0;            // leaf potentials (N) + skeleton potentials
  std::vector<GemvPhase> up;         // M2M, leaves first, then coarser levels
  GemvPhase m2l;                     // all levels in one launch
  long long m2l_rows = 0;            // potential rows written by M2L
  std::vector<GemvPhase> down;       // L2L, coarse to fine
  // Adaptive trees: the near field as one more accumulating phase into the
  // leaf potentials P[0:N) (diag(kappa^2 q) B of every neighbour, + I on the
  // self block), after which the output is P[0:N). Uniform trees use the
  // factored colleague blocks instead (generic_near false).
  GemvPhase nearph;
  bool generic_near = false;
  std::vector<int> skeleton_dump;
  int max_rank = 0;
  double assemble_seconds = 0.0;
  double stage_seconds[LS_ASSEMBLE_STAGES] = {};  // ls_op_info_t::assemble_stage_seconds
};

// One adaptive quadrature of the assembly's precomputations over [-1,1]^2:
// kind 0 the near-field integral of H0(k |X - p|) T_a(p_x) T_b(p_y) for a
// target X = (xx, xy); kind 1 the far moment of J_n(k |p|) e^{-i n arg p}
// T_a(p_x) T_b(p_y).
struct QuadTask {
  double xx, xy, k;
  int a, b, n, kind;
};
// Integrates the tasks on the GPU `device` with the host's adaptive
// 10 x 10 panel rule (gx, gw: its Gauss-Legendre nodes and weights);
// returns false, out untouched, when that is not possible (no device, or
// a bounded integral that did not finish), and the caller integrates on
// the host. csrc/quadrature.cu; a host-only build (tests/cpp) gets a stub
// that returns false.
bool gpu_quadrature(int device, const std::vector<QuadTask>& tasks, const std::vector<double>& gx,
                    const std::vector<double>& gw, std::vector<cd>& out);

// The far-field entry tables of a uniform tree (the x and y parts of
// p_i - c_leaf take few distinct values): ux / uy the distinct values;
// xid[xrow * ncol + lcol] the index in ux of fl(gx_i - cx_leaf) for a point
// of x row xrow (x node * ncol + x column of its leaf) and a leaf of x
// column lcol; likewise yid. A far-field entry's 31-term sums then sit at
// S[(xid * ny + yid) * rank + node].
struct FarTables {
  int rank = 0, ncol = 0, findPhi = 0;
  double kappa = 0.0;
  std::vector<double> ux, uy;
  std::vector<int> xid, yid;    // (nChebNodes * ncol) x ncol
  std::vector<int> xrow, yrow;  // per point
  std::vector<int> lcol, lrow;  // per leaf
  std::vector<double> kq;       // kappa^2 q per point
  std::vector<cd> M;            // rank x 31, the leaf moments
};
// One tile of a phase filled from the far-field table: A[a_off + 32 q +
// lane] for lane = sl * R + r (R = 32 >> log2s rows, sl < 1 << log2s) is
// K(rowpts[row_off + r], colpts[col_off + q * S + sl]) for r < rows and
// q * S + sl < K, zero elsewhere (the layout of GemvTile).
struct FillTile {
  long long a_off, row_off, col_off;
  int qmax, rows, log2s, K;
};
// One NCA block for the GPU: rows idx[idx_off, +n1), columns
// idx[idx_off + n1, +n2) (point indices); pivots up to R = min(n1, n2, cap):
// rows at piv[out_off, +R), columns at piv[out_off + R, +R).
struct NcaTask {
  long long idx_off;
  int n1, n2, R, out_off;
};
// csrc/far_gpu.cu. gpu_far_open builds the far-field sum table on `device`
// and copies it into S_host (ux.size() * uy.size() * rank elements);
// nullptr when that is not possible. gpu_far_nca runs the NCA of a batch
// of blocks with tolerance eps (status 1 marks a block whose rank reached
// R < min(n1, n2)); false when the batch could not run. gpu_far_close
// frees the device state. A host-only build gets stubs that fail, and the
// host does the work.
struct GpuFar;
GpuFar* gpu_far_open(int device, const FarTables& t, cd* S_host);
bool gpu_far_nca(GpuFar* f, const std::vector<NcaTask>& tasks, const std::vector<int>& idx, double eps,
                 std::vector<int>& ranks, std::vector<int>& piv, std::vector<int>& status);
void gpu_far_close(GpuFar* f);
// Fills `elems` complex doubles of tiles from the table on the device;
// returns the cudaMalloc'd array, or nullptr (the host fills them instead).
void* gpu_far_fill(GpuFar* f, const std::vector<FillTile>& tiles, const std::vector<int>& rowpts,
                   const std::vector<int>& colpts, long long elems);
void gpu_far_free(void* p);

// assemble.cpp. Process-wide cache of precomputation records (far
// moments, near blocks), keyed on every input they depend on: dir nullptr
// turns it off (the default), "" keeps records in memory, a path also
// stores them as binary files there (shared between processes).
void precompute_cache_set(const char* dir);
void precompute_cache_stats(long long& hits, long long& misses);

bool assemble(const ls_config& cfg, HostOperator& op, std::string& err);
// The GPU that the calling thread's assemblies may use for their
// precomputation quadratures and far field (-1: none), set by ls_op_create
// around assemble().
void set_assembly_device(int device);
// The contrast plugin q(x, y) selected by cfg (userkernel::ContrastFunction).
double contrast_at(const ls_config& cfg, double x, double y);

// Thread-local last error message used by the C ABI.
void set_error(const std::string& msg);

}  // namespace lsg
