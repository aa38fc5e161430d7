// Device-side operator state shared by matvec.cu, gmres.cu and capi.cpp.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "ls_internal.h"

namespace lsg {

// One phase of gather-GEMV items resident on the device.
template <class C>
struct DevPhase {
  C* A = nullptr;            // tiles (double2 or float2)
  int* idx = nullptr;        // gather indices, one per tile, step and slice
  int* out = nullptr;        // output element per row
  int* klen = nullptr;       // steps per lane
  GemvTile* tiles = nullptr;
  int n_tiles = 0;
  int accumulate = 0;
  long long entries = 0;     // true block entries (without tile padding)
  long long stored = 0;      // stored elements (with padding)
};

struct GmresWorkspace;  // gmres.cu: Krylov basis and scratch, kept between solves
template <int NR>
struct BatchWorkspace;  // batched.cu: state of the many-right-hand-side solver
struct TcOperator;      // batched_tc.cu: the FP32 operator in tensor-core form

// Right-hand sides handled together by the batched solver (batched.cu):
// 8 with the CUDA-core block apply, 64 with the tensor-core one.
constexpr int kBatchRhs = 8;
constexpr int kTcRhs = 64;

struct DevOperator {
  int device = 0;
  cudaStream_t stream = nullptr;
  int N = 0, n_leaves = 0, rank = 0;
  int find_phi = 1;
  long long charges_len = 0, pots_len = 0;
  // Adaptive trees: the near field as a gather-GEMV phase accumulating into
  // P[0:N), then y = P[0:N) (HostOperator::generic_near).
  bool generic_near = false;
  DevPhase<double2> nearph;
  DevPhase<float2> nearph32;
  DevPhase<float4> nearph_df;
  // FP64 operator
  std::vector<DevPhase<double2>> up, down;
  DevPhase<double2> m2l;
  double2* S = nullptr;      // charges: x then skeleton charges
  double2* P = nullptr;      // potentials: leaves then skeleton potentials
  double2* nearB = nullptr;  // 9 x rank x rank
  double* kq = nullptr;      // kappa^2 q at the grid points
  int* colleague = nullptr;  // n_leaves x 9
  // Factored near field: B_q = Vt_q Q^+ + E_q (E_q: 6-digit rounding residual)
  int n_bases = 0;
  double2* nearVt = nullptr; // [q][l][row]: 9 x n_bases x rank (transposed)
  double* Qp = nullptr;      // n_bases x rank
  float2* nearE = nullptr;   // [q][k][row]: 9 x rank x rank (FP32, transposed)
  double2* cbuf = nullptr;   // n_leaves x n_bases: Q^+ x per leaf
  float2* x32 = nullptr;     // N: x in FP32 for the E_q term
  // The factored near field overlapped with the upward, M2L and downward
  // phases: its contribution goes to Zn on near_stream (the same priority),
  // forked after the load of x and joined before the combine with P.
  cudaStream_t near_stream = nullptr;
  cudaEvent_t near_fork = nullptr, near_join = nullptr;
  double2* Zn = nullptr;     // N: the near-field contribution
  // The matvec on page-locked host buffers as one CUDA graph (ls_matvec_host),
  // captured for one (x, y, kernel family, schedule) and launched as one
  // operation; recaptured when any of them changes.
  cudaGraphExec_t mv_graph = nullptr;
  const void* mv_x = nullptr;
  const void* mv_y = nullptr;
  int mv_key = -1;
  // FP32 operator (mixed precision), built on request
  bool has_f32 = false;
  std::vector<DevPhase<float2>> up32, down32;
  DevPhase<float2> m2l32;
  float2* S32 = nullptr;
  float2* P32 = nullptr;
  float2* nearB32 = nullptr;  // [q][k][row]: 9 x rank x rank (transposed)
  float* kq32 = nullptr;
  float2* Z32 = nullptr;      // near field, pass 1: [leaf][q][row]
  // Double-float form of the FP64 operator (matvec_df.cu), built on request.
  // f64_kernels selects what the FP64 entry points run: LS_F64_NATIVE or
  // LS_F64_DOUBLE_FLOAT.
  int f64_kernels = LS_F64_NATIVE;
  // Element type of the inner Krylov basis of the mixed-precision solvers
  // (LS_INNER_BASIS_F64: FP64 Gram-Schmidt and Givens over the FP32 operator).
  int inner_basis = LS_INNER_BASIS_F64;
  bool has_df = false;
  std::vector<DevPhase<float4>> up_df, down_df;
  DevPhase<float4> m2l_df;
  float4* S_df = nullptr;    // (re_hi, im_hi, re_lo, im_lo)
  float4* P_df = nullptr;
  float4* Vt_df = nullptr;
  float2* Qp_df = nullptr;   // (hi, lo)
  float4* c_df = nullptr;
  float4* Z_df = nullptr;    // near field, pass 1: [leaf][q][row] contribution of a leaf
  float2* ZE_df = nullptr;   // same for the E_q term (FP32)
  // scratch device vectors (N complex) for host-buffer calls
  double2* xbuf = nullptr;
  double2* ybuf = nullptr;
  GmresWorkspace* gws = nullptr;
  BatchWorkspace<kBatchRhs>* bws = nullptr;
  BatchWorkspace<kTcRhs>* bws_tc = nullptr;
  TcOperator* tc = nullptr;
  // Right-hand sides per block of the batched solver: kBatchRhs (CUDA-core
  // block apply) or kTcRhs (tensor-core block apply, built on first use).
  int batch_width = kTcRhs;
  // events for phase timing
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // recorded after the downward phases (before the near field) when phases
  // are marked: [0] FP64 operator, [1] FP32 operator
  cudaEvent_t ev_down[2] = {nullptr, nullptr};
  long long device_bytes = 0;
  int launches_per_matvec = 0;
};

// Capacity of the static scratch array of ls_matvec_noalloc, in complex
// doubles (16 MiB).
constexpr long long kStaticScratchElems = LS_STATIC_SCRATCH_ELEMS;

// matvec.cu
bool dev_upload(const HostOperator& h, DevOperator& d, std::string& err);
void dev_free(DevOperator& d);
bool dev_enable_f32(DevOperator& d, std::string& err);
// y = A x; x, y device pointers (N complex). mark_m2l: record events around M2L.
cudaError_t dev_matvec(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool mark_m2l);
cudaError_t dev_matvec_f32(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool mark_m2l);
// The FP32 operator with FP32 vectors on both sides (inner solves of ls_gmres_mixed).
cudaError_t dev_matvec_f32v(DevOperator& d, const float2* x, float2* y, cudaStream_t s);
// Same product with its scratch in a static device array (no allocation).
cudaError_t dev_matvec_static(DevOperator& d, const double2* x, double2* y, cudaStream_t s);

// matvec_df.cu
bool dev_enable_df(DevOperator& d, std::string& err);
void dev_free_df(DevOperator& d);
cudaError_t dev_matvec_df(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool mark_m2l);

// batched_tc.cu
bool dev_enable_tc(DevOperator& d, const HostOperator& h, std::string& err);
void dev_free_tc(DevOperator& d);
// y = A32 x for kTcRhs right-hand sides stored rhs-minor, on the tensor
// cores; S (charges_len + 1 rows, the last one zero) and P (pots_len rows)
// are the block's work buffers.
cudaError_t dev_matvec_f32_wide(DevOperator& d, const float2* x, float2* y, float2* S, float2* P, cudaStream_t s);
cudaError_t dev_tc_error(DevOperator& d, unsigned* flag);
long long dev_tc_operator_bytes(const DevOperator& d);
long long dev_tc_stages(const DevOperator& d);
bool dev_near_overlap(const DevOperator& d);  // the native matvec overlaps its near field (see ls_set_near_overlap)
cudaError_t dev_tc_wait_probe(int device, long long polls, unsigned* gave_up);  // stages of one tensor-core block apply (0 before it is built)

// batched.cu
void dev_free_batch(DevOperator& d);
// y_j = A32 x_j for the kBatchRhs vectors of a block stored rhs-minor
// (element (i, j) at i * kBatchRhs + j); FP32 operator.
cudaError_t dev_matvec_f32_batch(DevOperator& d, const float2* x, float2* y, cudaStream_t s);
// Mixed-precision refinement for nrhs right-hand sides (device arrays,
// column j at b + j * N), solved kBatchRhs at a time with a shared FP32
// operator apply. n_matvec counts FP32 block applies and FP64 residual
// products; relres gets each column's final FP64 relative residual.
// d.batch_width selects the block width (the tensor-core form must have
// been enabled for kTcRhs).
cudaError_t dev_gmres_mixed_batch(DevOperator& d, int nrhs, const double2* b, double2* x, int max_outer, int inner,
                                  double tol, int& n_matvec, std::vector<double>& relres);
// Same apply on kTcRhs vectors through the block solver's work buffers.
cudaError_t dev_matvec_f32_wide_ws(DevOperator& d, const float2* x, float2* y, cudaStream_t s);
// Y = A32 X for nrhs FP64 columns (column j at j * N), kTcRhs at a time on
// the tensor cores; synchronises the operator's stream.
cudaError_t dev_matvec_f32_many(DevOperator& d, int nrhs, const double2* X, double2* Y);
// Mean ms of one block apply of `width` (kBatchRhs or kTcRhs) resident
// right-hand sides, CUDA events on the operator's stream.
cudaError_t dev_time_block_apply(DevOperator& d, int width, int warmup, int iters, float* ms);

// gmres.cu
void dev_free_gmres(DevOperator& d);
struct GmresResult {
  int iters = 0;
  double rel_residual = 0.0;
  bool converged = false;
};
cudaError_t dev_gmres(DevOperator& d, const double2* b, double2* x, int max_iter, double tol,
                      std::vector<double>& hist, GmresResult& res);
cudaError_t dev_gmres_restarted(DevOperator& d, const double2* b, double2* x, int m, int restarts);
cudaError_t dev_gmres_mixed(DevOperator& d, const double2* b, double2* x, int max_outer, int inner,
                            double tol, std::vector<double>& hist, int& n_matvec, double& relres);

// A right preconditioner z = M(v) on FP32 vectors of the operator's size,
// queued on stream s without waiting on the host. M may be nonlinear
// (flexible GMRES keeps each z).
struct Precond32 {
  virtual ~Precond32() = default;
  virtual cudaError_t apply(const float2* v, float2* z, cudaStream_t s) = 0;
};
struct FlexReport {
  int n_matvec = 0;       // FP32 operator applies + FP64 residual products
  int n_precond = 0;      // applications of M (the initial guess included)
  double guess_residual = 1.0;  // |b - A x0| / |b| of the initial guess (1 without one)
  bool fell_back = false; // M was dropped after an outer step that did not reduce the residual
};
// dev_gmres_mixed with flexible inner GMRES right-preconditioned by M (may be
// null), starting from x0 = guess(b) when guess is given (kept only if it
// beats x0 = 0). The residual is the FP64 one throughout. M is used only in
// outer steps whose inner target is a reduction below 1e-3 (looser ones
// take a few plain steps), and it is turned off for the remaining steps,
// so that the solve ends as plain dev_gmres_mixed would, when an outer step
// (at most 24 preconditioned inner steps) did not halve the residual.
cudaError_t dev_gmres_mixed_flex(DevOperator& d, const double2* b, double2* x, Precond32* M, Precond32* guess,
                                 int max_outer, int inner, double tol, std::vector<double>& hist, FlexReport& rep,
                                 double& relres);

}  // namespace lsg
