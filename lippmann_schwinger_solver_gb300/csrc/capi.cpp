// extern "C" entry points of liblsdafmm.so (declared in include/ls_dafmm.h).

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/ls_fno.h"
#include "device.h"
#include "ls_internal.h"
#include "nn_precond.h"

struct ls_op {
  lsg::HostOperator host;
  lsg::DevOperator dev;
  bool on_device = false;  // false: assembled on the host only (device < 0)
  // Network preconditioner of the last ls_fgmres_nn (built for nn_net).
  std::unique_ptr<lsg::NnPrecond> nn;
  const void* nn_net = nullptr;
  // Nodes -> grid sampler of the last ls_op_grid_sample.
  std::unique_ptr<lsg::GridSampler> sampler;
  ~ls_op() {
    if (nn) nn->release();
    if (sampler) sampler->release();
  }
};

struct ls_fno {
  lsg::FnoNet net;
  float* ssq = nullptr;  // per-sample |f|^2 of ls_fno_make_batch
  ~ls_fno() {
    cudaFree(ssq);
    net.release();
  }
};

namespace lsg {
static thread_local std::string t_last_error;
void set_error(const std::string& msg) { t_last_error = msg; }

// Programmatic dependent launch of the kernel chains (launch.h): read from
// LS_PDL on first use (0 turns it off), then set by ls_set_pdl.
static std::atomic<int> g_pdl{-1};
int pdl_enabled() {
  int v = g_pdl.load(std::memory_order_relaxed);
  if (v < 0) {
    const char* e = std::getenv("LS_PDL");
    v = (e && e[0] == '0') ? 0 : 1;
    int expected = -1;
    if (!g_pdl.compare_exchange_strong(expected, v)) v = expected;
  }
  return v;
}
void set_pdl_enabled(int on) { g_pdl.store(on ? 1 : 0); }

cudaError_t raise_smem_limit(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> limit;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  int& cur = limit[{kernel, dev}];
  cur = std::max(cur, bytes);
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, cur);
}

std::atomic<int> g_near_overlap{-1};
int near_overlap_enabled() {
  int v = g_near_overlap.load(std::memory_order_relaxed);
  if (v < 0) {
    const char* e = std::getenv("LS_NEAR_OVERLAP");
    v = (e && e[0] == '0') ? 0 : 1;
    int expected = -1;
    if (!g_near_overlap.compare_exchange_strong(expected, v)) v = expected;
  }
  return v;
}
void set_near_overlap_enabled(int on) { g_near_overlap.store(on ? 1 : 0); }
}  // namespace lsg

using namespace lsg;

namespace {

ls_status fail(ls_status code, const std::string& msg) {
  set_error(msg);
  return code;
}

ls_status cuda_fail(cudaError_t e, const char* where) {
  return fail(LS_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Entry points built on the uniform tree's leaf grid and colleague table.
bool adaptive(const ls_op* op) { return op->host.generic_near; }
ls_status adaptive_refused(const char* who) {
  return fail(LS_E_STATE, std::string(who) + ": not available for operators on adaptive trees");
}

}  // namespace

extern "C" {

ls_status ls_op_create(const ls_config* cfg, int device, ls_op** out) {
  if (!cfg || !out) return fail(LS_E_INVALID, "ls_op_create: null argument");
  *out = nullptr;
  if (device >= 0) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(LS_E_CUDA, "ls_op_create: no CUDA device available");
    if (device >= ndev) return fail(LS_E_INVALID, "ls_op_create: device index out of range");
  }
  ls_op* op = new (std::nothrow) ls_op();
  if (!op) return fail(LS_E_NOMEM, "ls_op_create: out of host memory");
  std::string err;
  set_assembly_device(device);  // the precomputation quadratures may use this GPU
  const bool assembled = assemble(*cfg, op->host, err);
  set_assembly_device(-1);
  if (!assembled) {
    gpu_far_free(op->host.m2l.dev_A);
    delete op;
    return fail(LS_E_INVALID, "ls_op_create: " + err);
  }
  if (device < 0) {  // inspection only: skeletons, precomputations, geometry
    *out = op;
    return LS_OK;
  }
  op->on_device = true;
  op->dev.device = device;
  if (!dev_upload(op->host, op->dev, err)) {
    // Device-filled tiles the upload did not adopt are freed here.
    if (op->host.m2l.dev_A && op->dev.m2l.A != op->host.m2l.dev_A) gpu_far_free(op->host.m2l.dev_A);
    dev_free(op->dev);
    delete op;
    return fail(LS_E_CUDA, "ls_op_create: " + err);
  }
  op->host.m2l.dev_A = nullptr;  // owned by the device operator now
  // Host copies of the tiles are no longer needed.
  auto drop = [](GemvPhase& p) {
    PackedBlocks().swap(p.A);
    std::vector<int>().swap(p.idx);
  };
  for (auto& p : op->host.up) drop(p);
  for (auto& p : op->host.down) drop(p);
  drop(op->host.m2l);
  drop(op->host.nearph);
  *out = op;
  return LS_OK;
}

ls_status ls_op_destroy(ls_op* op) {
  if (!op) return LS_OK;
  if (op->on_device) {
    cudaSetDevice(op->dev.device);
    if (op->nn) op->nn->release();
    if (op->sampler) op->sampler->release();
    dev_free(op->dev);
  }
  delete op;
  return LS_OK;
}

ls_status ls_op_info(const ls_op* op, ls_op_info_t* o) {
  if (!op || !o) return fail(LS_E_INVALID, "ls_op_info: null argument");
  const HostOperator& h = op->host;
  const DevOperator& d = op->dev;
  std::memset(o, 0, sizeof(*o));
  o->N = h.N;
  o->n_leaves = h.n_leaves;
  o->n_levels = h.n_levels;
  o->level_LFR = h.level_LFR;
  o->rank = h.rank;
  long long far = 0;
  if (op->on_device) {
    for (auto& p : d.up) far += p.entries;
    far += d.m2l.entries;
    for (auto& p : d.down) far += p.entries;
  } else {
    for (auto& p : h.up) far += p.entries();
    far += h.m2l.entries();
    for (auto& p : h.down) far += p.entries();
  }
  o->far_entries = far;
  o->near_entries = h.generic_near ? (op->on_device ? d.nearph.entries : h.nearph.entries()) : 9LL * h.rank * h.rank;
  // Algorithmic bytes of one FP64 matvec: every far block once, the shared
  // near blocks once, x read and y written once, every skeleton charge and
  // potential written and read once, kappa^2 q read once.
  const long long sk = (h.charges_len - h.N) + (h.pots_len - h.N);
  o->matvec_bytes = 16LL * far + 16LL * o->near_entries + 16LL * 2 * h.N + 16LL * 2 * sk + 8LL * h.N;
  long long nnz_near = 0;
  if (!h.generic_near)
    for (int t = 0; t < h.n_leaves; ++t)
      for (int q = 0; q < 9; ++q) nnz_near += h.colleague[(size_t)t * 9 + q] >= 0;
  o->matvec_flops = 8LL * far + (h.generic_near ? 8LL * o->near_entries : 8LL * nnz_near * h.rank * h.rank);
  o->device_bytes = d.device_bytes;
  o->assemble_seconds = h.assemble_seconds;
  for (int i = 0; i < LS_ASSEMBLE_STAGES; ++i) o->assemble_stage_seconds[i] = h.stage_seconds[i];
  o->max_rank = h.max_rank;
  // double-float: the near field takes a GEMM and a gather kernel
  o->n_kernels_per_matvec = d.launches_per_matvec + (d.f64_kernels == LS_F64_DOUBLE_FLOAT ? 1 : 0) +
                            (d.f64_kernels == LS_F64_NATIVE && dev_near_overlap(d) ? 1 : 0);
  // M2L: every block once (16 B per complex entry), every source charge of
  // the charge buffer once, every potential it writes once.
  o->m2l_entries = op->on_device ? d.m2l.entries : h.m2l.entries();
  o->m2l_bytes = 16LL * o->m2l_entries + 16LL * h.charges_len + 16LL * h.m2l_rows;
  o->m2l_flops = 8LL * o->m2l_entries;
  return LS_OK;
}

ls_status ls_op_points(const ls_op* op, double* xy) {
  if (!op || !xy) return fail(LS_E_INVALID, "ls_op_points: null argument");
  for (int i = 0; i < op->host.N; ++i) { xy[2 * i] = op->host.px[i]; xy[2 * i + 1] = op->host.py[i]; }
  return LS_OK;
}

ls_status ls_op_contrast(const ls_op* op, double* q) {
  if (!op || !q) return fail(LS_E_INVALID, "ls_op_contrast: null argument");
  std::memcpy(q, op->host.q.data(), sizeof(double) * op->host.N);
  return LS_OK;
}

ls_status ls_op_rhs(const ls_op* op, double* b) {
  if (!op || !b) return fail(LS_E_INVALID, "ls_op_rhs: null argument");
  const HostOperator& h = op->host;
  const double k = h.cfg.kappa;
  for (int i = 0; i < h.N; ++i) {
    const cd inc = std::exp(cd(0.0, 1.0) * k * h.px[i]);
    const cd v = -1.0 * k * k * h.q[i] * inc;
    b[2 * i] = v.real();
    b[2 * i + 1] = v.imag();
  }
  return LS_OK;
}

ls_status ls_op_rhs_angles(const ls_op* op, const double* thetas, int n, double* b) {
  if (!op || !thetas || !b) return fail(LS_E_INVALID, "ls_op_rhs_angles: null argument");
  if (n < 1) return fail(LS_E_INVALID, "ls_op_rhs_angles: n must be >= 1");
  const HostOperator& h = op->host;
  const double k = h.cfg.kappa;
  const long long N = h.N;
#pragma omp parallel for schedule(static)
  for (long long u = 0; u < N * n; ++u) {
    const int t = (int)(u / N);
    const long long i = u - (long long)t * N;
    const double phase = h.px[i] * std::cos(thetas[t]) + h.py[i] * std::sin(thetas[t]);
    const cd inc = std::exp(cd(0.0, k * phase));
    const cd v = -1.0 * k * k * h.q[i] * inc;
    b[2 * u] = v.real();
    b[2 * u + 1] = v.imag();
  }
  return LS_OK;
}

ls_status ls_matvec(ls_op* op, const double* x, double* y, void* stream) {
  if (!op || !x || !y) return fail(LS_E_INVALID, "ls_matvec: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_matvec: operator was assembled without a device");
  cudaError_t e = dev_matvec(op->dev, (const double2*)x, (double2*)y, (cudaStream_t)stream, false);
  if (e != cudaSuccess) return cuda_fail(e, "ls_matvec");
  return LS_OK;
}

ls_status ls_op_enable_f32(ls_op* op) {
  if (!op) return fail(LS_E_INVALID, "ls_op_enable_f32: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_op_enable_f32: operator was assembled without a device");
  std::string err;
  if (!dev_enable_f32(op->dev, err)) return fail(LS_E_CUDA, "ls_op_enable_f32: " + err);
  return LS_OK;
}

ls_status ls_op_set_f64_kernels(ls_op* op, int kernels) {
  if (!op) return fail(LS_E_INVALID, "ls_op_set_f64_kernels: null argument");
  if (kernels != LS_F64_NATIVE && kernels != LS_F64_DOUBLE_FLOAT)
    return fail(LS_E_INVALID, "ls_op_set_f64_kernels: unknown kernel choice " + std::to_string(kernels));
  if (!op->on_device) return fail(LS_E_STATE, "ls_op_set_f64_kernels: operator was assembled without a device");
  if (kernels == LS_F64_DOUBLE_FLOAT) {
    std::string err;
    if (!dev_enable_df(op->dev, err)) return fail(LS_E_CUDA, "ls_op_set_f64_kernels: " + err);
  }
  op->dev.f64_kernels = kernels;
  return LS_OK;
}

ls_status ls_op_set_inner_basis(ls_op* op, int basis) {
  if (!op) return fail(LS_E_INVALID, "ls_op_set_inner_basis: null argument");
  if (basis != LS_INNER_BASIS_F64 && basis != LS_INNER_BASIS_F32)
    return fail(LS_E_INVALID, "ls_op_set_inner_basis: unknown basis " + std::to_string(basis));
  if (!op->on_device) return fail(LS_E_STATE, "ls_op_set_inner_basis: operator was assembled without a device");
  op->dev.inner_basis = basis;
  return LS_OK;
}

ls_status ls_matvec_f32(ls_op* op, const double* x, double* y, void* stream) {
  if (!op || !x || !y) return fail(LS_E_INVALID, "ls_matvec_f32: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_matvec_f32: operator was assembled without a device");
  if (!op->dev.has_f32) return fail(LS_E_STATE, "ls_matvec_f32: call ls_op_enable_f32 first");
  cudaError_t e = dev_matvec_f32(op->dev, (const double2*)x, (double2*)y, (cudaStream_t)stream, false);
  if (e != cudaSuccess) return cuda_fail(e, "ls_matvec_f32");
  return LS_OK;
}

ls_status ls_matvec_noalloc(ls_op* op, const double* x, double* y, void* stream) {
  if (!op || !x || !y) return fail(LS_E_INVALID, "ls_matvec_noalloc: null argument");
  if (adaptive(op)) return adaptive_refused("ls_matvec_noalloc");
  const long long need = op->host.charges_len + op->host.pots_len;
  if (need > LS_STATIC_SCRATCH_ELEMS)
    return fail(LS_E_INVALID, "ls_matvec_noalloc: operator needs " + std::to_string(need) +
                                  " complex scratch entries, the static array holds " +
                                  std::to_string((long long)LS_STATIC_SCRATCH_ELEMS));
  if (!op->on_device) return fail(LS_E_STATE, "ls_matvec_noalloc: operator was assembled without a device");
  cudaError_t e = dev_matvec_static(op->dev, (const double2*)x, (double2*)y, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "ls_matvec_noalloc");
  return LS_OK;
}

// Device address of a page-locked host buffer (cudaMallocHost,
// cudaHostRegister, torch pin_memory), or nullptr for any other pointer.
static void* pinned_device_address(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

ls_status ls_matvec_host(ls_op* op, const double* x, double* y) {
  if (!op || !x || !y) return fail(LS_E_INVALID, "ls_matvec_host: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_matvec_host: operator was assembled without a device");
  DevOperator& d = op->dev;
  cudaSetDevice(d.device);
  // Page-locked buffers: the matvec's first kernel reads x from host memory
  // and its output kernel writes y there, so the transfers overlap the
  // kernels instead of running as separate copies.
  void* xd = pinned_device_address(x);
  void* yd = xd ? pinned_device_address(y) : nullptr;
  if (xd && yd && xd != yd) {
    // One call is synchronous, so the host's enqueueing of the matvec's
    // launches and events would sit on its path: the sequence is captured
    // once into a CUDA graph (programmatic launches and the near-field
    // fork/join become its edges) and launched as one operation.
    const int key = d.f64_kernels * 4 + near_overlap_enabled() * 2 + pdl_enabled();
    if (!(d.mv_graph && d.mv_x == xd && d.mv_y == yd && d.mv_key == key)) {
      if (d.mv_graph) cudaGraphExecDestroy(d.mv_graph);
      d.mv_graph = nullptr;
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        const cudaError_t em = dev_matvec(d, (const double2*)xd, (double2*)yd, d.stream, false);
        e = cudaStreamEndCapture(d.stream, &g);
        if (e == cudaSuccess) e = em;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&d.mv_graph, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {  // not capturable here: launch the sequence directly
        if (d.mv_graph) cudaGraphExecDestroy(d.mv_graph);
        d.mv_graph = nullptr;
        cudaGetLastError();
        e = dev_matvec(d, (const double2*)xd, (double2*)yd, d.stream, false);
        if (e != cudaSuccess) return cuda_fail(e, "ls_matvec_host");
        if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return cuda_fail(e, "ls_matvec_host sync");
        return LS_OK;
      }
      d.mv_x = xd;
      d.mv_y = yd;
      d.mv_key = key;
    }
    cudaError_t e = cudaGraphLaunch(d.mv_graph, d.stream);
    if (e != cudaSuccess) return cuda_fail(e, "ls_matvec_host");
    if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return cuda_fail(e, "ls_matvec_host sync");
    return LS_OK;
  }
  const size_t bytes = (size_t)d.N * sizeof(double2);
  cudaError_t e = cudaMemcpyAsync(d.xbuf, x, bytes, cudaMemcpyHostToDevice, d.stream);
  if (e != cudaSuccess) return cuda_fail(e, "ls_matvec_host H2D");
  if ((e = dev_matvec(d, d.xbuf, d.ybuf, d.stream, false)) != cudaSuccess) return cuda_fail(e, "ls_matvec_host");
  if ((e = cudaMemcpyAsync(y, d.ybuf, bytes, cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess)
    return cuda_fail(e, "ls_matvec_host D2H");
  if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return cuda_fail(e, "ls_matvec_host sync");
  return LS_OK;
}

ls_status ls_gmres(ls_op* op, const double* b, int max_iter, double tol, double* x, double* history, int* n_iter,
                   double* rel_residual) {
  if (!op || !b || !x) return fail(LS_E_INVALID, "ls_gmres: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_gmres: operator was assembled without a device");
  if (max_iter < 1) return fail(LS_E_INVALID, "ls_gmres: max_iter must be >= 1");
  DevOperator& d = op->dev;
  cudaSetDevice(d.device);
  const size_t bytes = (size_t)d.N * sizeof(double2);
  cudaError_t e = cudaMemcpyAsync(d.xbuf, b, bytes, cudaMemcpyHostToDevice, d.stream);
  if (e != cudaSuccess) return cuda_fail(e, "ls_gmres H2D");
  std::vector<double> hist;
  GmresResult res;
  if ((e = dev_gmres(d, d.xbuf, d.ybuf, max_iter, tol, hist, res)) != cudaSuccess)
    return cuda_fail(e, "ls_gmres");
  if ((e = cudaMemcpyAsync(x, d.ybuf, bytes, cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess)
    return cuda_fail(e, "ls_gmres D2H");
  if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return cuda_fail(e, "ls_gmres sync");
  if (history) for (size_t i = 0; i < hist.size() && i <= (size_t)max_iter; ++i) history[i] = hist[i];
  if (n_iter) *n_iter = res.iters;
  if (rel_residual) *rel_residual = res.rel_residual;
  if (!res.converged) return fail(LS_E_NOT_CONVERGED, "ls_gmres: tolerance not reached within max_iter");
  return LS_OK;
}

ls_status ls_gmres_restarted(ls_op* op, const double* b, int m, int restarts, double* x) {
  if (!op || !b || !x) return fail(LS_E_INVALID, "ls_gmres_restarted: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_gmres_restarted: operator was assembled without a device");
  if (m < 1 || restarts < 1) return fail(LS_E_INVALID, "ls_gmres_restarted: m and restarts must be >= 1");
  DevOperator& d = op->dev;
  cudaSetDevice(d.device);
  const size_t bytes = (size_t)d.N * sizeof(double2);
  cudaError_t e = cudaMemcpyAsync(d.xbuf, b, bytes, cudaMemcpyHostToDevice, d.stream);
  if (e != cudaSuccess) return cuda_fail(e, "ls_gmres_restarted H2D");
  if ((e = dev_gmres_restarted(d, d.xbuf, d.ybuf, m, restarts)) != cudaSuccess) return cuda_fail(e, "ls_gmres_restarted");
  if ((e = cudaMemcpyAsync(x, d.ybuf, bytes, cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess)
    return cuda_fail(e, "ls_gmres_restarted D2H");
  if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return cuda_fail(e, "ls_gmres_restarted sync");
  return LS_OK;
}

ls_status ls_gmres_mixed(ls_op* op, const double* b, int max_outer, int inner_iter, double tol, double* x,
                         double* history, int* n_matvec, double* rel_residual) {
  if (!op || !b || !x) return fail(LS_E_INVALID, "ls_gmres_mixed: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_gmres_mixed: operator was assembled without a device");
  if (max_outer < 1 || inner_iter < 1) return fail(LS_E_INVALID, "ls_gmres_mixed: iteration counts must be >= 1");
  if (!op->dev.has_f32) return fail(LS_E_STATE, "ls_gmres_mixed: call ls_op_enable_f32 first");
  DevOperator& d = op->dev;
  cudaSetDevice(d.device);
  const size_t bytes = (size_t)d.N * sizeof(double2);
  cudaError_t e = cudaMemcpyAsync(d.xbuf, b, bytes, cudaMemcpyHostToDevice, d.stream);
  if (e != cudaSuccess) return cuda_fail(e, "ls_gmres_mixed H2D");
  std::vector<double> hist;
  int nmv = 0;
  double rr = 1.0;
  if ((e = dev_gmres_mixed(d, d.xbuf, d.ybuf, max_outer, inner_iter, tol, hist, nmv, rr)) != cudaSuccess)
    return cuda_fail(e, "ls_gmres_mixed");
  if ((e = cudaMemcpyAsync(x, d.ybuf, bytes, cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess)
    return cuda_fail(e, "ls_gmres_mixed D2H");
  if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return cuda_fail(e, "ls_gmres_mixed sync");
  if (history) for (size_t i = 0; i < hist.size() && i <= (size_t)max_outer; ++i) history[i] = hist[i];
  if (n_matvec) *n_matvec = nmv;
  if (rel_residual) *rel_residual = rr;
  if (rr > tol) return fail(LS_E_NOT_CONVERGED, "ls_gmres_mixed: tolerance not reached");
  return LS_OK;
}

ls_status ls_op_set_batch_width(ls_op* op, int width) {
  if (!op) return fail(LS_E_INVALID, "ls_op_set_batch_width: null argument");
  if (width != 8 && width != 64)
    return fail(LS_E_INVALID, "ls_op_set_batch_width: width must be 8 or 64, not " + std::to_string(width));
  if (!op->on_device) return fail(LS_E_STATE, "ls_op_set_batch_width: operator was assembled without a device");
  op->dev.batch_width = width;
  return LS_OK;
}

namespace {
// Builds the tensor-core form of the FP32 operator on first use.
ls_status ensure_tc(ls_op* op, const char* who) {
  DevOperator& d = op->dev;
  if (d.tc) return LS_OK;
  std::string err;
  if (!dev_enable_tc(d, op->host, err)) return fail(LS_E_CUDA, std::string(who) + ": " + err);
  d.device_bytes += dev_tc_operator_bytes(d);
  return LS_OK;
}
ls_status tc_status(ls_op* op, const char* who) {
  unsigned flag = 0;
  cudaError_t e = dev_tc_error(op->dev, &flag);
  if (e != cudaSuccess) return cuda_fail(e, who);
  if (flag) return fail(LS_E_TIMEOUT, std::string(who) + ": a tensor-core pipeline wait gave up");
  return LS_OK;
}
}  // namespace

ls_status ls_matvec_f32_many(ls_op* op, int nrhs, const double* X, double* Y) {
  if (!op || !X || !Y || nrhs < 1) return fail(LS_E_INVALID, "ls_matvec_f32_many: bad argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_matvec_f32_many: operator was assembled without a device");
  if (!op->dev.has_f32) return fail(LS_E_STATE, "ls_matvec_f32_many: call ls_op_enable_f32 first");
  DevOperator& d = op->dev;
  cudaSetDevice(d.device);
  ls_status st = ensure_tc(op, "ls_matvec_f32_many");
  if (st != LS_OK) return st;
  const size_t bytes = (size_t)d.N * nrhs * sizeof(double2);
  double2 *dx = nullptr, *dy = nullptr;
  cudaError_t e = cudaMalloc(&dx, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&dy, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(dx, X, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = dev_matvec_f32_many(d, nrhs, dx, dy);
  if (e == cudaSuccess) e = cudaMemcpy(Y, dy, bytes, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  if (e != cudaSuccess) return cuda_fail(e, "ls_matvec_f32_many");
  return tc_status(op, "ls_matvec_f32_many");
}

ls_status ls_time_block_apply(ls_op* op, int width, int warmup, int iters, float* ms) {
  if (!op || !ms || iters < 1 || warmup < 0 || (width != 8 && width != 64))
    return fail(LS_E_INVALID, "ls_time_block_apply: bad argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_time_block_apply: operator was assembled without a device");
  if (!op->dev.has_f32) return fail(LS_E_STATE, "ls_time_block_apply: call ls_op_enable_f32 first");
  cudaSetDevice(op->dev.device);
  if (width == 64) {
    ls_status st = ensure_tc(op, "ls_time_block_apply");
    if (st != LS_OK) return st;
  }
  cudaError_t e = dev_time_block_apply(op->dev, width, warmup, iters, ms);
  if (e != cudaSuccess) return cuda_fail(e, "ls_time_block_apply");
  return width == 64 ? tc_status(op, "ls_time_block_apply") : LS_OK;
}

ls_status ls_tc_wait_probe(int device, long long polls, int* gave_up) {
  if (!gave_up || polls < 1 || polls > 100000000LL) return fail(LS_E_INVALID, "ls_tc_wait_probe: bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return fail(LS_E_CUDA, "ls_tc_wait_probe: no such CUDA device");
  unsigned flag = 0;
  const cudaError_t e = dev_tc_wait_probe(device, polls, &flag);
  if (e != cudaSuccess) return cuda_fail(e, "ls_tc_wait_probe");
  *gave_up = flag ? 1 : 0;
  return LS_OK;
}

ls_status ls_op_tc_stages(const ls_op* op, long long* stages) {
  if (!op || !stages) return fail(LS_E_INVALID, "ls_op_tc_stages: null argument");
  *stages = op->on_device ? dev_tc_stages(op->dev) : 0;
  return LS_OK;
}

ls_status ls_gmres_mixed_batched(ls_op* op, int nrhs, const double* B, int max_outer, int inner_iter, double tol,
                                 double* X, int* n_matvec, double* rel_residuals) {
  if (!op || !B || !X) return fail(LS_E_INVALID, "ls_gmres_mixed_batched: null argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_gmres_mixed_batched: operator was assembled without a device");
  if (nrhs < 1 || max_outer < 1 || inner_iter < 1)
    return fail(LS_E_INVALID, "ls_gmres_mixed_batched: nrhs and iteration counts must be >= 1");
  if (!op->dev.has_f32) return fail(LS_E_STATE, "ls_gmres_mixed_batched: call ls_op_enable_f32 first");
  DevOperator& d = op->dev;
  cudaSetDevice(d.device);
  if (d.batch_width == 64) {
    ls_status st = ensure_tc(op, "ls_gmres_mixed_batched");
    if (st != LS_OK) return st;
  }
  const size_t bytes = (size_t)d.N * nrhs * sizeof(double2);
  double2 *db = nullptr, *dx = nullptr;
  cudaError_t e = cudaMalloc(&db, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&dx, bytes);
  if (e != cudaSuccess) {
    cudaFree(db);
    return cuda_fail(e, "ls_gmres_mixed_batched alloc");
  }
  std::vector<double> rr;
  int nmv = 0;
  if ((e = cudaMemcpyAsync(db, B, bytes, cudaMemcpyHostToDevice, d.stream)) == cudaSuccess)
    e = dev_gmres_mixed_batch(d, nrhs, db, dx, max_outer, inner_iter, tol, nmv, rr);
  if (e == cudaSuccess) e = cudaMemcpyAsync(X, dx, bytes, cudaMemcpyDeviceToHost, d.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d.stream);
  cudaFree(db);
  cudaFree(dx);
  if (e != cudaSuccess) return cuda_fail(e, "ls_gmres_mixed_batched");
  if (d.tc) {
    ls_status st = tc_status(op, "ls_gmres_mixed_batched");
    if (st != LS_OK) return st;
  }
  if (n_matvec) *n_matvec = nmv;
  bool ok = true;
  for (int j = 0; j < nrhs; ++j) {
    if (rel_residuals) rel_residuals[j] = rr[j];
    ok = ok && rr[j] <= tol;
  }
  if (!ok) return fail(LS_E_NOT_CONVERGED, "ls_gmres_mixed_batched: a column did not reach the tolerance");
  return LS_OK;
}

ls_status ls_time_matvec(ls_op* op, int precision, int warmup, int iters, float* ms_matvec, float* ms_m2l) {
  if (!op || iters < 1 || warmup < 0) return fail(LS_E_INVALID, "ls_time_matvec: bad argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_time_matvec: operator was assembled without a device");
  DevOperator& d = op->dev;
  if (precision == LS_PREC_F32 && !d.has_f32) return fail(LS_E_STATE, "ls_time_matvec: FP32 operator not enabled");
  cudaSetDevice(d.device);
  const bool f32 = precision == LS_PREC_F32;
  cudaError_t e;
  for (int i = 0; i < warmup; ++i) {
    e = f32 ? dev_matvec_f32(d, d.xbuf, d.ybuf, d.stream, false) : dev_matvec(d, d.xbuf, d.ybuf, d.stream, false);
    if (e != cudaSuccess) return cuda_fail(e, "ls_time_matvec warmup");
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return cuda_fail(e, "ls_time_matvec sync");
  float m2l_total = 0.0f;
  float total = 0.0f;
  for (int i = 0; i < iters; ++i) {
    cudaEventRecord(a, d.stream);
    e = f32 ? dev_matvec_f32(d, d.xbuf, d.ybuf, d.stream, true) : dev_matvec(d, d.xbuf, d.ybuf, d.stream, true);
    if (e != cudaSuccess) return cuda_fail(e, "ls_time_matvec");
    cudaEventRecord(b, d.stream);
    if ((e = cudaEventSynchronize(b)) != cudaSuccess) return cuda_fail(e, "ls_time_matvec event");
    float t = 0.0f, tm = 0.0f;
    cudaEventElapsedTime(&t, a, b);
    cudaEventElapsedTime(&tm, f32 ? d.ev[2] : d.ev[0], f32 ? d.ev[3] : d.ev[1]);
    total += t;
    m2l_total += tm;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (ms_matvec) *ms_matvec = total / iters;
  if (ms_m2l) *ms_m2l = m2l_total / iters;
  return LS_OK;
}

ls_status ls_time_matvec_phases(ls_op* op, int precision, int warmup, int iters, float* ms) {
  if (!op || iters < 1 || warmup < 0 || !ms) return fail(LS_E_INVALID, "ls_time_matvec_phases: bad argument");
  if (!op->on_device) return fail(LS_E_STATE, "ls_time_matvec_phases: operator was assembled without a device");
  DevOperator& d = op->dev;
  if (precision == LS_PREC_F32 && !d.has_f32)
    return fail(LS_E_STATE, "ls_time_matvec_phases: FP32 operator not enabled");
  cudaSetDevice(d.device);
  const bool f32 = precision == LS_PREC_F32;
  cudaError_t e;
  for (int i = 0; i < warmup; ++i) {
    e = f32 ? dev_matvec_f32(d, d.xbuf, d.ybuf, d.stream, false) : dev_matvec(d, d.xbuf, d.ybuf, d.stream, false);
    if (e != cudaSuccess) return cuda_fail(e, "ls_time_matvec_phases warmup");
  }
  cudaEvent_t a, b;
  if ((e = cudaEventCreate(&a)) != cudaSuccess) return cuda_fail(e, "ls_time_matvec_phases event");
  if ((e = cudaEventCreate(&b)) != cudaSuccess) {
    cudaEventDestroy(a);
    return cuda_fail(e, "ls_time_matvec_phases event");
  }
  double acc[5] = {0, 0, 0, 0, 0};
  const cudaEvent_t m0 = f32 ? d.ev[2] : d.ev[0], m1 = f32 ? d.ev[3] : d.ev[1], m2 = d.ev_down[f32 ? 1 : 0];
  for (int i = 0; i < iters && e == cudaSuccess; ++i) {
    cudaEventRecord(a, d.stream);
    e = f32 ? dev_matvec_f32(d, d.xbuf, d.ybuf, d.stream, true) : dev_matvec(d, d.xbuf, d.ybuf, d.stream, true);
    if (e != cudaSuccess) break;
    cudaEventRecord(b, d.stream);
    if ((e = cudaEventSynchronize(b)) != cudaSuccess) break;
    float t[5] = {0, 0, 0, 0, 0};
    cudaEventElapsedTime(&t[0], a, b);
    cudaEventElapsedTime(&t[1], a, m0);
    cudaEventElapsedTime(&t[2], m0, m1);
    cudaEventElapsedTime(&t[3], m1, m2);
    cudaEventElapsedTime(&t[4], m2, b);
    for (int k = 0; k < 5; ++k) acc[k] += t[k];
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return cuda_fail(e, "ls_time_matvec_phases");
  for (int k = 0; k < 5; ++k) ms[k] = (float)(acc[k] / iters);
  return LS_OK;
}

long ls_op_skeleton_dump(const ls_op* op, int* buf, long cap) {
  if (!op) return -1;
  const auto& v = op->host.skeleton_dump;
  if (buf) {
    const long n = std::min<long>(cap, (long)v.size());
    std::memcpy(buf, v.data(), sizeof(int) * n);
  }
  return (long)v.size();
}

ls_status ls_op_precomputations(const ls_op* op, double* M, double* near) {
  if (!op) return fail(LS_E_INVALID, "ls_op_precomputations: null argument");
  if (adaptive(op)) return adaptive_refused("ls_op_precomputations");
  if (M) std::memcpy(M, op->host.M.data(), op->host.M.size() * sizeof(cd));
  if (near) std::memcpy(near, op->host.nearB.data(), op->host.nearB.size() * sizeof(cd));
  return LS_OK;
}

ls_status ls_op_interpolate(const ls_op* op, int npts, const double* xy, const double* phi, double* psi) {
  if (!op || npts < 0 || (npts > 0 && (!xy || !phi || !psi)))
    return fail(LS_E_INVALID, "ls_op_interpolate: bad argument");
  if (adaptive(op)) return adaptive_refused("ls_op_interpolate");
  const HostOperator& h = op->host;
  const double L = h.cfg.L;
  for (int i = 0; i < npts; ++i)
    if (!(std::fabs(xy[2 * i]) <= L && std::fabs(xy[2 * i + 1]) <= L))
      return fail(LS_E_INVALID, "ls_op_interpolate: point " + std::to_string(i) + " outside [-L, L]^2");
  const LeafInterpolator li(h);
  const cd* ph = reinterpret_cast<const cd*>(phi);
  std::vector<double> w(h.rank);
  for (int i = 0; i < npts; ++i) {
    const int t = li.row(xy[2 * i], xy[2 * i + 1], w.data());
    cd s(0.0, 0.0);
    for (int r = 0; r < h.rank; ++r) s += w[r] * ph[(size_t)t * h.rank + r];
    psi[2 * i] = s.real();
    psi[2 * i + 1] = s.imag();
  }
  return LS_OK;
}

ls_status ls_write_result(const char* path, int n, const double* v) {
  if (!path || n < 0 || (n > 0 && !v)) return fail(LS_E_INVALID, "ls_write_result: bad argument");
  std::ofstream f(path);
  if (!f) return fail(LS_E_INVALID, std::string("ls_write_result: cannot open ") + path);
  for (int i = 0; i < n; ++i) f << cd(v[2 * i], v[2 * i + 1]) << '\n';
  f.close();
  if (!f) return fail(LS_E_INVALID, std::string("ls_write_result: write to ") + path + " failed");
  return LS_OK;
}

// ------------------------------------------------------------------ learned preconditioner (ls_fno.h)

ls_status ls_fno_create(const ls_fno_config* cfg, int device, unsigned long long seed, ls_fno** out) {
  if (!cfg || !out) return fail(LS_E_INVALID, "ls_fno_create: null argument");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(LS_E_CUDA, "ls_fno_create: no CUDA device available");
  if (device < 0 || device >= ndev) return fail(LS_E_INVALID, "ls_fno_create: device index out of range");
  ls_fno* f = new (std::nothrow) ls_fno();
  if (!f) return fail(LS_E_NOMEM, "ls_fno_create: out of host memory");
  FnoShape sh;
  sh.grid = cfg->grid;
  sh.modes = cfg->modes;
  sh.layers = cfg->layers;
  sh.proj = cfg->proj_width;
  std::string err;
  if (!f->net.init(device, sh, seed, err)) {
    delete f;
    return fail(err.rfind("device", 0) == 0 ? LS_E_CUDA : LS_E_INVALID, "ls_fno_create: " + err);
  }
  if ((e = cudaMalloc(&f->ssq, kFnoMaxBatch * sizeof(float))) != cudaSuccess) {
    delete f;
    return cuda_fail(e, "ls_fno_create");
  }
  *out = f;
  return LS_OK;
}

ls_status ls_fno_destroy(ls_fno* net) {
  if (!net) return LS_OK;
  cudaSetDevice(net->net.device);
  delete net;
  return LS_OK;
}

ls_status ls_fno_num_params(const ls_fno* net, long long* n) {
  if (!net || !n) return fail(LS_E_INVALID, "ls_fno_num_params: null argument");
  *n = net->net.lay.total;
  return LS_OK;
}

namespace {
ls_status fno_copy(const ls_fno* net, float* host, const float* dev_src, float* dev_dst, const float* host_src,
                   const char* where) {
  if (!net || !(host || host_src)) return fail(LS_E_INVALID, std::string(where) + ": null argument");
  cudaSetDevice(net->net.device);
  const size_t bytes = (size_t)net->net.lay.total * sizeof(float);
  cudaError_t e = cudaDeviceSynchronize();  // the net's kernels may be on any stream
  if (e == cudaSuccess) e = dev_dst ? cudaMemcpy(dev_dst, host_src, bytes, cudaMemcpyHostToDevice)
                                    : cudaMemcpy(host, dev_src, bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, where);
  return LS_OK;
}
cudaStream_t fno_stream(const ls_fno*, void* stream) { return static_cast<cudaStream_t>(stream); }
}  // namespace

ls_status ls_fno_get_params(const ls_fno* net, float* host) {
  return fno_copy(net, host, net ? net->net.params : nullptr, nullptr, nullptr, "ls_fno_get_params");
}
ls_status ls_fno_set_params(ls_fno* net, const float* host) {
  if (!net || !host) return fail(LS_E_INVALID, "ls_fno_set_params: null argument");
  return fno_copy(net, nullptr, nullptr, net->net.params, host, "ls_fno_set_params");
}
ls_status ls_fno_get_grads(const ls_fno* net, float* host) {
  return fno_copy(net, host, net ? net->net.grads : nullptr, nullptr, nullptr, "ls_fno_get_grads");
}

ls_status ls_fno_forward(ls_fno* net, int batch, const float* in, float* out, void* stream) {
  if (!net || !in || !out) return fail(LS_E_INVALID, "ls_fno_forward: null argument");
  if (batch < 1 || batch > kFnoMaxBatch) return fail(LS_E_INVALID, "ls_fno_forward: batch out of range");
  cudaSetDevice(net->net.device);
  cudaError_t e = net->net.forward(batch, in, out, nullptr, fno_stream(net, stream));
  if (e != cudaSuccess) return cuda_fail(e, "ls_fno_forward");
  return LS_OK;
}

ls_status ls_fno_loss_grad(ls_fno* net, int batch, const float* in, const float* target, float* loss, void* stream) {
  if (!net || !in || !target) return fail(LS_E_INVALID, "ls_fno_loss_grad: null argument");
  if (batch < 1 || batch > kFnoMaxBatch) return fail(LS_E_INVALID, "ls_fno_loss_grad: batch out of range");
  cudaSetDevice(net->net.device);
  cudaStream_t s = fno_stream(net, stream);
  cudaError_t e = net->net.loss_grad(batch, in, target, s);
  if (e == cudaSuccess && loss) {
    e = cudaMemcpyAsync(loss, net->net.loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "ls_fno_loss_grad");
  return LS_OK;
}

ls_status ls_fno_adam_step(ls_fno* net, float lr, float beta1, float beta2, float eps, void* stream) {
  if (!net) return fail(LS_E_INVALID, "ls_fno_adam_step: null argument");
  if (!(lr > 0.f) || !(beta1 >= 0.f && beta1 < 1.f) || !(beta2 >= 0.f && beta2 < 1.f) || !(eps > 0.f))
    return fail(LS_E_INVALID, "ls_fno_adam_step: bad hyper-parameters");
  cudaSetDevice(net->net.device);
  cudaError_t e = net->net.adam(lr, beta1, beta2, eps, fno_stream(net, stream));
  if (e != cudaSuccess) return cuda_fail(e, "ls_fno_adam_step");
  return LS_OK;
}

ls_status ls_fno_make_batch(ls_fno* net, int batch, int n_basis, int n_scatterers, const float* F, const float* PHI,
                            const float* Q, const float* kappa, const int* scatterer, const float* coef, float* in,
                            float* target, void* stream) {
  if (!net || !F || !PHI || !Q || !kappa || !scatterer || !coef || !in || !target)
    return fail(LS_E_INVALID, "ls_fno_make_batch: null argument");
  if (batch < 1 || batch > kFnoMaxBatch || n_basis < 1 || n_basis > 64 || n_scatterers < 1)
    return fail(LS_E_INVALID, "ls_fno_make_batch: batch must be in [1, 64], n_basis in [1, 64], n_scatterers >= 1");
  cudaSetDevice(net->net.device);
  cudaError_t e = fno_make_batch(net->net.shape.grid, batch, n_basis, n_scatterers, reinterpret_cast<const float2*>(F),
                                 reinterpret_cast<const float2*>(PHI), Q, kappa, scatterer,
                                 reinterpret_cast<const float2*>(coef), in, target, net->ssq, fno_stream(net, stream));
  if (e != cudaSuccess) return cuda_fail(e, "ls_fno_make_batch");
  return LS_OK;
}

namespace {
bool valid_grid(int g) { return g >= 8 && g <= 1024 && (g & (g - 1)) == 0; }
}  // namespace

ls_status ls_op_grid_weights(const ls_op* op, int grid, float* w, int* leaf) {
  if (!op || !w || !leaf) return fail(LS_E_INVALID, "ls_op_grid_weights: null argument");
  if (adaptive(op)) return adaptive_refused("ls_op_grid_weights");
  if (!valid_grid(grid)) return fail(LS_E_INVALID, "ls_op_grid_weights: grid must be a power of two in [8, 1024]");
  std::vector<float> hw;
  std::vector<int> hl;
  grid_sampling_weights(op->host, grid, hw, hl);
  std::memcpy(w, hw.data(), hw.size() * sizeof(float));
  std::memcpy(leaf, hl.data(), hl.size() * sizeof(int));
  return LS_OK;
}

ls_status ls_op_grid_contrast(const ls_op* op, int grid, float* q) {
  if (!op || !q) return fail(LS_E_INVALID, "ls_op_grid_contrast: null argument");
  if (adaptive(op)) return adaptive_refused("ls_op_grid_contrast");
  if (!valid_grid(grid)) return fail(LS_E_INVALID, "ls_op_grid_contrast: grid must be a power of two in [8, 1024]");
  std::vector<float> hq;
  grid_contrast(op->host.cfg, grid, hq);
  std::memcpy(q, hq.data(), hq.size() * sizeof(float));
  return LS_OK;
}

ls_status ls_op_grid_sample(ls_op* op, int grid, int nvec, const double* x, float* out, void* stream) {
  if (!op || !x || !out) return fail(LS_E_INVALID, "ls_op_grid_sample: null argument");
  if (adaptive(op)) return adaptive_refused("ls_op_grid_sample");
  if (!op->on_device) return fail(LS_E_STATE, "ls_op_grid_sample: operator was assembled without a device");
  if (!valid_grid(grid) || nvec < 1 || nvec > 65535)
    return fail(LS_E_INVALID, "ls_op_grid_sample: bad grid or vector count");
  DevOperator& d = op->dev;
  cudaSetDevice(d.device);
  std::string err;
  if (!op->sampler || op->sampler->G != grid) {
    if (!op->sampler) op->sampler.reset(new GridSampler());
    if (!op->sampler->init(op->host, grid, err)) return fail(LS_E_CUDA, "ls_op_grid_sample: " + err);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = op->sampler->sample(reinterpret_cast<const double2*>(x), nvec, d.N, reinterpret_cast<float2*>(out), s);
  if (e != cudaSuccess) return cuda_fail(e, "ls_op_grid_sample");
  return LS_OK;
}

ls_status ls_fgmres_nn(ls_op* op, ls_fno* net, const double* b, int flags, int max_outer, int inner_iter, double tol,
                       double* x, double* history, ls_nn_report* report) {
  if (!op || !b || !x) return fail(LS_E_INVALID, "ls_fgmres_nn: null argument");
  if (adaptive(op)) return adaptive_refused("ls_fgmres_nn");
  if (!op->on_device) return fail(LS_E_STATE, "ls_fgmres_nn: operator was assembled without a device");
  if (max_outer < 1 || inner_iter < 1 || flags < 0 || flags > (LS_NN_GUESS | LS_NN_PRECOND))
    return fail(LS_E_INVALID, "ls_fgmres_nn: bad iteration counts or flags");
  if (flags && !net) return fail(LS_E_INVALID, "ls_fgmres_nn: flags need a network");
  DevOperator& d = op->dev;
  if (!d.has_f32) return fail(LS_E_STATE, "ls_fgmres_nn: call ls_op_enable_f32 first");
  if (flags && net->net.device != d.device) return fail(LS_E_INVALID, "ls_fgmres_nn: network on another device");
  cudaSetDevice(d.device);
  std::string err;
  Precond32* M = nullptr;
  if (flags) {
    // Rebuilt for another net, or for one with another grid (a new net may
    // reuse a destroyed one's address).
    if (!op->nn || op->nn_net != net || op->nn->gs.G != net->net.shape.grid) {
      if (!op->nn) op->nn.reset(new NnPrecond());
      op->nn_net = nullptr;
      if (!op->nn->init(op->host, &net->net, err)) return fail(LS_E_CUDA, "ls_fgmres_nn: " + err);
      op->nn_net = net;
    }
    M = op->nn.get();
  }
  const size_t bytes = (size_t)d.N * sizeof(double2);
  cudaError_t e = cudaMemcpyAsync(d.xbuf, b, bytes, cudaMemcpyHostToDevice, d.stream);
  std::vector<double> hist;
  FlexReport rep;
  double rr = 1.0;
  if (e == cudaSuccess)
    e = dev_gmres_mixed_flex(d, d.xbuf, d.ybuf, (flags & LS_NN_PRECOND) ? M : nullptr,
                             (flags & LS_NN_GUESS) ? M : nullptr, max_outer, inner_iter, tol, hist, rep, rr);
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, d.ybuf, bytes, cudaMemcpyDeviceToHost, d.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d.stream);
  if (e != cudaSuccess) return cuda_fail(e, "ls_fgmres_nn");
  if (history)
    for (size_t i = 0; i < hist.size() && i < (size_t)max_outer + 2; ++i) history[i] = hist[i];
  if (report) {
    report->n_matvec = rep.n_matvec;
    report->n_precond = rep.n_precond;
    report->outer = (int)hist.size() - 1;
    report->fell_back = rep.fell_back ? 1 : 0;
    report->guess_residual = rep.guess_residual;
    report->rel_residual = rr;
  }
  if (!(rr <= tol)) return fail(LS_E_NOT_CONVERGED, "ls_fgmres_nn: tolerance not reached");
  return LS_OK;
}

ls_status ls_set_pdl(int on) {
  set_pdl_enabled(on);
  return LS_OK;
}
int ls_get_pdl(void) { return pdl_enabled(); }

ls_status ls_set_near_overlap(int on) {
  set_near_overlap_enabled(on);
  return LS_OK;
}
int ls_get_near_overlap(void) { return near_overlap_enabled(); }

ls_status ls_set_precompute_cache(const char* dir) {
  precompute_cache_set(dir);
  return LS_OK;
}

ls_status ls_precompute_cache_stats(long long* hits, long long* misses) {
  if (!hits || !misses) return fail(LS_E_INVALID, "ls_precompute_cache_stats: null argument");
  precompute_cache_stats(*hits, *misses);
  return LS_OK;
}

const char* ls_last_error(void) { return t_last_error.c_str(); }
const char* ls_version(void) { return "lsdafmm-gb300 0.1 (sm_103a)"; }

}  // extern "C"
