// DAFMM matvec on the GPU (sm_103a).
//
// y = A x runs as (GMRES/GMRES.cpp:201-254, DFMM::MatVecProduct):
//   1. S[0:N) <- x                          (assignLeafCharges, G_FMM2DTree.hpp:1139)
//   2. P <- 0
//   3. upward, leaves first, one launch per level:
//        S[own] = T * S[children]            (LFR_M2M :2472, HFR_M2M :3772)
//   4. M2L, every level in one launch:
//        P[node] = sum_IL M2L * S[source]     (LFR_M2L :2577, HFR_M2L :3882)
//   5. downward, root side first, one launch per level:
//        P[child] += W * P[parent]            (HFR_L2L :4208, LFR_L2L :2800)
//   6. near field + identity, fused with the output write:
//        y = P[0:N) + kappa^2 q .* sum_n B_n x_nb + x
//                                            (evaluate_NearField_Using_Precomputations_LS :2884,
//                                             collectPotential :3045)
// Steps 3-5 share one gather-GEMV kernel. Each warp owns one output row
// block, so every output element is written by exactly one warp and the
// sums are deterministic (no atomics).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "device.h"

namespace lsg {

template <class C> struct Real;
template <> struct Real<double2> { using T = double; };
template <> struct Real<float2> { using T = float; };

__device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }

// Streaming loads for the operator blocks: every block entry is read once
// per matvec, so it should not displace the gathered charges from L2.
__device__ __forceinline__ double2 ld_stream(const double2* p) { return __ldcs(p); }
__device__ __forceinline__ float2 ld_stream(const float2* p) { return __ldcs(p); }

// Warp reduction of kRowsPerItem complex partial sums (2 * kRowsPerItem
// reals per lane) that halves the values each lane carries at every step:
// after offsets 16, 8, 4 a lane holds 3 of the 24 values, summed over the 8
// lanes that share its bits 2..4, and offsets 2, 1 finish the sum. It needs
// 12 + 6 + 3 + 3 + 3 = 27 additions per lane instead of 5 * 24 = 120.
// On return the lanes with (lane & 3) == 0 hold values base..base+2 with
// base = 12 * bit4 + 6 * bit3 + 3 * bit2; value v is row v / 2, part v % 2.
template <class R>
__device__ __forceinline__ void transpose_reduce24(R (&v)[24], int lane, R (&out)[3]) {
  static_assert(kRowsPerItem == 12, "reduction written for 12 rows");
  R w[12];
  {
    const bool hi = lane & 16;
#pragma unroll
    for (int i = 0; i < 12; ++i) {
      const R send = hi ? v[i] : v[i + 12];
      const R keep = hi ? v[i + 12] : v[i];
      w[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
  }
  R u[6];
  {
    const bool hi = lane & 8;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const R send = hi ? w[i] : w[i + 6];
      const R keep = hi ? w[i + 6] : w[i];
      u[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
  }
  {
    const bool hi = lane & 4;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const R send = hi ? u[i] : u[i + 3];
      const R keep = hi ? u[i + 3] : u[i];
      out[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    out[i] += __shfl_xor_sync(0xffffffffu, out[i], 2);
    out[i] += __shfl_xor_sync(0xffffffffu, out[i], 1);
  }
}

// Gather-GEMV over a list of warp items (see GemvItem). PHASE only names the
// instantiation (0 upward, 1 M2L, 2 downward) so that profilers can tell the
// launches apart.
template <class C, int PHASE>
__global__ void __launch_bounds__(256) gemv_items_kernel(const GemvItem* __restrict__ items, int n_items,
                                                         const C* __restrict__ A, const int* __restrict__ idx,
                                                         const C* __restrict__ src, C* __restrict__ dst,
                                                         int accumulate) {
  using R = typename Real<C>::T;
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_items; w += nw) {
    const GemvItem it = items[w];
    const C* __restrict__ Ab = A + it.a_off;
    const int* __restrict__ ib = idx + it.idx_off;
    if (it.layout == 0) {
      // Row major: lanes stride over the K columns, kRowsPerItem rows per warp.
      R v[2 * kRowsPerItem];
#pragma unroll
      for (int r = 0; r < 2 * kRowsPerItem; ++r) v[r] = R(0);
      const int K = it.K, nr = it.nr;
      int k = lane;
      for (; k + 32 < K; k += 64) {
        const C x0 = src[ib[k]];
        const C x1 = src[ib[k + 32]];
#pragma unroll
        for (int r = 0; r < kRowsPerItem; ++r) {
          if (r < nr) {
            const C a0 = ld_stream(Ab + (size_t)r * K + k);
            const C a1 = ld_stream(Ab + (size_t)r * K + k + 32);
            v[2 * r] = fma(a0.x, x0.x, v[2 * r]);
            v[2 * r] = fma(-a0.y, x0.y, v[2 * r]);
            v[2 * r + 1] = fma(a0.x, x0.y, v[2 * r + 1]);
            v[2 * r + 1] = fma(a0.y, x0.x, v[2 * r + 1]);
            v[2 * r] = fma(a1.x, x1.x, v[2 * r]);
            v[2 * r] = fma(-a1.y, x1.y, v[2 * r]);
            v[2 * r + 1] = fma(a1.x, x1.y, v[2 * r + 1]);
            v[2 * r + 1] = fma(a1.y, x1.x, v[2 * r + 1]);
          }
        }
      }
      if (k < K) {
        const C x0 = src[ib[k]];
#pragma unroll
        for (int r = 0; r < kRowsPerItem; ++r) {
          if (r < nr) {
            const C a0 = ld_stream(Ab + (size_t)r * K + k);
            v[2 * r] = fma(a0.x, x0.x, v[2 * r]);
            v[2 * r] = fma(-a0.y, x0.y, v[2 * r]);
            v[2 * r + 1] = fma(a0.x, x0.y, v[2 * r + 1]);
            v[2 * r + 1] = fma(a0.y, x0.x, v[2 * r + 1]);
          }
        }
      }
      R out[3];
      transpose_reduce24(v, lane, out);
      if ((lane & 3) == 0) {
        const int base = 12 * ((lane >> 4) & 1) + 6 * ((lane >> 3) & 1) + 3 * ((lane >> 2) & 1);
        R* d = reinterpret_cast<R*>(dst + it.out_off);
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          const int vv = base + t;
          if ((vv >> 1) < nr) {
            if (accumulate) d[vv] += out[t];
            else d[vv] = out[t];
          }
        }
      }
    } else {
      // Column major: one lane per row, loop over the (few) columns.
      if (lane < it.nr) {
        R sr = R(0), si = R(0);
        const C* __restrict__ col = Ab + lane;
        const int K = it.K;
        const int lda = it.lda;
        for (int k = 0; k < K; ++k) {
          const C x = src[ib[k]];
          const C a = ld_stream(col + (size_t)k * lda);
          sr = fma(a.x, x.x, sr);
          sr = fma(-a.y, x.y, sr);
          si = fma(a.x, x.y, si);
          si = fma(a.y, x.x, si);
        }
        C* out = dst + it.out_off + lane;
        if (accumulate) {
          C o = *out;
          o.x += sr;
          o.y += si;
          *out = o;
        } else {
          *out = mk(sr, si);
        }
      }
    }
  }
}

// Near field of every leaf (colleague blocks shared by all leaves of the
// leaf level), fused with the far-field potential and the identity.
template <class C>
__global__ void __launch_bounds__(256) near_kernel(int n_out, int rank, const C* __restrict__ B,
                                                   const typename Real<C>::T* __restrict__ kq,
                                                   const int* __restrict__ coll, const C* __restrict__ x,
                                                   const C* __restrict__ P, double2* __restrict__ y, int find_phi) {
  using R = typename Real<C>::T;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_out) return;
  const int leaf = t / rank, row = t - leaf * rank;
  R ar = R(0), ai = R(0);
#pragma unroll 1
  for (int n = 0; n < 9; ++n) {
    const int nb = coll[leaf * 9 + n];
    if (nb < 0) continue;
    const C* __restrict__ Bn = B + ((size_t)n * rank + row) * rank;
    const C* __restrict__ xn = x + (size_t)nb * rank;
    for (int c = 0; c < rank; ++c) {
      const C a = Bn[c];
      const C v = xn[c];
      ar = fma(a.x, v.x, ar);
      ar = fma(-a.y, v.y, ar);
      ai = fma(a.x, v.y, ai);
      ai = fma(a.y, v.x, ai);
    }
  }
  const C p = P[t];
  if (find_phi) {
    const R s = kq[t];
    const C xs = x[t];
    y[t] = make_double2((double)(p.x + s * ar + xs.x), (double)(p.y + s * ai + xs.y));
  } else {
    y[t] = make_double2((double)(p.x + ar), (double)(p.y + ai));
  }
}

__global__ void d2f_kernel(const double2* __restrict__ a, float2* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void d2f_real_kernel(const double* __restrict__ a, float* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

static int g_sm_count = 0;

static int sm_count(int dev) {
  if (g_sm_count == 0) {
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 148;
  }
  return g_sm_count;
}

template <int PHASE, class C>
static void launch_gemv(const DevPhase<C>& ph, const C* src, C* dst, cudaStream_t s, int dev) {
  if (ph.n_items == 0) return;
  const int warps_per_block = 8;
  int blocks = (ph.n_items + warps_per_block - 1) / warps_per_block;
  blocks = std::min(blocks, sm_count(dev) * 8);
  gemv_items_kernel<C, PHASE><<<blocks, 256, 0, s>>>(ph.items, ph.n_items, ph.A, ph.idx, src, dst, ph.accumulate);
}

template <class T>
static bool dmalloc(T** p, size_t n, long long& total, std::string& err) {
  if (n == 0) { *p = nullptr; return true; }
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    err = std::string("cudaMalloc failed: ") + cudaGetErrorString(e);
    *p = nullptr;
    return false;
  }
  total += (long long)(n * sizeof(T));
  return true;
}

static bool upload_phase(const GemvPhase& h, DevPhase<double2>& d, long long& total, std::string& err) {
  d.n_items = (int)h.items.size();
  d.accumulate = h.accumulate;
  d.entries = (long long)h.A.size();
  if (!dmalloc(&d.A, h.A.size(), total, err)) return false;
  if (!dmalloc(&d.idx, h.idx.size(), total, err)) return false;
  if (!dmalloc(&d.items, h.items.size(), total, err)) return false;
  if (h.A.size() && cudaMemcpy(d.A, h.A.data(), h.A.size() * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess) { err = "upload A"; return false; }
  if (h.idx.size() && cudaMemcpy(d.idx, h.idx.data(), h.idx.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) { err = "upload idx"; return false; }
  if (h.items.size() && cudaMemcpy(d.items, h.items.data(), h.items.size() * sizeof(GemvItem), cudaMemcpyHostToDevice) != cudaSuccess) { err = "upload items"; return false; }
  return true;
}

bool dev_upload(const HostOperator& h, DevOperator& d, std::string& err) {
  cudaError_t e = cudaSetDevice(d.device);
  if (e != cudaSuccess) { err = std::string("cudaSetDevice: ") + cudaGetErrorString(e); return false; }
  if ((e = cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking)) != cudaSuccess) {
    err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    return false;
  }
  for (auto& ev : d.ev)
    if (cudaEventCreate(&ev) != cudaSuccess) { err = "cudaEventCreate"; return false; }
  d.N = h.N;
  d.n_leaves = h.n_leaves;
  d.rank = h.rank;
  d.find_phi = h.cfg.findPhi;
  d.charges_len = h.charges_len;
  d.pots_len = h.pots_len;
  long long& tot = d.device_bytes;
  d.up.resize(h.up.size());
  for (size_t i = 0; i < h.up.size(); ++i) if (!upload_phase(h.up[i], d.up[i], tot, err)) return false;
  if (!upload_phase(h.m2l, d.m2l, tot, err)) return false;
  d.down.resize(h.down.size());
  for (size_t i = 0; i < h.down.size(); ++i) if (!upload_phase(h.down[i], d.down[i], tot, err)) return false;
  if (!dmalloc(&d.S, (size_t)h.charges_len, tot, err)) return false;
  if (!dmalloc(&d.P, (size_t)h.pots_len, tot, err)) return false;
  if (!dmalloc(&d.nearB, h.nearB.size(), tot, err)) return false;
  if (!dmalloc(&d.kq, h.kq.size(), tot, err)) return false;
  if (!dmalloc(&d.colleague, h.colleague.size(), tot, err)) return false;
  if (!dmalloc(&d.xbuf, (size_t)h.N, tot, err)) return false;
  if (!dmalloc(&d.ybuf, (size_t)h.N, tot, err)) return false;
  cudaMemcpy(d.nearB, h.nearB.data(), h.nearB.size() * sizeof(double2), cudaMemcpyHostToDevice);
  cudaMemcpy(d.kq, h.kq.data(), h.kq.size() * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(d.colleague, h.colleague.data(), h.colleague.size() * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemset(d.xbuf, 0, (size_t)h.N * sizeof(double2));
  cudaMemset(d.ybuf, 0, (size_t)h.N * sizeof(double2));
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { err = std::string("upload: ") + cudaGetErrorString(e); return false; }
  int launches = 1;  // near kernel
  for (auto& p : d.up) launches += p.n_items > 0;
  launches += d.m2l.n_items > 0;
  for (auto& p : d.down) launches += p.n_items > 0;
  d.launches_per_matvec = launches;
  return true;
}

template <class C>
static void free_phase(DevPhase<C>& p) {
  cudaFree(p.A);
  cudaFree(p.idx);
  cudaFree(p.items);
  p = DevPhase<C>();
}

void dev_free(DevOperator& d) {
  cudaSetDevice(d.device);
  for (auto& p : d.up) free_phase(p);
  for (auto& p : d.down) free_phase(p);
  free_phase(d.m2l);
  // FP32 phases share idx / items with the FP64 phases; only A is theirs.
  for (auto& p : d.up32) cudaFree(p.A);
  for (auto& p : d.down32) cudaFree(p.A);
  cudaFree(d.m2l32.A);
  cudaFree(d.S); cudaFree(d.P); cudaFree(d.nearB); cudaFree(d.kq); cudaFree(d.colleague);
  cudaFree(d.S32); cudaFree(d.P32); cudaFree(d.nearB32); cudaFree(d.kq32);
  cudaFree(d.xbuf); cudaFree(d.ybuf);
  for (auto& ev : d.ev) if (ev) cudaEventDestroy(ev);
  if (d.stream) cudaStreamDestroy(d.stream);
  d = DevOperator();
}

static bool f32_phase(const DevPhase<double2>& a, DevPhase<float2>& b, long long& tot, std::string& err) {
  b.n_items = a.n_items;
  b.accumulate = a.accumulate;
  b.entries = a.entries;
  if (!dmalloc(&b.A, (size_t)a.entries, tot, err)) return false;
  b.idx = a.idx;      // shared with the FP64 phase
  b.items = a.items;  // shared
  if (a.entries) d2f_kernel<<<1024, 256>>>(a.A, b.A, a.entries);
  return true;
}

bool dev_enable_f32(DevOperator& d, std::string& err) {
  if (d.has_f32) return true;
  cudaSetDevice(d.device);
  long long& tot = d.device_bytes;
  d.up32.resize(d.up.size());
  for (size_t i = 0; i < d.up.size(); ++i) if (!f32_phase(d.up[i], d.up32[i], tot, err)) return false;
  if (!f32_phase(d.m2l, d.m2l32, tot, err)) return false;
  d.down32.resize(d.down.size());
  for (size_t i = 0; i < d.down.size(); ++i) if (!f32_phase(d.down[i], d.down32[i], tot, err)) return false;
  if (!dmalloc(&d.S32, (size_t)d.charges_len, tot, err)) return false;
  if (!dmalloc(&d.P32, (size_t)d.pots_len, tot, err)) return false;
  const long long nb = 9LL * d.rank * d.rank;
  if (!dmalloc(&d.nearB32, (size_t)nb, tot, err)) return false;
  if (!dmalloc(&d.kq32, (size_t)d.N, tot, err)) return false;
  d2f_kernel<<<256, 256>>>(d.nearB, d.nearB32, nb);
  d2f_real_kernel<<<256, 256>>>(d.kq, d.kq32, d.N);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { err = std::string("enable_f32: ") + cudaGetErrorString(e); return false; }
  d.has_f32 = true;
  return true;
}

cudaError_t dev_matvec(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool mark_m2l) {
  if (!s) s = d.stream;
  cudaMemcpyAsync(d.S, x, (size_t)d.N * sizeof(double2), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(d.P, 0, (size_t)d.pots_len * sizeof(double2), s);
  for (auto& ph : d.up) launch_gemv<0>(ph, (const double2*)d.S, d.S, s, d.device);
  if (mark_m2l) cudaEventRecord(d.ev[0], s);
  launch_gemv<1>(d.m2l, (const double2*)d.S, d.P, s, d.device);
  if (mark_m2l) cudaEventRecord(d.ev[1], s);
  for (auto& ph : d.down) launch_gemv<2>(ph, (const double2*)d.P, d.P, s, d.device);
  const int n = d.N;
  near_kernel<double2><<<(n + 255) / 256, 256, 0, s>>>(n, d.rank, d.nearB, d.kq, d.colleague, d.S, d.P, y, d.find_phi);
  return cudaGetLastError();
}

cudaError_t dev_matvec_f32(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool mark_m2l) {
  if (!d.has_f32) return cudaErrorInvalidValue;
  if (!s) s = d.stream;
  d2f_kernel<<<256, 256, 0, s>>>(x, d.S32, d.N);
  cudaMemsetAsync(d.P32, 0, (size_t)d.pots_len * sizeof(float2), s);
  for (auto& ph : d.up32) launch_gemv<0>(ph, (const float2*)d.S32, d.S32, s, d.device);
  if (mark_m2l) cudaEventRecord(d.ev[2], s);
  launch_gemv<1>(d.m2l32, (const float2*)d.S32, d.P32, s, d.device);
  if (mark_m2l) cudaEventRecord(d.ev[3], s);
  for (auto& ph : d.down32) launch_gemv<2>(ph, (const float2*)d.P32, d.P32, s, d.device);
  const int n = d.N;
  near_kernel<float2><<<(n + 255) / 256, 256, 0, s>>>(n, d.rank, d.nearB32, d.kq32, d.colleague, d.S32, d.P32, y, d.find_phi);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free matvec (ls_matvec_noalloc).
//
// Some callers must not allocate device memory while they run: a solver
// embedded in a framework whose caching allocator owns the device heap
// (a cudaMalloc behind its back can fail once that allocator has reserved
// the memory, or force a device-wide synchronisation in its middle), and
// drivers that hand over every buffer they use up front. For them the
// matvec's two scratch vectors -- the skeleton charges and the skeleton
// potentials -- live in the fixed, file-scope device array below instead of
// buffers owned by the operator. Every GPU that loads this library reserves
// it (kStaticScratchElems complex doubles, 16 MiB) until the process exits.
//
// The array is shared by all calls and keeps the last call's contents, so
// each call clears what must start at zero. Calls whose work overlaps on the
// GPU (two streams, two operators, two threads) race on it and must be
// serialised by the caller.

namespace {

constexpr int kMaxScratchDevices = 64;

static __device__ __align__(256) double2 g_static_scratch[kStaticScratchElems];

std::mutex g_scratch_mu;
double2* g_scratch_ptr[kMaxScratchDevices] = {};

// Device address of g_static_scratch on `device`. In host code the symbol
// is only a host-side stand-in, so the address is looked up once per device
// with that device current (the first call on a device does this set-up and
// should come before any stream capture).
cudaError_t static_scratch_address(int device, double2** out) {
  if (device < 0 || device >= kMaxScratchDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[device]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return e;
    if (cur != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (cur != device) cudaSetDevice(cur);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = static_cast<double2*>(p);
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

}  // namespace

cudaError_t dev_matvec_static(DevOperator& d, const double2* x, double2* y, cudaStream_t s) {
  if (d.charges_len + d.pots_len > kStaticScratchElems) return cudaErrorInvalidValue;
  if (!s) s = d.stream;
  double2* base = nullptr;
  cudaError_t e = static_scratch_address(d.device, &base);
  if (e != cudaSuccess) return e;
  double2* S = base;
  double2* P = base + d.charges_len;
  cudaMemcpyAsync(S, x, (size_t)d.N * sizeof(double2), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(S + d.N, 0, (size_t)(d.charges_len - d.N) * sizeof(double2), s);
  cudaMemsetAsync(P, 0, (size_t)d.pots_len * sizeof(double2), s);
  for (auto& ph : d.up) launch_gemv<0>(ph, (const double2*)S, S, s, d.device);
  launch_gemv<1>(d.m2l, (const double2*)S, P, s, d.device);
  for (auto& ph : d.down) launch_gemv<2>(ph, (const double2*)P, P, s, d.device);
  const int n = d.N;
  near_kernel<double2><<<(n + 255) / 256, 256, 0, s>>>(n, d.rank, d.nearB, d.kq, d.colleague, S, P, y, d.find_phi);
  return cudaGetLastError();
}

}  // namespace lsg
