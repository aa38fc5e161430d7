// Many right-hand sides on one operator: the incident fields of many
// directions on one scatterer (the reference solves them one GMRES run at a
// time, GMRES/GMRES.cpp:336-470).
//
// A block of kBatchRhs right-hand sides is carried through the FP32
// operator together. Block vectors are stored rhs-minor, element (i, j) at
// i * kBatchRhs + j, so the kBatchRhs values a gather needs sit in one
// 64-byte segment and every operator entry read from HBM serves kBatchRhs
// products: the single-vector gather-GEMV reads 8 bytes per 8 flops, the
// block one 8 bytes per 64 flops.
//
// The solver is the mixed-precision refinement of gmres.cu with a block
// inner solve: per right-hand side an FP32 GMRES (its own Krylov basis,
// Hessenberg and Givens rotations, its own stopping test), all of them
// sharing each operator apply and each orthogonalisation launch; the
// residuals are formed with the FP64 operator one column at a time.
//
// Two block widths share this solver (template parameter NR): kBatchRhs (8)
// right-hand sides with the CUDA-core block apply below, and kTcRhs (64)
// with the tensor-core block apply of batched_tc.cu, where 64 columns make
// every operator block a dense contraction.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "device.h"
#include "launch.h"

namespace lsg {

namespace {
constexpr int NR8 = kBatchRhs;  // width of the CUDA-core block kernels
constexpr int kBDotThreads = 128;
constexpr int kBDotBlocks = 304;
}  // namespace

template <int NR>
struct BatchWorkspace {
  // FP32 operator work vectors of one block.
  float2* S = nullptr;   // (charges_len + 1) x NR; the last row stays zero
  float2* P = nullptr;   // pots_len x NR
  float2* Z = nullptr;   // near field, pass 1: n_leaves x 9 x rank x NR (CUDA-core apply only)
  // Block Arnoldi: V [step][point][rhs], w, right-hand side, correction.
  float2* V = nullptr;
  float2* w = nullptr;
  float2* rhs = nullptr;
  float2* dx = nullptr;
  double2* partial = nullptr;  // (m + 2) x NR x kBDotBlocks
  double2* h = nullptr;        // (m + 2) x NR
  double2* h2 = nullptr;
  double2* nrm = nullptr;      // NR
  double2* pinned = nullptr;   // host: h, h2 ((m + 2) x NR each), nrm (NR)
  cudaEvent_t copied = nullptr;
  cudaEvent_t orthogonalised = nullptr;  // a step's Gram-Schmidt kernels are done
  cudaStream_t side = nullptr;           // the coefficient copies, off the operator's stream
  // FP64 outer loop: residual columns, one product, right-hand sides and
  // solutions of a call (device copies of the caller's host arrays).
  double2* res = nullptr;      // N x NR
  double2* tmp = nullptr;      // N
  int n = 0, cap = -1;
  long long mem = 0;           // device bytes held
  bool vec_ready = false;
  void release() {
    cudaFree(S); cudaFree(P); cudaFree(Z); cudaFree(V); cudaFree(w); cudaFree(rhs); cudaFree(dx);
    cudaFree(partial); cudaFree(h); cudaFree(h2); cudaFree(nrm); cudaFree(res); cudaFree(tmp);
    S = P = Z = V = w = rhs = dx = nullptr;
    partial = h = h2 = nrm = res = tmp = nullptr;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    if (copied) cudaEventDestroy(copied);
    if (orthogonalised) cudaEventDestroy(orthogonalised);
    if (side) cudaStreamDestroy(side);
    copied = orthogonalised = nullptr;
    side = nullptr;
    n = 0;
    cap = -1;
    vec_ready = false;
  }
  cudaError_t ensure_vectors(const DevOperator& d) {
    if (vec_ready) return cudaSuccess;
    cudaError_t e = cudaMalloc(&S, (size_t)(d.charges_len + 1) * NR * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemset(S, 0, (size_t)(d.charges_len + 1) * NR * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&P, (size_t)d.pots_len * NR * sizeof(float2));
    if (e == cudaSuccess && NR == NR8) e = cudaMalloc(&Z, (size_t)d.n_leaves * 9 * d.rank * NR * sizeof(float2));
    if (e != cudaSuccess) return e;
    vec_ready = true;
    return cudaSuccess;
  }
  cudaError_t ensure_basis(int n_, int m) {
    if (n_ == n && m <= cap) return cudaSuccess;
    cudaFree(V); cudaFree(w); cudaFree(rhs); cudaFree(dx); cudaFree(partial); cudaFree(h); cudaFree(h2);
    cudaFree(nrm); cudaFree(res); cudaFree(tmp);
    V = w = rhs = dx = nullptr;
    partial = h = h2 = nrm = res = tmp = nullptr;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    if (copied) cudaEventDestroy(copied);
    if (orthogonalised) cudaEventDestroy(orthogonalised);
    if (side) cudaStreamDestroy(side);
    copied = orthogonalised = nullptr;
    side = nullptr;
    n = 0;
    cap = -1;
    const size_t blk = (size_t)n_ * NR * sizeof(float2);
    cudaError_t e = cudaMalloc(&V, blk * (m + 1));
    if (e == cudaSuccess) e = cudaMalloc(&w, blk);
    if (e == cudaSuccess) e = cudaMalloc(&rhs, blk);
    if (e == cudaSuccess) e = cudaMalloc(&dx, blk);
    if (e == cudaSuccess) e = cudaMalloc(&partial, (size_t)(m + 2) * NR * kBDotBlocks * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&h, (size_t)(m + 2) * NR * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&h2, (size_t)(m + 2) * NR * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&nrm, (size_t)NR * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&res, (size_t)n_ * NR * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&tmp, (size_t)n_ * sizeof(double2));
    if (e == cudaSuccess) e = cudaMallocHost(&pinned, (size_t)(2 * (m + 2) * NR + NR) * sizeof(double2));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&orthogonalised, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    n = n_;
    cap = m;
    return cudaSuccess;
  }
};

template <int NR> BatchWorkspace<NR>& batch_ws(DevOperator& d);
template <> BatchWorkspace<kBatchRhs>& batch_ws<kBatchRhs>(DevOperator& d) {
  if (!d.bws) d.bws = new BatchWorkspace<kBatchRhs>();
  return *d.bws;
}
template <> BatchWorkspace<kTcRhs>& batch_ws<kTcRhs>(DevOperator& d) {
  if (!d.bws_tc) d.bws_tc = new BatchWorkspace<kTcRhs>();
  return *d.bws_tc;
}

void dev_free_batch(DevOperator& d) {
  if (d.bws) {
    d.bws->release();
    delete d.bws;
    d.bws = nullptr;
  }
  if (d.bws_tc) {
    d.bws_tc->release();
    delete d.bws_tc;
    d.bws_tc = nullptr;
  }
}

namespace {

__device__ __forceinline__ void cmac32(float& sr, float& si, float2 a, float xr, float xi) {
  sr = fmaf(a.x, xr, sr);
  sr = fmaf(-a.y, xi, sr);
  si = fmaf(a.x, xi, si);
  si = fmaf(a.y, xr, si);
}

// Gather-GEMV over the warp tiles of matvec.cu (GemvTile) for a block of
// NR right-hand sides: each lane keeps NR complex sums and every entry of
// A it loads multiplies NR gathered values (two 32-byte loads).
template <int PHASE>
__global__ void __launch_bounds__(256, 2) gemv_block_kernel(const GemvTile* __restrict__ tiles, int n_tiles,
                                                            const float2* __restrict__ A, const int* __restrict__ idx,
                                                            const int* __restrict__ out,
                                                            const int* __restrict__ qlen,
                                                            const float2* __restrict__ src, float2* __restrict__ dst,
                                                            int accumulate) {
  pdl_enter();
  constexpr int NV = NR8 / 2;  // float4 per gathered point
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const float4* __restrict__ src4 = reinterpret_cast<const float4*>(src);
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_tiles; w += nw) {
    const GemvTile t = tiles[w];
    const int ql = qlen[t.lane_base + lane];
    const int S = 1 << t.log2s;
    const float2* __restrict__ a = A + t.a_off + lane;
    const int* __restrict__ ix = idx + t.i_off + (lane >> (5 - t.log2s));
    float sr[NR8], si[NR8];
#pragma unroll
    for (int j = 0; j < NR8; ++j) sr[j] = si[j] = 0.f;
    int q = 0;
    for (; q + 2 <= ql; q += 2) {
      const int i0 = ix[S * q], i1 = ix[S * (q + 1)];
      const float2 a0 = __ldcs(a + 32 * q), a1 = __ldcs(a + 32 * (q + 1));
      float4 v0[NV], v1[NV];
#pragma unroll
      for (int p = 0; p < NV; ++p) v0[p] = ld_chain(src4 + (size_t)i0 * NV + p);
#pragma unroll
      for (int p = 0; p < NV; ++p) v1[p] = ld_chain(src4 + (size_t)i1 * NV + p);
#pragma unroll
      for (int p = 0; p < NV; ++p) {
        cmac32(sr[2 * p], si[2 * p], a0, v0[p].x, v0[p].y);
        cmac32(sr[2 * p + 1], si[2 * p + 1], a0, v0[p].z, v0[p].w);
        cmac32(sr[2 * p], si[2 * p], a1, v1[p].x, v1[p].y);
        cmac32(sr[2 * p + 1], si[2 * p + 1], a1, v1[p].z, v1[p].w);
      }
    }
    if (q < ql) {
      const int i0 = ix[S * q];
      const float2 a0 = __ldcs(a + 32 * q);
#pragma unroll
      for (int p = 0; p < NV; ++p) {
        const float4 v = ld_chain(src4 + (size_t)i0 * NV + p);
        cmac32(sr[2 * p], si[2 * p], a0, v.x, v.y);
        cmac32(sr[2 * p + 1], si[2 * p + 1], a0, v.z, v.w);
      }
    }
    for (int o = 16; o >= (32 >> t.log2s); o >>= 1) {
#pragma unroll
      for (int j = 0; j < NR8; ++j) {
        sr[j] += __shfl_xor_sync(0xffffffffu, sr[j], o);
        si[j] += __shfl_xor_sync(0xffffffffu, si[j], o);
      }
    }
    if (lane < t.rows) {
      float4* __restrict__ o4 = reinterpret_cast<float4*>(dst) + (size_t)out[t.row_base + lane] * NV;
#pragma unroll
      for (int p = 0; p < NV; ++p) {
        float4 v = make_float4(sr[2 * p], si[2 * p], sr[2 * p + 1], si[2 * p + 1]);
        if (accumulate) {
          const float4 u = ld_chain(o4 + p);
          v.x += u.x;
          v.y += u.y;
          v.z += u.z;
          v.w += u.w;
        }
        o4[p] = v;
      }
    }
  }
}

// Near field for a block, pass 1 (as near_gemm32_kernel, matvec.cu):
// Z[s][q][row][j] = B_q(row, :) x_s[:, j]. A thread block takes two
// leaves (their NR8 columns staged in shared memory); thread (q, row) keeps
// 2 x NR8 sums, so every block entry it loads serves 16 products.
constexpr int kBatchNearSources = 2;

__global__ void __launch_bounds__(352, 2) near_gemm_block_kernel(int n_leaves, int rank,
                                                                 const float2* __restrict__ BT,
                                                                 const float2* __restrict__ x,
                                                                 float2* __restrict__ Z) {
  pdl_enter();
  constexpr int NS = kBatchNearSources;
  constexpr int NV = NR8 / 2;
  extern __shared__ float4 sx4[];  // [s][k][p]
  const int s0 = blockIdx.x * NS;
  const int tot = NS * rank * NV;
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int s = i / (rank * NV);
    sx4[i] = s0 + s < n_leaves ? ld_chain(reinterpret_cast<const float4*>(x) + (size_t)s0 * rank * NV + i)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  for (int qr = threadIdx.x; qr < 9 * rank; qr += blockDim.x) {
    const int q = qr / rank, row = qr - q * rank;
    float ar[NS][NR8], ai[NS][NR8];
#pragma unroll
    for (int s = 0; s < NS; ++s)
#pragma unroll
      for (int j = 0; j < NR8; ++j) ar[s][j] = ai[s][j] = 0.f;
    const float2* __restrict__ b = BT + (size_t)q * rank * rank + row;
    for (int k = 0; k < rank; ++k) {
      const float2 a = b[(size_t)k * rank];
#pragma unroll
      for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int p = 0; p < NV; ++p) {
          const float4 v = sx4[(s * rank + k) * NV + p];
          cmac32(ar[s][2 * p], ai[s][2 * p], a, v.x, v.y);
          cmac32(ar[s][2 * p + 1], ai[s][2 * p + 1], a, v.z, v.w);
        }
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      if (s0 + s >= n_leaves) break;
      float4* __restrict__ z4 = reinterpret_cast<float4*>(Z) + ((size_t)(s0 + s) * 9 * rank + qr) * NV;
#pragma unroll
      for (int p = 0; p < NV; ++p) z4[p] = make_float4(ar[s][2 * p], ai[s][2 * p], ar[s][2 * p + 1], ai[s][2 * p + 1]);
    }
  }
}

// Pass 2, one thread per (output point, right-hand side).
__global__ void __launch_bounds__(256) near_gather_block_kernel(int n_out, int rank, const float2* __restrict__ Z,
                                                                const float* __restrict__ kq,
                                                                const int* __restrict__ coll,
                                                                const float2* __restrict__ x,
                                                                const float2* __restrict__ P,
                                                                float2* __restrict__ y, int find_phi) {
  pdl_enter();
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)n_out * NR8) return;
  const int t = (int)(e / NR8), j = (int)(e - (long long)t * NR8);
  const int leaf = t / rank, row = t - leaf * rank;
  float ar = 0.f, ai = 0.f;
  const size_t per = (size_t)9 * rank;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int nbx = coll[leaf * 9 + q];
    if (nbx < 0) continue;
    const float2 z = ld_chain(Z + ((size_t)nbx * per + (size_t)q * rank + row) * NR8 + j);
    ar += z.x;
    ai += z.y;
  }
  const float2 p = ld_chain(P + e);
  if (find_phi) {
    const float s = kq[t];
    const float2 xs = ld_chain(x + e);
    y[e] = make_float2(p.x + s * ar + xs.x, p.y + s * ai + xs.y);
  } else {
    y[e] = make_float2(p.x + ar, p.y + ai);
  }
}

// partial[((col * NR) + j) * gridDim.x + block] = sum_{rows of block}
// conj(V[col][row][j]) * w[row][j] for the NR right-hand sides. Thread t
// owns right-hand side t % NR and every (128 / NR)-th row of the block's
// chunk, so a warp reads 256 contiguous bytes per step; the row groups are
// summed in shared memory in a fixed order (deterministic).
template <int NR>
__global__ void __launch_bounds__(kBDotThreads) multidot_block_kernel(const float2* __restrict__ V, int n,
                                                                      const float2* __restrict__ w,
                                                                      double2* __restrict__ partial) {
  pdl_enter();
  constexpr int G = kBDotThreads / NR;
  __shared__ float2 red[G][NR];
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * chunk;
  const int len = max(0, min(chunk, n - r0));
  const int col = blockIdx.y;
  const int j = threadIdx.x % NR, grp = threadIdx.x / NR;
  const float2* __restrict__ v = V + ((size_t)col * n + r0) * NR + j;
  const float2* __restrict__ wv = w + (size_t)r0 * NR + j;
  float ar = 0.f, ai = 0.f;
  for (int i = grp; i < len; i += G) {
    const float2 a = ld_chain(v + (size_t)i * NR), b = ld_chain(wv + (size_t)i * NR);
    ar = fmaf(a.x, b.x, fmaf(a.y, b.y, ar));
    ai = fmaf(a.x, b.y, fmaf(-a.y, b.x, ai));
  }
  red[grp][j] = make_float2(ar, ai);
  __syncthreads();
  if (threadIdx.x < NR) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < G; ++k) {
      a += (double)red[k][threadIdx.x].x;
      b += (double)red[k][threadIdx.x].y;
    }
    partial[((size_t)col * NR + threadIdx.x) * gridDim.x + blockIdx.x] = make_double2(a, b);
  }
}

// out[c] = sum_b partial[c * nb + b], one warp per entry (fixed order).
__global__ void reduce_block_partials_kernel(const double2* __restrict__ partial, int nb, int nent,
                                             double2* __restrict__ out) {
  pdl_enter();
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= nent) return;
  double a = 0.0, b = 0.0;
  for (int k = lane; k < nb; k += 32) {
    const double2 p = ld_chain(partial + (size_t)c * nb + k);
    a += p.x;
    b += p.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) out[c] = make_double2(a, b);
}

// w[i][j] += sign * sum_c V[c][i][j] * h[c][j]
template <int NR>
__global__ void __launch_bounds__(256, 4) multi_axpy_block_kernel(float2* __restrict__ w, const float2* __restrict__ V,
                                                               int n, int ncols, const double2* __restrict__ h,
                                                               float sign) {
  pdl_enter();
  const long long tot = (long long)n * NR;
  const long long stride = (long long)n * NR;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e % NR);
    float sr = 0.f, si = 0.f;
    int c = 0;
    for (; c + 4 <= ncols; c += 4) {
      float2 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = ld_chain(V + (size_t)(c + u) * stride + e);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const double2 hc = ld_chain(h + (size_t)(c + u) * NR + j);
        cmac32(sr, si, v[u], (float)hc.x, (float)hc.y);
      }
    }
    for (; c < ncols; ++c) {
      const double2 hc = ld_chain(h + (size_t)c * NR + j);
      cmac32(sr, si, ld_chain(V + (size_t)c * stride + e), (float)hc.x, (float)hc.y);
    }
    float2 o = ld_chain(w + e);
    o.x += sign * sr;
    o.y += sign * si;
    w[e] = o;
  }
}

// b[i][j] = a[i][j] / sqrt(nrm[j]), zero for a zero norm. The NR factors
// are formed once per thread block (FP64 divides are slow on GB300).
template <int NR>
__global__ void scale_block_kernel(const float2* __restrict__ a, float2* __restrict__ b,
                                   const double2* __restrict__ nrm, int n) {
  pdl_enter();
  __shared__ float f[NR];
  if (threadIdx.x < NR) {
    const double nn = ld_chain(nrm + threadIdx.x).x;
    f[threadIdx.x] = nn > 0.0 ? (float)(1.0 / sqrt(nn)) : 0.f;
  }
  __syncthreads();
  const long long tot = (long long)n * NR;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x) {
    const float s = f[e % NR];
    const float2 v = ld_chain(a + e);
    b[e] = make_float2(v.x * s, v.y * s);
  }
}

// r32[i][j] = (float) r[j * n + i] for active columns, 0 otherwise.
template <int NR>
__global__ void pack_block_kernel(const double2* __restrict__ r, float2* __restrict__ r32, int n,
                                  unsigned long long active) {
  pdl_enter();
  const long long tot = (long long)n * NR;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / NR), j = (int)(e % NR);
    if ((active >> j) & 1ull) {
      const double2 v = ld_chain(r + (size_t)j * n + i);
      r32[e] = make_float2((float)v.x, (float)v.y);
    } else {
      r32[e] = make_float2(0.f, 0.f);
    }
  }
}

// x[j * n + i] += dx[i][j] for active columns.
template <int NR>
__global__ void unpack_add_block_kernel(double2* __restrict__ x, const float2* __restrict__ dx, int n, int ncols,
                                        unsigned long long active) {
  pdl_enter();
  const long long tot = (long long)n * ncols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / n), i = (int)(e % n);
    if (!((active >> j) & 1ull)) continue;
    const float2 d = ld_chain(dx + (size_t)i * NR + j);
    double2 u = ld_chain(x + e);
    u.x += (double)d.x;
    u.y += (double)d.y;
    x[e] = u;
  }
}

__global__ void sub64_kernel(const double2* __restrict__ a, const double2* __restrict__ b, double2* __restrict__ c,
                             int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 u = ld_chain(a + i), v = ld_chain(b + i);
    c[i] = make_double2(u.x - v.x, u.y - v.y);
  }
}

// partial[col * gridDim.x + block] = |A[:, col]|^2 over the block's rows (FP64 columns, leading dimension n).
__global__ void __launch_bounds__(kBDotThreads) colnorm_kernel(const double2* __restrict__ A, int n,
                                                               double2* __restrict__ partial) {
  pdl_enter();
  __shared__ double red[kBDotThreads / 32];
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * chunk;
  const int len = max(0, min(chunk, n - r0));
  const double2* __restrict__ a = A + (size_t)blockIdx.y * n + r0;
  double s = 0.0;
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    const double2 v = ld_chain(a + i);
    s = fma(v.x, v.x, fma(v.y, v.y, s));
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kBDotThreads / 32; ++k) t += red[k];
    partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = make_double2(t, 0.0);
  }
}

int grid_n(long long n) { return (int)std::min<long long>((n + 255) / 256, 152 * 8); }

__global__ void zero_f2_block_kernel(float2* __restrict__ p, long long n) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = make_float2(0.f, 0.f);
}

int sms_b(int dev) {
  static int v = 0;
  if (v == 0) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (v <= 0) v = 148;
  }
  return v;
}

template <int PHASE>
void launch_block(const DevPhase<float2>& ph, const float2* src, float2* dst, cudaStream_t s, int dev) {
  if (ph.n_tiles == 0) return;
  int blocks = (ph.n_tiles + 7) / 8;
  blocks = std::min(blocks, sms_b(dev) * 8);
  launch_pdl(gemv_block_kernel<PHASE>, blocks, 256, 0, s, ph.tiles, ph.n_tiles, ph.A, ph.idx, ph.out, ph.klen, src, dst,
                                                  ph.accumulate);
}

// |columns|^2 of an n x ncols FP64 array into out (host), ncols <= NR.
template <int NR>
cudaError_t colnorms(const double2* A, int n, int ncols, BatchWorkspace<NR>& B, cudaStream_t s, double* out) {
  launch_pdl(colnorm_kernel, dim3(kBDotBlocks, ncols), kBDotThreads, 0, s, A, n, B.partial);
  launch_pdl(reduce_block_partials_kernel, (ncols * 32 + 255) / 256, 256, 0, s, B.partial, kBDotBlocks, ncols, B.nrm);
  std::vector<double2> v(ncols);
  cudaError_t e = cudaMemcpyAsync(v.data(), B.nrm, (size_t)ncols * sizeof(double2), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  for (int j = 0; j < ncols; ++j) out[j] = v[j].x;
  return cudaSuccess;
}

template <int NR>
void block_multidot(const float2* V, int n, int ncols, const float2* w, BatchWorkspace<NR>& B, double2* h,
                    cudaStream_t s) {
  launch_pdl(multidot_block_kernel<NR>, dim3(kBDotBlocks, ncols), kBDotThreads, 0, s, V, n, w, B.partial);
  launch_pdl(reduce_block_partials_kernel, (ncols * NR * 32 + 255) / 256, 256, 0, s, B.partial, kBDotBlocks, ncols * NR, h);
}

using cdh = std::complex<double>;

// Per right-hand side state of the block Arnoldi process.
struct RhsState {
  std::vector<std::vector<cdh>> H;
  std::vector<cdh> cs, sn, g;
  double bnorm = 1.0, tol = 0.0;
  int K = 0;
  bool done = false;
};

// y = A32 x for one block of NR right-hand sides.
template <int NR> cudaError_t block_apply(DevOperator& d, BatchWorkspace<NR>& B, const float2* x, float2* y,
                                          cudaStream_t s);
template <> cudaError_t block_apply<kBatchRhs>(DevOperator& d, BatchWorkspace<kBatchRhs>&, const float2* x, float2* y,
                                               cudaStream_t s) {
  return dev_matvec_f32_batch(d, x, y, s);
}
template <> cudaError_t block_apply<kTcRhs>(DevOperator& d, BatchWorkspace<kTcRhs>& B, const float2* x, float2* y,
                                            cudaStream_t s) {
  return dev_matvec_f32_wide(d, x, y, B.S, B.P, s);
}

// Block Arnoldi (FP32 basis, one GMRES per column sharing the launches):
// solves A32 x_j = rhs_j for the columns with rs[j].done == false, x = 0
// start. Returns the block operator applies made.
template <int NR>
cudaError_t block_arnoldi(DevOperator& d, BatchWorkspace<NR>& B, int m, std::vector<RhsState>& rs, int& applies) {
  cudaStream_t s = d.stream;
  const int n = d.N;
  const size_t blk = (size_t)n * NR;
  cudaError_t e;
  applies = 0;
  // beta_j = |rhs_j|, V_0 = rhs / beta
  block_multidot(B.rhs, n, 1, B.rhs, B, B.nrm, s);
  std::vector<double2> nv(NR);
  if ((e = cudaMemcpyAsync(nv.data(), B.nrm, NR * sizeof(double2), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  bool any = false;
  for (int j = 0; j < NR; ++j) {
    RhsState& r = rs[j];
    r.H.clear(); r.cs.clear(); r.sn.clear();
    r.K = 0;
    const double beta = std::sqrt(nv[j].x);
    r.g.assign(1, cdh(beta, 0.0));
    if (beta == 0.0) r.done = true;
    any = any || !r.done;
  }
  cudaMemsetAsync(B.dx, 0, blk * sizeof(float2), s);
  if (!any) return cudaStreamSynchronize(s);
  launch_pdl(scale_block_kernel<NR>, grid_n((long long)blk), 256, 0, s, B.rhs, B.V, B.nrm, n);
  if ((e = block_apply<NR>(d, B, B.V, B.w, s)) != cudaSuccess) return e;
  ++applies;
  double2* hp = B.pinned;
  double2* hp2 = B.pinned + (size_t)(m + 2) * NR;
  double2* np = B.pinned + (size_t)2 * (m + 2) * NR;
  int kmax = 0;
  for (int k = 0; k < m; ++k) {
    const float2* Vk = B.V;
    block_multidot(Vk, n, k + 1, B.w, B, B.h, s);
    launch_pdl(multi_axpy_block_kernel<NR>, grid_n((long long)blk), 256, 0, s, B.w, B.V, n, k + 1, B.h, -1.f);
    block_multidot(Vk, n, k + 1, B.w, B, B.h2, s);
    launch_pdl(multi_axpy_block_kernel<NR>, grid_n((long long)blk), 256, 0, s, B.w, B.V, n, k + 1, B.h2, -1.f);
    block_multidot(B.w, n, 1, B.w, B, B.nrm, s);
    launch_pdl(scale_block_kernel<NR>, grid_n((long long)blk), 256, 0, s, B.w, B.V + (size_t)(k + 1) * blk, B.nrm, n);
    // Coefficients to the host on a side stream (as in the single-vector
    // Arnoldi step of gmres.cu): the next block apply follows directly.
    if ((e = cudaEventRecord(B.orthogonalised, s)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(B.side, B.orthogonalised, 0)) != cudaSuccess) return e;
    cudaMemcpyAsync(hp, B.h, (size_t)(k + 1) * NR * sizeof(double2), cudaMemcpyDeviceToHost, B.side);
    cudaMemcpyAsync(hp2, B.h2, (size_t)(k + 1) * NR * sizeof(double2), cudaMemcpyDeviceToHost, B.side);
    cudaMemcpyAsync(np, B.nrm, (size_t)NR * sizeof(double2), cudaMemcpyDeviceToHost, B.side);
    if ((e = cudaEventRecord(B.copied, B.side)) != cudaSuccess) return e;
    if (k + 1 < m) {
      if ((e = block_apply<NR>(d, B, B.V + (size_t)(k + 1) * blk, B.w, s)) != cudaSuccess) return e;
      ++applies;
    }
    if ((e = cudaEventSynchronize(B.copied)) != cudaSuccess) return e;
    kmax = k + 1;
    bool all = true;
    for (int j = 0; j < NR; ++j) {
      RhsState& r = rs[j];
      if (r.done) continue;
      std::vector<cdh> hk(k + 2);
      for (int i = 0; i <= k; ++i)
        hk[i] = cdh(hp[(size_t)i * NR + j].x + hp2[(size_t)i * NR + j].x,
                    hp[(size_t)i * NR + j].y + hp2[(size_t)i * NR + j].y);
      hk[k + 1] = std::sqrt(np[j].x);
      const bool breakdown = std::abs(hk[k + 1]) == 0.0;
      for (int i = 0; i < k; ++i) {
        const cdh t = std::conj(r.cs[i]) * hk[i] + std::conj(r.sn[i]) * hk[i + 1];
        hk[i + 1] = -r.sn[i] * hk[i] + r.cs[i] * hk[i + 1];
        hk[i] = t;
      }
      const double nr = std::sqrt(std::norm(hk[k]) + std::norm(hk[k + 1]));
      const cdh c = nr == 0.0 ? cdh(1.0, 0.0) : hk[k] / nr;
      const cdh sv = nr == 0.0 ? cdh(0.0, 0.0) : hk[k + 1] / nr;
      r.cs.push_back(c);
      r.sn.push_back(sv);
      hk[k] = std::conj(c) * hk[k] + std::conj(sv) * hk[k + 1];
      hk[k + 1] = 0.0;
      r.H.push_back(hk);
      r.g.push_back(-sv * r.g[k]);
      r.g[k] = std::conj(c) * r.g[k];
      r.K = k + 1;
      const double est = std::abs(r.g[k + 1]) / r.bnorm;
      if (est <= r.tol || breakdown) r.done = true;
      all = all && r.done;
    }
    if (all) break;
  }
  // Back substitution per column; y[k][j] (zero past K_j); dx = V y.
  std::vector<double2> y((size_t)kmax * NR, make_double2(0.0, 0.0));
  for (int j = 0; j < NR; ++j) {
    RhsState& r = rs[j];
    std::vector<cdh> yj(r.K);
    for (int i = r.K - 1; i >= 0; --i) {
      cdh sum = r.g[i];
      for (int l = i + 1; l < r.K; ++l) sum -= r.H[l][i] * yj[l];
      yj[i] = sum / r.H[i][i];
    }
    for (int i = 0; i < r.K; ++i) y[(size_t)i * NR + j] = make_double2(yj[i].real(), yj[i].imag());
  }
  if (kmax > 0) {
    cudaMemcpyAsync(B.h, y.data(), y.size() * sizeof(double2), cudaMemcpyHostToDevice, s);
    launch_pdl(multi_axpy_block_kernel<NR>, grid_n((long long)blk), 256, 0, s, B.dx, B.V, n, kmax, B.h, 1.f);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

}  // namespace

cudaError_t dev_matvec_f32_batch(DevOperator& d, const float2* x, float2* y, cudaStream_t s) {
  if (!d.has_f32) return cudaErrorInvalidValue;
  if (!s) s = d.stream;
  BatchWorkspace<kBatchRhs>& B = batch_ws<kBatchRhs>(d);
  cudaError_t e = B.ensure_vectors(d);
  if (e != cudaSuccess) return e;
  cudaMemcpyAsync(B.S, x, (size_t)d.N * NR8 * sizeof(float2), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(B.P, 0, (size_t)d.pots_len * NR8 * sizeof(float2), s);
  for (auto& ph : d.up32) launch_block<0>(ph, (const float2*)B.S, B.S, s, d.device);
  launch_block<1>(d.m2l32, (const float2*)B.S, B.P, s, d.device);
  for (auto& ph : d.down32) launch_block<2>(ph, (const float2*)B.P, B.P, s, d.device);
  if (d.generic_near) {  // adaptive trees: the near phase accumulates into P[0:N), which is y
    launch_block<3>(d.nearph32, (const float2*)B.S, B.P, s, d.device);
    cudaMemcpyAsync(y, B.P, (size_t)d.N * NR8 * sizeof(float2), cudaMemcpyDeviceToDevice, s);
    return cudaGetLastError();
  }
  const int NS = kBatchNearSources;
  launch_pdl(near_gemm_block_kernel, (d.n_leaves + NS - 1) / NS, 352, (size_t)NS * d.rank * NR8 * sizeof(float2), s, 
      d.n_leaves, d.rank, d.nearB32, B.S, B.Z);
  launch_pdl(near_gather_block_kernel, (int)(((long long)d.N * NR8 + 255) / 256), 256, 0, s, d.N, d.rank, B.Z, d.kq32,
                                                                                   d.colleague, B.S, B.P, y,
                                                                                   d.find_phi);
  return cudaGetLastError();
}

cudaError_t dev_matvec_f32_wide_ws(DevOperator& d, const float2* x, float2* y, cudaStream_t s) {
  if (!d.tc) return cudaErrorInvalidValue;
  if (!s) s = d.stream;
  BatchWorkspace<kTcRhs>& B = batch_ws<kTcRhs>(d);
  cudaError_t e = B.ensure_vectors(d);
  if (e != cudaSuccess) return e;
  return dev_matvec_f32_wide(d, x, y, B.S, B.P, s);
}

namespace {

template <int NR>
cudaError_t gmres_mixed_batch(DevOperator& d, int nrhs, const double2* b, double2* x, int max_outer, int inner,
                              double tol, int& n_matvec, std::vector<double>& relres) {
  const int n = d.N;
  cudaStream_t s = d.stream;
  BatchWorkspace<NR>& B = batch_ws<NR>(d);
  cudaError_t e = B.ensure_vectors(d);
  if (e == cudaSuccess) e = B.ensure_basis(n, inner);
  if (e != cudaSuccess) return e;
  n_matvec = 0;
  relres.assign(nrhs, 0.0);
  for (int j0 = 0; j0 < nrhs; j0 += NR) {
    const int nb = std::min(NR, nrhs - j0);
    const double2* bb = b + (size_t)j0 * n;
    double2* xb = x + (size_t)j0 * n;
    std::vector<double> bn2(NR, 0.0);
    if ((e = colnorms(bb, n, nb, B, s, bn2.data())) != cudaSuccess) return e;
    std::vector<double> bn(NR, 0.0), rel(NR, 0.0);
    cudaMemsetAsync(xb, 0, (size_t)n * nb * sizeof(double2), s);
    cudaMemcpyAsync(B.res, bb, (size_t)n * nb * sizeof(double2), cudaMemcpyDeviceToDevice, s);
    for (int j = 0; j < nb; ++j) {
      bn[j] = std::sqrt(bn2[j]);
      rel[j] = bn[j] > 0.0 ? 1.0 : 0.0;
    }
    std::vector<RhsState> rs(NR);
    for (int o = 0; o < max_outer; ++o) {
      unsigned long long active = 0;
      for (int j = 0; j < nb; ++j)
        if (rel[j] > tol) active |= 1ull << j;
      if (!active) break;
      for (int j = 0; j < NR; ++j) {
        rs[j].done = !((active >> j) & 1u);
        // Inner solve to roughly the FP32 operator accuracy.
        rs[j].tol = rs[j].done ? 0.0 : std::max(tol / std::max(rel[j], 1e-300), 1e-6);
        rs[j].bnorm = rs[j].done ? 1.0 : std::max(rel[j] * bn[j], 1e-300);
      }
      launch_pdl(pack_block_kernel<NR>, grid_n((long long)n * NR), 256, 0, s, B.res, B.rhs, n, active);
      int applies = 0;
      if ((e = block_arnoldi(d, B, inner, rs, applies)) != cudaSuccess) return e;
      n_matvec += applies;
      launch_pdl(unpack_add_block_kernel<NR>, grid_n((long long)n * nb), 256, 0, s, xb, B.dx, n, nb, active);
      // FP64 residuals of the active columns.
      for (int j = 0; j < nb; ++j) {
        if (!((active >> j) & 1ull)) continue;
        if ((e = dev_matvec(d, xb + (size_t)j * n, B.tmp, s, false)) != cudaSuccess) return e;
        ++n_matvec;
        launch_pdl(sub64_kernel, grid_n(n), 256, 0, s, bb + (size_t)j * n, B.tmp, B.res + (size_t)j * n, n);
      }
      std::vector<double> rn2(NR, 0.0);
      if ((e = colnorms(B.res, n, nb, B, s, rn2.data())) != cudaSuccess) return e;
      for (int j = 0; j < nb; ++j)
        if ((active >> j) & 1ull) rel[j] = bn[j] > 0.0 ? std::sqrt(rn2[j]) / bn[j] : 0.0;
    }
    for (int j = 0; j < nb; ++j) relres[j0 + j] = rel[j];
  }
  return cudaStreamSynchronize(s);
}

}  // namespace

cudaError_t dev_matvec_f32_many(DevOperator& d, int nrhs, const double2* X, double2* Y) {
  if (!d.tc) return cudaErrorInvalidValue;
  cudaStream_t s = d.stream;
  const int n = d.N;
  BatchWorkspace<kTcRhs>& B = batch_ws<kTcRhs>(d);
  cudaError_t e = B.ensure_vectors(d);
  if (e == cudaSuccess) e = B.ensure_basis(n, 1);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(Y, 0, (size_t)n * nrhs * sizeof(double2), s);
  for (int j0 = 0; j0 < nrhs; j0 += kTcRhs) {
    const int nb = std::min(kTcRhs, nrhs - j0);
    const unsigned long long active = nb == 64 ? ~0ull : ((1ull << nb) - 1);
    launch_pdl(pack_block_kernel<kTcRhs>, grid_n((long long)n * kTcRhs), 256, 0, s, X + (size_t)j0 * n, B.rhs, n,
               active);
    if ((e = dev_matvec_f32_wide(d, B.rhs, B.w, B.S, B.P, s)) != cudaSuccess) return e;
    launch_pdl(unpack_add_block_kernel<kTcRhs>, grid_n((long long)n * nb), 256, 0, s, Y + (size_t)j0 * n,
               (const float2*)B.w, n, nb, active);
  }
  return cudaStreamSynchronize(s);
}

namespace {
template <int NR>
cudaError_t time_block_apply(DevOperator& d, int warmup, int iters, float* ms) {
  cudaStream_t s = d.stream;
  BatchWorkspace<NR>& B = batch_ws<NR>(d);
  cudaError_t e = B.ensure_vectors(d);
  if (e == cudaSuccess) e = B.ensure_basis(d.N, 1);
  if (e != cudaSuccess) return e;
  launch_pdl(zero_f2_block_kernel, grid_n((long long)d.N * NR), 256, 0, s, B.rhs, (long long)d.N * NR);
  for (int i = 0; i < warmup && e == cudaSuccess; ++i) e = block_apply<NR>(d, B, B.rhs, B.w, s);
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, s);
  for (int i = 0; i < iters && e == cudaSuccess; ++i) e = block_apply<NR>(d, B, B.rhs, B.w, s);
  cudaEventRecord(b, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float t = 0.f;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = t / iters;
  return e;
}
}  // namespace

cudaError_t dev_time_block_apply(DevOperator& d, int width, int warmup, int iters, float* ms) {
  if (!d.has_f32) return cudaErrorInvalidValue;
  if (width == kTcRhs) {
    if (!d.tc) return cudaErrorInvalidValue;
    return time_block_apply<kTcRhs>(d, warmup, iters, ms);
  }
  return time_block_apply<kBatchRhs>(d, warmup, iters, ms);
}

cudaError_t dev_gmres_mixed_batch(DevOperator& d, int nrhs, const double2* b, double2* x, int max_outer, int inner,
                                  double tol, int& n_matvec, std::vector<double>& relres) {
  if (!d.has_f32) return cudaErrorInvalidValue;
  if (d.batch_width == kTcRhs) {
    if (!d.tc) return cudaErrorInvalidValue;
    return gmres_mixed_batch<kTcRhs>(d, nrhs, b, x, max_outer, inner, tol, n_matvec, relres);
  }
  return gmres_mixed_batch<kBatchRhs>(d, nrhs, b, x, max_outer, inner, tol, n_matvec, relres);
}

}  // namespace lsg
