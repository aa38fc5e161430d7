// Double-float form of the FP64 operator (sm_103a).
//
// Every complex double of the operator -- block entries, charges,
// potentials, the near-field factors -- is held as a float4
// (re_hi, im_hi, re_lo, im_lo) with hi = fl32(v) and lo = fl32(v - hi), so
// |v - hi - lo| <= 2^-48 |v|. Products and sums run on the FP32 pipe with
// error-free transformations: TwoProduct through FMA and Knuth's TwoSum
// (the compensated dot product "Dot2" of Ogita, Rump and Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26(6), 2005), extended with the
// cross terms hi*lo of split operands. A sum of K products then carries a
// relative error of order K * 2^-48 of the sum of magnitudes, against
// K * 2^-53 for FP64 arithmetic.
//
// Why: on GB300 the FP64 pipe runs 1.25 TFLOP/s against 71 TFLOP/s for FP32,
// so an FP64 complex multiply-add (8 flops per 16-byte block entry) caps a
// gather-GEMV at about 2.5 TB/s of block stream, a third of HBM bandwidth.
// At about 48 FP32 instructions per complex multiply-add the double-float
// product needs less FP32 issue than the HBM stream of its 16-byte entries
// takes, so the phases become bandwidth-bound again.
//
// The phases, their order and their tiles are those of matvec.cu
// (DFMM::MatVecProduct, GMRES/GMRES.cpp:201-254): only the arithmetic type
// changes. The tiles, gather indices and output maps are shared with the
// FP64 phases. The identity term and the final sum y = P + kappa^2 q .* near
// + x are formed in FP64.

#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "device.h"
#include "launch.h"

namespace lsg {
namespace {

// s + e = a + b exactly (Knuth's TwoSum; no assumption on |a|, |b|).
// The _rn intrinsics keep the compiler from fusing these steps.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  const float t = __fadd_rn(a, b);
  const float bb = __fsub_rn(t, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(t, bb)), __fsub_rn(b, bb));
  s = t;
}

// (h, l) += (ah + al) * (bh + bl); al * bl (below 2^-48 of the product) is
// dropped. ah * bh is split exactly into p + e by one FMA, the cross terms
// join e, and p enters the running high part through TwoSum.
__device__ __forceinline__ void dd_mac(float& h, float& l, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  float s, t;
  two_sum(h, p, s, t);
  h = s;
  l = __fadd_rn(l, __fadd_rn(t, e));
}

// Complex (rh, rl) + i (ih, il) += a * x for float4 (re_hi, im_hi, re_lo, im_lo).
__device__ __forceinline__ void cmac(float& rh, float& rl, float& ih, float& il, const float4 a, const float4 x) {
  dd_mac(rh, rl, a.x, a.z, x.x, x.z);
  dd_mac(rh, rl, -a.y, -a.w, x.y, x.w);
  dd_mac(ih, il, a.x, a.z, x.y, x.w);
  dd_mac(ih, il, a.y, a.w, x.x, x.z);
}

// (h, l) + (h2, l2) -> (h, l).
__device__ __forceinline__ void dd_add(float& h, float& l, float h2, float l2) {
  float s, t;
  two_sum(h, h2, s, t);
  h = s;
  l = __fadd_rn(l, __fadd_rn(l2, t));
}

__device__ __forceinline__ float4 pack(float rh, float rl, float ih, float il) {
  float sr, er, si, ei;
  two_sum(rh, rl, sr, er);
  two_sum(ih, il, si, ei);
  return make_float4(sr, si, er, ei);
}

__device__ __forceinline__ float4 split(double2 v) {
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  return make_float4(rh, ih, __double2float_rn(v.x - (double)rh), __double2float_rn(v.y - (double)ih));
}

__device__ __forceinline__ double2 join(float4 v) {
  return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
}

__global__ void split_kernel(const double2* __restrict__ a, float4* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = split(a[i]);
}

// First kernel of a matvec: S[0:n) = split(x) and P = 0.
__global__ void split_zero_kernel(const double2* __restrict__ x, float4* __restrict__ S, long long n,
                                  float4* __restrict__ P, long long np) {
  pdl_enter();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) S[i] = split(ld_chain(x + i));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np; i += stride)
    P[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void split_real_kernel(const double* __restrict__ a, float2* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float h = __double2float_rn(a[i]);
    b[i] = make_float2(h, __double2float_rn(a[i] - (double)h));
  }
}

// Gather-GEMV over the warp tiles of matvec.cu (GemvTile), double-float.
template <int PHASE>
__global__ void __launch_bounds__(256, 3) gemv_df_kernel(const GemvTile* __restrict__ tiles, int n_tiles,
                                                         const float4* __restrict__ A, const int* __restrict__ idx,
                                                         const int* __restrict__ out, const int* __restrict__ qlen,
                                                         const float4* __restrict__ src, float4* __restrict__ dst,
                                                         int accumulate) {
  pdl_enter();
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_tiles; w += nw) {
    const GemvTile t = tiles[w];
    const int ql = qlen[t.lane_base + lane];
    const float4* __restrict__ a = A + t.a_off + lane;
    const int S = 1 << t.log2s;
    const int* __restrict__ ix = idx + t.i_off + (lane >> (5 - t.log2s));  // slice s = lane / R
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    int q = 0;
    for (; q + 4 <= ql; q += 4) {
      const int i0 = ix[S * q], i1 = ix[S * (q + 1)], i2 = ix[S * (q + 2)], i3 = ix[S * (q + 3)];
      const float4 a0 = __ldcs(a + 32 * q), a1 = __ldcs(a + 32 * (q + 1));
      const float4 a2 = __ldcs(a + 32 * (q + 2)), a3 = __ldcs(a + 32 * (q + 3));
      const float4 x0 = ld_chain(src + i0), x1 = ld_chain(src + i1), x2 = ld_chain(src + i2), x3 = ld_chain(src + i3);
      cmac(rh, rl, ih, il, a0, x0);
      cmac(rh, rl, ih, il, a1, x1);
      cmac(rh, rl, ih, il, a2, x2);
      cmac(rh, rl, ih, il, a3, x3);
    }
    for (; q < ql; ++q) cmac(rh, rl, ih, il, __ldcs(a + 32 * q), ld_chain(src + ix[S * q]));
    for (int o = 16; o >= (32 >> t.log2s); o >>= 1) {
      const float rh2 = __shfl_xor_sync(0xffffffffu, rh, o), rl2 = __shfl_xor_sync(0xffffffffu, rl, o);
      const float ih2 = __shfl_xor_sync(0xffffffffu, ih, o), il2 = __shfl_xor_sync(0xffffffffu, il, o);
      dd_add(rh, rl, rh2, rl2);
      dd_add(ih, il, ih2, il2);
    }
    if (lane < t.rows) {
      float4* o = dst + out[t.row_base + lane];
      if (accumulate) {
        const float4 v = ld_chain(o);
        dd_add(rh, rl, v.x, v.z);
        dd_add(ih, il, v.y, v.w);
      }
      *o = pack(rh, rl, ih, il);
    }
  }
}

// c_s = Q^+ x_s per leaf (double-float), and x_hi in FP32 for the E_q term.
__global__ void __launch_bounds__(256) near_coeff_df_kernel(int n_leaves, int rank, int nb,
                                                            const float2* __restrict__ Qp,
                                                            const float4* __restrict__ x, float4* __restrict__ c,
                                                            float2* __restrict__ x32) {
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = n_leaves * rank;
  for (int i = t; i < n; i += gridDim.x * blockDim.x) {
    const float4 v = ld_chain(x + i);
    x32[i] = make_float2(v.x, v.y);
  }
  if (t >= n_leaves * nb) return;
  const int s = t / nb, j = t - s * nb;
  const float2* __restrict__ q = Qp + (size_t)j * rank;
  const float4* __restrict__ xs = x + (size_t)s * rank;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  for (int i = 0; i < rank; ++i) {
    const float2 w = q[i];
    const float4 v = ld_chain(xs + i);
    dd_mac(rh, rl, w.x, w.y, v.x, v.z);
    dd_mac(ih, il, w.x, w.y, v.y, v.w);
  }
  c[t] = pack(rh, rl, ih, il);
}

// Near field in two passes (the colleague blocks are shared by all leaves,
// so the product is a GEMM with a gathered epilogue).
//
// Pass 1: for every leaf s and direction q, the contribution of s to the
// colleague that sees it in direction q:
//   Z[s][q][row]  = Vt_q(row, :) c_s      (double-float)
//   ZE[s][q][row] = E_q(row, :) x32_s      (FP32, the rounding residual)
// A block takes kNearSources leaves; thread (q, row) keeps one accumulator
// per leaf, so every factor entry it loads serves kNearSources products and
// each thread has that many independent dependency chains. The leaves'
// coefficients are staged in shared memory (broadcast reads). Four leaves
// per block and three blocks per SM measured fastest on GB300 (69 us at
// level 6, against 82 us for eight leaves and two blocks).
constexpr int kNearSources = 4;

constexpr int kNearThreads = 352;    // threads of a near-field GEMM block (loop over 9 * rank outputs)
constexpr int kNearMinBlocks = 3;    // resident blocks per SM the register budget must allow

__global__ void __launch_bounds__(kNearThreads, kNearMinBlocks) near_gemm_df_kernel(int n_leaves, int rank, int nb,
                                                           const float4* __restrict__ Vt,
                                                           const float2* __restrict__ E,
                                                           const float4* __restrict__ c,
                                                           const float2* __restrict__ x32,
                                                           float4* __restrict__ Z, float2* __restrict__ ZE) {
  pdl_enter();
  constexpr int NS = kNearSources;
  extern __shared__ float4 sc[];                    // [j][l]: c of source j
  float2* sx = reinterpret_cast<float2*>(sc + NS * nb);  // [j][k]: x32 of source j
  const int s0 = blockIdx.x * NS;
  for (int i = threadIdx.x; i < NS * nb; i += blockDim.x) {
    const int j = i / nb;
    sc[i] = s0 + j < n_leaves ? ld_chain(c + (size_t)s0 * nb + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int i = threadIdx.x; i < NS * rank; i += blockDim.x) {
    const int j = i / rank;
    sx[i] = s0 + j < n_leaves ? ld_chain(x32 + (size_t)s0 * rank + i) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int qr = threadIdx.x; qr < 9 * rank; qr += blockDim.x) {
    const int q = qr / rank, row = qr - q * rank;
    float h[NS][4];
    float er[NS], ei[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      h[j][0] = h[j][1] = h[j][2] = h[j][3] = 0.f;
      er[j] = ei[j] = 0.f;
    }
    const float4* __restrict__ v = Vt + (size_t)q * nb * rank + row;
    for (int l = 0; l < nb; ++l) {
      const float4 a = v[(size_t)l * rank];
#pragma unroll
      for (int j = 0; j < NS; ++j) cmac(h[j][0], h[j][1], h[j][2], h[j][3], a, sc[j * nb + l]);
    }
    const float2* __restrict__ e = E + (size_t)q * rank * rank + row;
    for (int k = 0; k < rank; ++k) {
      const float2 a = e[(size_t)k * rank];
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        const float2 b = sx[j * rank + k];
        er[j] = fmaf(a.x, b.x, er[j]);
        er[j] = fmaf(-a.y, b.y, er[j]);
        ei[j] = fmaf(a.x, b.y, ei[j]);
        ei[j] = fmaf(a.y, b.x, ei[j]);
      }
    }
    const size_t per = (size_t)9 * rank;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      if (s0 + j >= n_leaves) break;
      Z[(size_t)(s0 + j) * per + qr] = pack(h[j][0], h[j][1], h[j][2], h[j][3]);
      ZE[(size_t)(s0 + j) * per + qr] = make_float2(er[j], ei[j]);
    }
  }
}

// Pass 2: y = P + kappa^2 q .* sum_q (Z + ZE)[nb(q)][q][row] + x, one
// thread per output; the double-float partials are added in q order, the
// final sum is formed in FP64 with x read from the caller's FP64 input.
__global__ void __launch_bounds__(256) near_gather_df_kernel(int n_out, int rank, const float4* __restrict__ Z,
                                                             const float2* __restrict__ ZE,
                                                             const double* __restrict__ kq,
                                                             const int* __restrict__ coll,
                                                             const double2* __restrict__ x,
                                                             const float4* __restrict__ P,
                                                             double2* __restrict__ y, int find_phi) {
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_out) return;
  const int leaf = t / rank, row = t - leaf * rank;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f, er = 0.f, ei = 0.f;
  const size_t per = (size_t)9 * rank;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int nbx = coll[leaf * 9 + q];
    if (nbx < 0) continue;
    const size_t o = (size_t)nbx * per + (size_t)q * rank + row;
    const float4 z = ld_chain(Z + o);
    dd_add(rh, rl, z.x, z.z);
    dd_add(ih, il, z.y, z.w);
    const float2 w = ld_chain(ZE + o);
    er += w.x;
    ei += w.y;
  }
  const double ar = ((double)rh + (double)rl) + (double)er;
  const double ai = ((double)ih + (double)il) + (double)ei;
  const double2 p = join(ld_chain(P + t));
  if (find_phi) {
    const double s = kq[t];
    const double2 xs = ld_chain(x + t);
    y[t] = make_double2(p.x + s * ar + xs.x, p.y + s * ai + xs.y);
  } else {
    y[t] = make_double2(p.x + ar, p.y + ai);
  }
}

int g_sms = 0;

int sms(int dev) {
  if (g_sms == 0) {
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 148;
  }
  return g_sms;
}

// y = P[0:n) joined to FP64 (adaptive trees, after the near-field phase).
__global__ void join_out_kernel(const float4* __restrict__ P, double2* __restrict__ y, int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = join(ld_chain(P + i));
}

template <int PHASE>
void launch_df(const DevPhase<float4>& ph, const float4* src, float4* dst, cudaStream_t s, int dev) {
  if (ph.n_tiles == 0) return;
  int blocks = (ph.n_tiles + 7) / 8;
  blocks = std::min(blocks, sms(dev) * 8);
  launch_pdl(gemv_df_kernel<PHASE>, blocks, 256, 0, s, ph.tiles, ph.n_tiles, ph.A, ph.idx, ph.out, ph.klen, src,
             dst, ph.accumulate);
}

template <class T>
bool dalloc(T** p, size_t n, long long& total, std::string& err) {
  if (n == 0) { *p = nullptr; return true; }
  const cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    err = std::string("cudaMalloc failed: ") + cudaGetErrorString(e);
    *p = nullptr;
    return false;
  }
  total += (long long)(n * sizeof(T));
  return true;
}

bool df_phase(const DevPhase<double2>& a, DevPhase<float4>& b, long long& tot, std::string& err) {
  b.n_tiles = a.n_tiles;
  b.accumulate = a.accumulate;
  b.entries = a.entries;
  b.stored = a.stored;
  if (!dalloc(&b.A, (size_t)a.stored, tot, err)) return false;
  b.idx = a.idx;  // shared with the FP64 phase
  b.out = a.out;
  b.klen = a.klen;
  b.tiles = a.tiles;
  if (a.stored) split_kernel<<<1024, 256>>>(a.A, b.A, a.stored);
  return true;
}

}  // namespace

bool dev_enable_df(DevOperator& d, std::string& err) {
  if (d.has_df) return true;
  cudaSetDevice(d.device);
  long long& tot = d.device_bytes;
  d.up_df.resize(d.up.size());
  for (size_t i = 0; i < d.up.size(); ++i) if (!df_phase(d.up[i], d.up_df[i], tot, err)) return false;
  if (!df_phase(d.m2l, d.m2l_df, tot, err)) return false;
  d.down_df.resize(d.down.size());
  for (size_t i = 0; i < d.down.size(); ++i) if (!df_phase(d.down[i], d.down_df[i], tot, err)) return false;
  if (d.generic_near && !df_phase(d.nearph, d.nearph_df, tot, err)) return false;
  if (!dalloc(&d.S_df, (size_t)d.charges_len, tot, err)) return false;
  if (!dalloc(&d.P_df, (size_t)d.pots_len, tot, err)) return false;
  if (!d.generic_near) {  // the uniform tree's factored near field
    const long long nvt = 9LL * d.rank * d.n_bases;
    const long long nqp = (long long)d.n_bases * d.rank;
    if (!dalloc(&d.Vt_df, (size_t)nvt, tot, err)) return false;
    if (!dalloc(&d.Qp_df, (size_t)nqp, tot, err)) return false;
    if (!dalloc(&d.c_df, (size_t)d.n_leaves * d.n_bases, tot, err)) return false;
    if (!dalloc(&d.Z_df, (size_t)d.n_leaves * 9 * d.rank, tot, err)) return false;
    if (!dalloc(&d.ZE_df, (size_t)d.n_leaves * 9 * d.rank, tot, err)) return false;
    split_kernel<<<64, 256>>>(d.nearVt, d.Vt_df, nvt);
    split_real_kernel<<<16, 256>>>(d.Qp, d.Qp_df, nqp);
  }
  const cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { err = std::string("enable double-float: ") + cudaGetErrorString(e); return false; }
  d.has_df = true;
  return true;
}

void dev_free_df(DevOperator& d) {
  for (auto& p : d.up_df) cudaFree(p.A);
  for (auto& p : d.down_df) cudaFree(p.A);
  cudaFree(d.m2l_df.A);
  cudaFree(d.nearph_df.A);
  d.nearph_df = DevPhase<float4>();
  cudaFree(d.S_df); cudaFree(d.P_df); cudaFree(d.Vt_df); cudaFree(d.Qp_df); cudaFree(d.c_df);
  cudaFree(d.Z_df); cudaFree(d.ZE_df);
  d.up_df.clear();
  d.down_df.clear();
  d.m2l_df = DevPhase<float4>();
  d.S_df = nullptr; d.P_df = nullptr; d.Vt_df = nullptr; d.Qp_df = nullptr; d.c_df = nullptr;
  d.Z_df = nullptr; d.ZE_df = nullptr;
  d.has_df = false;
}

cudaError_t dev_matvec_df(DevOperator& d, const double2* x, double2* y, cudaStream_t s, bool mark_m2l) {
  if (!d.has_df) return cudaErrorInvalidValue;
  if (!s) s = d.stream;
  const int n = d.N;
  launch_pdl(split_zero_kernel, (unsigned)sms(d.device) * 4, 256, 0, s, x, d.S_df, (long long)n, d.P_df,
             d.pots_len);
  const size_t near_smem = (size_t)kNearSources * (d.n_bases * sizeof(float4) + d.rank * sizeof(float2));
  const unsigned near_blocks = (unsigned)((d.n_leaves + kNearSources - 1) / kNearSources);
  // near-field coefficients and pass 1 beside the far-field chain (ls_set_near_overlap)
  const bool overlap = !mark_m2l && dev_near_overlap(d);
  if (overlap) {
    cudaEventRecord(d.near_fork, s);
    cudaStreamWaitEvent(d.near_stream, d.near_fork, 0);
    launch_pdl(near_coeff_df_kernel, (unsigned)((d.n_leaves * d.n_bases + 255) / 256), 256, 0, d.near_stream,
               d.n_leaves, d.rank, d.n_bases, d.Qp_df, d.S_df, d.c_df, d.x32);
    launch_pdl(near_gemm_df_kernel, near_blocks, kNearThreads, near_smem, d.near_stream, d.n_leaves, d.rank,
               d.n_bases, d.Vt_df, d.nearE, d.c_df, d.x32, d.Z_df, d.ZE_df);
    cudaEventRecord(d.near_join, d.near_stream);
  }
  for (auto& ph : d.up_df) launch_df<0>(ph, (const float4*)d.S_df, d.S_df, s, d.device);
  if (mark_m2l) cudaEventRecord(d.ev[0], s);
  launch_df<1>(d.m2l_df, (const float4*)d.S_df, d.P_df, s, d.device);
  if (mark_m2l) cudaEventRecord(d.ev[1], s);
  for (auto& ph : d.down_df) launch_df<2>(ph, (const float4*)d.P_df, d.P_df, s, d.device);
  if (mark_m2l) cudaEventRecord(d.ev_down[0], s);
  if (d.generic_near) {
    launch_df<3>(d.nearph_df, (const float4*)d.S_df, d.P_df, s, d.device);
    launch_pdl(join_out_kernel, (unsigned)((n + 255) / 256), 256, 0, s, (const float4*)d.P_df, y, n);
    return cudaGetLastError();
  }
  if (overlap) {
    cudaStreamWaitEvent(s, d.near_join, 0);
  } else {
    launch_pdl(near_coeff_df_kernel, (unsigned)((d.n_leaves * d.n_bases + 255) / 256), 256, 0, s, d.n_leaves, d.rank,
               d.n_bases, d.Qp_df, d.S_df, d.c_df, d.x32);
    launch_pdl(near_gemm_df_kernel, near_blocks, kNearThreads, near_smem, s, d.n_leaves, d.rank, d.n_bases, d.Vt_df,
               d.nearE, d.c_df, d.x32, d.Z_df, d.ZE_df);
  }
  launch_pdl(near_gather_df_kernel, (unsigned)((n + 255) / 256), 256, 0, s, n, d.rank, d.Z_df, d.ZE_df, d.kq,
             d.colleague, x, d.P_df, y, d.find_phi);
  return cudaGetLastError();
}

}  // namespace lsg
