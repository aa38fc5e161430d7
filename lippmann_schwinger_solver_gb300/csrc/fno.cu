// Spectral neural operator: forward, backward and Adam kernels (FP32).
//
// Shapes (fno.h): G x G grid, M kept modes per axis, 32 channels, P = B G^2
// points. Every kernel indexes with the channel in the lane (c = lane), so
// the channel-last activations are read and written as whole 128-byte rows.
//
// The kernels are launched one after another without programmatic
// dependent launch. With it, an earlier version of these kernels read, in
// the backward pass, stale values of a buffer that the kernel two launches
// before had read and the preceding kernel had rewritten: the weight
// gradients of the GELU layers came out wrong on GB300 although each kernel
// alone was correct. The present kernels measured correct with it too, but
// the failure depended on which kernels shared the SMs, so plain launches
// are kept (the forward pass of the preconditioner is replayed as a CUDA
// graph instead).
//
// Spectral convolution of one layer, forward:
//   H1 = r2c_y(h)        [B][G][M][32]    y-DFT, kept ky < M
//   H2 = dft_x(H1)       [B][2M][M][32]   x-DFT, kept kx
//   O  = mix(H2, W)      [B][2M][M][32]   per-mode 32 x 32 complex product
//   G1 = idft_x(O)       [B][G][M][32]
//   z  = c2r_y(G1) + Wpw h + b           (the half-spectrum synthesis of
//                                         irfft2, with its 1/G^2)
// Backward runs the adjoints: r2c_y and c2r_y are each other's adjoints up
// to the per-ky weights, dft_x and idft_x likewise, and mix's adjoint uses
// the conjugate transpose of each mode's weight matrix.

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "fno.h"
#include "launch.h"

namespace lsg {

namespace {

constexpr int kWgradChunk = 32;  // points staged per step of the weight-gradient reduction
constexpr int kXWarps = 8;       // warps of an x-DFT block (the input sum is split over them)
constexpr int kXOut = 16;        // most outputs of one x-DFT block (accumulators per lane)
constexpr int kC2rRows = 4;      // y rows per warp step of the c2r synthesis

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  return cdf + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// h[p][c] = b[c] + sum_j w[c][j] in[p][j]; with ssq the field channels
// (1, 2) are divided by the sample's RMS sqrt(ssq / G^2).
__global__ void lift_kernel(long long P, int GG, const float* __restrict__ in, const float* __restrict__ w,
                            const float* __restrict__ b, const float* __restrict__ ssq, float* __restrict__ h) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * kFnoWidth) return;
  const long long p = t >> 5;
  const int c = (int)(t & 31);
  const float sc = ssq ? rsqrtf(fmaxf(ssq[p / GG] / (float)GG, 1e-30f)) : 1.0f;
  const float* x = in + p * kFnoIn;
  float acc = b[c];
#pragma unroll
  for (int j = 0; j < kFnoIn; ++j) acc = fmaf(w[c * kFnoIn + j], (j == 1 || j == 2) ? x[j] * sc : x[j], acc);
  h[t] = acc;
}

// out[r][ky][c] = s_ky sum_y (cos, -sin)(2 pi ky y / G) x[r][y][c], ky < M.
// scaled: s_ky = (ky ? 2 : 1) / G^2 (adjoint of the c2r synthesis), else 1.
// z != null: x is replaced by x * gelu'(z), written to dz (GELU backward).
__global__ void r2c_kernel(int G, int M, int scaled, const float* __restrict__ x, const float* __restrict__ z,
                           float* __restrict__ dz, const float2* __restrict__ tw, float2* __restrict__ out) {
  extern __shared__ float smf[];
  float* xs = smf;                                        // [G][32]
  float2* ts = reinterpret_cast<float2*>(smf + G * 32);   // [G]
  const long long base = (long long)blockIdx.x * G * 32;
  for (int i = threadIdx.x; i < G * 32; i += blockDim.x) {
    float v = x[base + i];
    if (z) {
      v *= gelu_grad(z[base + i]);
      dz[base + i] = v;
    }
    xs[i] = v;
  }
  for (int i = threadIdx.x; i < G; i += blockDim.x) ts[i] = tw[i];
  __syncthreads();
  const int c = threadIdx.x & 31;
  // The kept ky are split over gridDim.y blocks (small batches fill the GPU).
  const int k_lo = (int)(((long long)blockIdx.y * M) / gridDim.y);
  const int k_hi = (int)(((long long)(blockIdx.y + 1) * M) / gridDim.y);
  for (int ky = k_lo + (threadIdx.x >> 5); ky < k_hi; ky += blockDim.x >> 5) {
    float ar = 0.f, ai = 0.f;
    for (int y = 0; y < G; ++y) {
      const float2 t = ts[(ky * y) & (G - 1)];
      const float v = xs[y * 32 + c];
      ar = fmaf(t.x, v, ar);
      ai = fmaf(-t.y, v, ai);
    }
    const float s = scaled ? (ky ? 2.f : 1.f) / ((float)G * (float)G) : 1.f;
    out[((long long)blockIdx.x * M + ky) * 32 + c] = make_float2(ar * s, ai * s);
  }
}

// Along x for one (sample, ky) and one chunk of outputs (blockIdx.y); the
// kept frequency of mode m is m < M ? m : G - 2M + m.
// analysis:  out[b][m][ky][c] = sum_x e^{-2 pi i f_m x / G} in[b][x][ky][c]
// synthesis: out[b][x][ky][c] = sum_m e^{+2 pi i f_m x / G} in[b][m][ky][c]
// The sum over inputs is split over the block's warps: each warp reads its
// own input rows (one coalesced 256-byte row per step) and keeps one
// accumulator pair per output of the chunk, so its FMA chains are
// independent; the warps' partial sums are added in shared memory.
__global__ void __launch_bounds__(kXWarps * 32) xdft_kernel(int G, int M, int analysis, const float2* __restrict__ in,
                                                            const float2* __restrict__ tw, float2* __restrict__ out) {
  __shared__ float2 ts[256];
  __shared__ float2 part[kXWarps][kXOut][32];
  const int NI = analysis ? G : 2 * M, NO = analysis ? 2 * M : G;
  const int b = blockIdx.x / M, ky = blockIdx.x - b * M;
  const int oc = (NO + gridDim.y - 1) / gridDim.y;
  const int o_lo = blockIdx.y * oc;
  const int no = min(oc, NO - o_lo);
  if (no <= 0) return;  // block-uniform
  for (int i = threadIdx.x; i < G; i += blockDim.x) ts[i] = tw[i];
  __syncthreads();
  const int c = threadIdx.x & 31, w = threadIdx.x >> 5;
  const float sg = analysis ? -1.f : 1.f;
  float ar[kXOut], ai[kXOut];
#pragma unroll
  for (int k = 0; k < kXOut; ++k) ar[k] = ai[k] = 0.f;
  const int j_lo = (w * NI) / kXWarps, j_hi = ((w + 1) * NI) / kXWarps;
#pragma unroll 2
  for (int j = j_lo; j < j_hi; ++j) {
    const float2 v = in[(((long long)b * NI + j) * M + ky) * 32 + c];
#pragma unroll
    for (int k = 0; k < kXOut; ++k) {
      if (k < no) {
        const int o = o_lo + k;
        const int m = analysis ? o : j;
        const int f = m < M ? m : G - 2 * M + m;
        const float2 t = ts[(f * (analysis ? j : o)) & (G - 1)];
        const float ti = sg * t.y;
        ar[k] = fmaf(t.x, v.x, fmaf(-ti, v.y, ar[k]));
        ai[k] = fmaf(t.x, v.y, fmaf(ti, v.x, ai[k]));
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kXOut; ++k)
    if (k < no) part[w][k][c] = make_float2(ar[k], ai[k]);
  __syncthreads();
  for (int i = threadIdx.x; i < no * 32; i += blockDim.x) {
    const int k = i >> 5, cc = i & 31;
    float2 acc = part[0][k][cc];
    for (int ww = 1; ww < kXWarps; ++ww) {
      acc.x += part[ww][k][cc].x;
      acc.y += part[ww][k][cc].y;
    }
    out[(((long long)b * NO + o_lo + k) * M + ky) * 32 + cc] = acc;
  }
}

// Per mode m (one block): forward out[b][m][o] = sum_i in[b][m][i] W[m][i][o];
// adjoint out[b][m][i] = sum_o in[b][m][o] conj(W[m][i][o]).
__global__ void mix_kernel(int B, int NM, int adjoint, const float2* __restrict__ in, const float2* __restrict__ W,
                           float2* __restrict__ out) {
  __shared__ float2 ws[32][33];  // ws[k][l]: coefficient of input k in output l
  extern __shared__ float2 xin[];  // [B][32]
  const int m = blockIdx.x;
  const float2* wm = W + (long long)m * 1024;
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
    const int a = i >> 5, bb = i & 31;
    const float2 w = wm[i];
    if (adjoint) ws[bb][a] = make_float2(w.x, -w.y);
    else ws[a][bb] = w;
  }
  for (int i = threadIdx.x; i < B * 32; i += blockDim.x) {
    const int b = i >> 5, k = i & 31;
    xin[i] = in[((long long)b * NM + m) * 32 + k];
  }
  __syncthreads();
  const int l = threadIdx.x & 31;
  for (int b = threadIdx.x >> 5; b < B; b += blockDim.x >> 5) {
    float ar = 0.f, ai = 0.f;
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      const float2 v = xin[b * 32 + k];
      const float2 w = ws[k][l];
      ar = fmaf(v.x, w.x, fmaf(-v.y, w.y, ar));
      ai = fmaf(v.x, w.y, fmaf(v.y, w.x, ai));
    }
    out[((long long)b * NM + m) * 32 + l] = make_float2(ar, ai);
  }
}

// dW[m][i][o] = sum_b conj(H[b][m][i]) dO[b][m][o]  (one block per mode).
__global__ void mix_wgrad_kernel(int B, int NM, const float2* __restrict__ H, const float2* __restrict__ dO,
                                 float2* __restrict__ dW) {
  extern __shared__ float2 hs[];  // [B][32] of H, then [B][32] of dO
  float2* ds = hs + B * 32;
  const int m = blockIdx.x;
  for (int i = threadIdx.x; i < B * 32; i += blockDim.x) {
    const int b = i >> 5, k = i & 31;
    hs[i] = H[((long long)b * NM + m) * 32 + k];
    ds[i] = dO[((long long)b * NM + m) * 32 + k];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 1024; t += blockDim.x) {
    const int i = t >> 5, o = t & 31;
    float ar = 0.f, ai = 0.f;
    for (int b = 0; b < B; ++b) {
      const float2 h = hs[b * 32 + i], d = ds[b * 32 + o];
      ar = fmaf(h.x, d.x, fmaf(h.y, d.y, ar));
      ai = fmaf(h.x, d.y, fmaf(-h.y, d.x, ai));
    }
    dW[(long long)m * 1024 + t] = make_float2(ar, ai);
  }
}

// out[r][y][c] = sum_{ky<M} s_ky (cos th Re g - sin th Im g) + sum_i P(c, i) hin[r][y][i] + bias[c],
// th = 2 pi ky y / G.
//   fwd: s_ky = (ky ? 2 : 1) / G^2, P(c, i) = pw[c][i]; z = value, h = act ? GELU(value) : value
//   bwd: s_ky = 1, P(c, i) = pw[i][c], no bias, no activation
__global__ void c2r_kernel(int G, int M, int fwd, const float2* __restrict__ Gin, const float2* __restrict__ tw,
                           const float* __restrict__ hin, const float* __restrict__ pw, const float* __restrict__ bias,
                           float* __restrict__ z_out, float* __restrict__ h_out, int act) {
  extern __shared__ float smf[];
  __shared__ float ps[32][33];
  float* hs = smf;                                        // [G][32]
  float2* gs = reinterpret_cast<float2*>(smf + G * 32);   // [M][32]
  float2* ts = gs + M * 32;                               // [G]
  const long long r = blockIdx.x;
  // The outputs y of the row are split over gridDim.y blocks; each stages
  // only its own rows of hin.
  const int y_lo = (int)(((long long)blockIdx.y * G) / gridDim.y);
  const int y_hi = (int)(((long long)(blockIdx.y + 1) * G) / gridDim.y);
  for (int i = threadIdx.x; i < (y_hi - y_lo) * 32; i += blockDim.x) hs[i] = hin[(r * G + y_lo) * 32 + i];
  for (int i = threadIdx.x; i < M * 32; i += blockDim.x) {
    float2 g = Gin[r * M * 32 + i];
    if (fwd) {
      const float s = ((i >> 5) ? 2.f : 1.f) / ((float)G * (float)G);
      g.x *= s;
      g.y *= s;
    }
    gs[i] = g;
  }
  for (int i = threadIdx.x; i < G; i += blockDim.x) ts[i] = tw[i];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
    const int a = i >> 5, bb = i & 31;
    if (fwd) ps[a][bb] = pw[i];
    else ps[bb][a] = pw[i];
  }
  __syncthreads();
  const int c = threadIdx.x & 31;
  const float bc = bias ? bias[c] : 0.f;
  // Each warp step produces kC2rRows rows: every spectral coefficient and
  // pointwise weight read from shared memory serves that many outputs.
  const int step = (blockDim.x >> 5) * kC2rRows;
  for (int y0 = y_lo + (threadIdx.x >> 5) * kC2rRows; y0 < y_hi; y0 += step) {
    float acc[kC2rRows];
#pragma unroll
    for (int q = 0; q < kC2rRows; ++q) acc[q] = bc;
    for (int ky = 0; ky < M; ++ky) {
      const float2 g = gs[ky * 32 + c];
#pragma unroll
      for (int q = 0; q < kC2rRows; ++q) {
        const float2 t = ts[(ky * (y0 + q)) & (G - 1)];
        acc[q] = fmaf(t.x, g.x, fmaf(-t.y, g.y, acc[q]));
      }
    }
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const float pc = ps[c][i];
#pragma unroll
      for (int q = 0; q < kC2rRows; ++q) {
        const int yy = min(y0 + q, y_hi - 1) - y_lo;
        acc[q] = fmaf(pc, hs[yy * 32 + i], acc[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < kC2rRows; ++q) {
      if (y0 + q < y_hi) {
        const long long o = (r * G + y0 + q) * 32 + c;
        if (z_out) z_out[o] = acc[q];
        h_out[o] = act ? gelu(acc[q]) : acc[q];
      }
    }
  }
}

// dW[o][i] += sum_p A[p][o] f(Bm[p][i]), db[o] += sum_p A[p][o]; f = GELU when
// gelu_b. CO, CI <= 128, CO * CI <= 4 * blockDim.x. Each block reduces a
// strided set of 32-point chunks in registers, then adds once atomically.
__global__ void __launch_bounds__(1024) wgrad_kernel(long long P, int CO, int CI, const float* __restrict__ A,
                                                     const float* __restrict__ Bm, int gelu_b, float* __restrict__ dW,
                                                     float* __restrict__ db) {
  __shared__ float as[kWgradChunk * 128];
  __shared__ float bs[kWgradChunk * 128];
  const int npair = CO * CI;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  float bacc = 0.f;
  for (long long p0 = (long long)blockIdx.x * kWgradChunk; p0 < P; p0 += (long long)gridDim.x * kWgradChunk) {
    const int np = (int)min((long long)kWgradChunk, P - p0);
    __syncthreads();
    for (int i = threadIdx.x; i < np * CO; i += blockDim.x) as[i] = A[p0 * CO + i];
    for (int i = threadIdx.x; i < np * CI; i += blockDim.x) {
      const float v = Bm[p0 * CI + i];
      bs[i] = gelu_b ? gelu(v) : v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int t = threadIdx.x + k * blockDim.x;
      if (t < npair) {
        const int o = t / CI, i = t - o * CI;
        float s = acc[k];
        for (int p = 0; p < np; ++p) s = fmaf(as[p * CO + o], bs[p * CI + i], s);
        acc[k] = s;
      }
    }
    if (db && (int)threadIdx.x < CO)
      for (int p = 0; p < np; ++p) bacc += as[p * CO + threadIdx.x];
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int t = threadIdx.x + k * blockDim.x;
    if (t < npair) atomicAdd(&dW[t], acc[k]);
  }
  if (db && (int)threadIdx.x < CO) atomicAdd(&db[threadIdx.x], bacc);
}

// One warp per point: u[p][j] = b1[j] + sum_i Q1[j][i] h[p][i] (j = lane + 32k),
// out[p][k] = (b2[k] + sum_j Q2[k][j] GELU(u[p][j])) * (ssq ? RMS : 1).
__global__ void proj_kernel(long long P, int PW, int GG, const float* __restrict__ h, const float* __restrict__ q1,
                            const float* __restrict__ b1, const float* __restrict__ q2, const float* __restrict__ b2,
                            const float* __restrict__ ssq, float* __restrict__ u_out, float* __restrict__ out) {
  __shared__ float q1s[128][33];
  __shared__ float b1s[128];
  __shared__ float q2s[2][128];
  for (int i = threadIdx.x; i < PW * 32; i += blockDim.x) q1s[i >> 5][i & 31] = q1[i];
  for (int i = threadIdx.x; i < PW; i += blockDim.x) {
    b1s[i] = b1[i];
    q2s[0][i] = q2[i];
    q2s[1][i] = q2[PW + i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nk = PW >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long p = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P; p += nw) {
    const float hv = h[p * 32 + lane];
    float uj[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) uj[k] = k < nk ? b1s[lane + 32 * k] : 0.f;
    for (int i = 0; i < 32; ++i) {
      const float hb = __shfl_sync(0xffffffffu, hv, i);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < nk) uj[k] = fmaf(q1s[lane + 32 * k][i], hb, uj[k]);
    }
    float o0 = 0.f, o1 = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k < nk) {
        const int j = lane + 32 * k;
        if (u_out) u_out[p * PW + j] = uj[k];
        const float a = gelu(uj[k]);
        o0 = fmaf(q2s[0][j], a, o0);
        o1 = fmaf(q2s[1][j], a, o1);
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      o0 += __shfl_xor_sync(0xffffffffu, o0, off);
      o1 += __shfl_xor_sync(0xffffffffu, o1, off);
    }
    if (lane == 0) {
      const float sc = ssq ? sqrtf(fmaxf(ssq[p / GG] / (float)GG, 1e-30f)) : 1.0f;
      out[p * 2] = (o0 + b2[0]) * sc;
      out[p * 2 + 1] = (o1 + b2[1]) * sc;
    }
  }
}

// One warp per point: du[p][j] = (sum_k Q2[k][j] dout[p][k]) GELU'(u[p][j]),
// dh[p][i] = sum_j Q1[j][i] du[p][j].
__global__ void proj_bwd_kernel(long long P, int PW, const float* __restrict__ u, const float* __restrict__ dout,
                                const float* __restrict__ q1, const float* __restrict__ q2, float* __restrict__ du,
                                float* __restrict__ dh) {
  __shared__ float q1s[128][33];
  __shared__ float q2s[2][128];
  for (int i = threadIdx.x; i < PW * 32; i += blockDim.x) q1s[i >> 5][i & 31] = q1[i];
  for (int i = threadIdx.x; i < PW; i += blockDim.x) {
    q2s[0][i] = q2[i];
    q2s[1][i] = q2[PW + i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nk = PW >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long p = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P; p += nw) {
    const float d0 = dout[p * 2], d1 = dout[p * 2 + 1];
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k < nk) {
        const int j = lane + 32 * k;
        const float v = (q2s[0][j] * d0 + q2s[1][j] * d1) * gelu_grad(u[p * PW + j]);
        du[p * PW + j] = v;
        for (int jj = 0; jj < 32; ++jj) acc = fmaf(q1s[32 * k + jj][lane], __shfl_sync(0xffffffffu, v, jj), acc);
      }
    }
    dh[p * 32 + lane] = acc;
  }
}

// sums[b][0] += |t_b|^2, sums[b][1] += |o_b - t_b|^2 (grid y = sample).
__global__ void loss_sums_kernel(long long n_per, const float* __restrict__ o, const float* __restrict__ t,
                                 float* __restrict__ sums) {
  const long long base = (long long)blockIdx.y * n_per;
  float st = 0.f, se = 0.f;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_per; i += (long long)gridDim.x * blockDim.x) {
    const float tv = t[base + i], e = o[base + i] - tv;
    st = fmaf(tv, tv, st);
    se = fmaf(e, e, se);
  }
  for (int off = 16; off > 0; off >>= 1) {
    st += __shfl_xor_sync(0xffffffffu, st, off);
    se += __shfl_xor_sync(0xffffffffu, se, off);
  }
  __shared__ float red[2][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[0][w] = st;
    red[1][w] = se;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, b = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      a += red[0][i];
      b += red[1][i];
    }
    atomicAdd(&sums[blockIdx.y * 2], a);
    atomicAdd(&sums[blockIdx.y * 2 + 1], b);
  }
}

// dout = 2 (o - t) / (B |t_b|^2); loss = mean_b |o_b - t_b|^2 / |t_b|^2.
__global__ void loss_grad_kernel(int B, long long n_per, const float* __restrict__ o, const float* __restrict__ t,
                                 const float* __restrict__ sums, float* __restrict__ dout, float* __restrict__ loss) {
  const long long n = (long long)B * n_per;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(i / n_per);
    dout[i] = 2.f * (o[i] - t[i]) / ((float)B * fmaxf(sums[2 * b], 1e-30f));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += sums[2 * b + 1] / fmaxf(sums[2 * b], 1e-30f);
    *loss = s / (float)B;
  }
}

// x[0:n) = 0.
__global__ void zero_kernel(long long n, float* __restrict__ x) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = 0.f;
}

// Adam with bias correction c1 = 1 - beta1^t, c2 = 1 - beta2^t.
__global__ void adam_kernel(long long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Training batch, pass 1: f = sum_m c_m F[s][m], t = sum_m c_m PHI[s][m]
// into the field channels and the target; ssq[b] += |f|^2 (grid y = sample).
// A scatterer index outside [0, S) gives an all-zero sample.
__global__ void superpose_kernel(int GG, int nb, int S, const float2* __restrict__ F, const float2* __restrict__ PHI,
                                 const int* __restrict__ sidx, const float2* __restrict__ coef, float* __restrict__ in,
                                 float* __restrict__ target, float* __restrict__ ssq) {
  __shared__ float2 cs[64];
  __shared__ float red[32];
  const int b = blockIdx.y;
  const int s0 = sidx[b];
  const bool valid = s0 >= 0 && s0 < S;
  const int s = valid ? s0 : 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) cs[i] = valid ? coef[b * nb + i] : make_float2(0.f, 0.f);
  __syncthreads();
  float acc = 0.f;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < GG; g += gridDim.x * blockDim.x) {
    float fr = 0.f, fi = 0.f, tr = 0.f, ti = 0.f;
    for (int m = 0; m < nb; ++m) {
      const float2 c = cs[m];
      const long long k = ((long long)s * nb + m) * GG + g;
      const float2 f = F[k], t = PHI[k];
      fr = fmaf(c.x, f.x, fmaf(-c.y, f.y, fr));
      fi = fmaf(c.x, f.y, fmaf(c.y, f.x, fi));
      tr = fmaf(c.x, t.x, fmaf(-c.y, t.y, tr));
      ti = fmaf(c.x, t.y, fmaf(c.y, t.x, ti));
    }
    const long long p = (long long)b * GG + g;
    in[p * kFnoIn + 1] = fr;
    in[p * kFnoIn + 2] = fi;
    target[p * 2] = tr;
    target[p * 2 + 1] = ti;
    acc = fmaf(fr, fr, fmaf(fi, fi, acc));
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) a += red[i];
    atomicAdd(&ssq[b], a);
  }
}

// Training batch, pass 2: unit-RMS fields and targets, the other channels.
__global__ void features_kernel(int G, int B, int S, const float* __restrict__ Q, const float* __restrict__ kap,
                                const int* __restrict__ sidx, const float* __restrict__ ssq, float* __restrict__ in,
                                float* __restrict__ target) {
  const long long GG = (long long)G * G;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * GG) return;
  const int b = (int)(t / GG);
  const int g = (int)(t - b * GG);
  const int s = sidx[b] >= 0 && sidx[b] < S ? sidx[b] : 0;
  const float sc = rsqrtf(fmaxf(ssq[b] / (float)GG, 1e-30f));
  float* x = in + t * kFnoIn;
  x[0] = Q[(long long)s * GG + g];
  x[1] *= sc;
  x[2] *= sc;
  x[3] = kap[s];
  x[4] = -1.f + (2.f * (g / G) + 1.f) / (float)G;
  x[5] = -1.f + (2.f * (g % G) + 1.f) / (float)G;
  target[t * 2] *= sc;
  target[t * 2 + 1] *= sc;
}

// ---------------------------------------------------------------------------
// The forward pass of ONE sample in one cooperative launch (the
// preconditioner's case, where 22 separate launches cost more than their
// work). The network is walked in alternating phases separated by grid-wide
// barriers:
//   row phase p (one grid row x per block): for p = 0 the lift of the row;
//     for p >= 1 the x-synthesis of the row's G1 values from the mixed
//     spectrum O of layer p-1, then the y-synthesis + pointwise path + bias
//     (+ GELU); then, while p < L, the y-DFT of the new row into H1, and at
//     p = L the projection of the row's points.
//   column phase p (one kept ky and kMixGroup kept kx per work item, so
//     that M * 2M / kMixGroup blocks share it): the x-DFT of the H1 column
//     at those kx and their per-mode channel mixing of layer p into O.
// A row needs only its own previous values and O, and a column item only
// its H1 column, so one barrier after each phase suffices (2 L in all).
// Same arithmetic as the separate kernels above, except that the DFT sums
// run as several interleaved partial sums (independent FMA chains).
struct Fwd1Args {
  int G, M, L, PW;
  const float* in;    // [G*G][6]
  const float* ssq;   // |field|^2 of the sample (may be null)
  float* out;         // [G*G][2]
  float* h;           // [G*G][32], updated row by row
  float2* H1;         // [G][M][32]
  float2* G1;         // [G][M][32]
  float2* O;          // [2M][M][32]: mixed spectrum of the layer
  const float2* tw;
  const float* lift_w;
  const float* lift_b;
  const float2* spec[8];
  const float* pw_w[8];
  const float* pw_b[8];
  const float* p1_w;
  const float* p1_b;
  const float* p2_w;
  const float* p2_b;
};

constexpr int kF1Threads = 512;
constexpr int kMixGroup = 8;  // kept kx per column work item of the fused pass

// Shared floats of the fused kernel: twiddles, then the larger of the row
// phase (two rows, a G1 row, pointwise weights, projection weights) and the
// column phase (an H1 column and two mode columns).
size_t fwd1_smem_floats(int G, int M) {
  const size_t row = 2 * (size_t)G * 32 + 2 * (size_t)M * 32 + 32 * 33 + 128 * 33 + 128 + 256;
  const size_t col = 2 * ((size_t)G * 32 + 2 * (2 * (size_t)M) * 32);
  return 2 * (size_t)G + std::max(row, col);
}

__global__ void __launch_bounds__(kF1Threads, 1) forward1_kernel(Fwd1Args a) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  extern __shared__ float smf[];
  const int G = a.G, M = a.M, L = a.L, PW = a.PW, NM2 = 2 * M;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  float2* ts = reinterpret_cast<float2*>(smf);
  float* region = smf + 2 * G;
  const float GG = (float)G * (float)G;
  const float sc_in = a.ssq ? rsqrtf(fmaxf(a.ssq[0] / GG, 1e-30f)) : 1.f;
  const float sc_out = a.ssq ? sqrtf(fmaxf(a.ssq[0] / GG, 1e-30f)) : 1.f;
  for (int i = tid; i < G; i += nt) ts[i] = a.tw[i];
  __syncthreads();
  for (int p = 0; p <= L; ++p) {
    // ---------------- row phase
    for (int r = blockIdx.x; r < G; r += gridDim.x) {
      float* hs_old = region;
      float* hs_new = region + G * 32;
      float2* gs = reinterpret_cast<float2*>(region + 2 * G * 32);
      float* ps = region + 2 * G * 32 + 2 * M * 32;  // [32][33]
      float* q1s = ps + 32 * 33;                      // [128][33]
      float* b1s = q1s + 128 * 33;
      float* q2s = b1s + 128;                         // [2][128]
      const long long row0 = (long long)r * G;
      if (p == 0) {
        for (int i = tid; i < G * 32; i += nt) {
          const int y = i >> 5, c = i & 31;
          const float* x = a.in + (row0 + y) * kFnoIn;
          float acc = a.lift_b[c];
#pragma unroll
          for (int j = 0; j < kFnoIn; ++j)
            acc = fmaf(a.lift_w[c * kFnoIn + j], (j == 1 || j == 2) ? x[j] * sc_in : x[j], acc);
          hs_new[i] = acc;
        }
      } else {
        const int l = p - 1;
        for (int i = tid; i < G * 32; i += nt) hs_old[i] = a.h[row0 * 32 + i];
        // x-synthesis of this row (x = r) from the layer's mixed spectrum:
        // two channels per thread (one 16-byte load per mode), so that the
        // M * 16 items take one round and 16 loads are in flight per thread.
        for (int i = tid; i < M * 16; i += nt) {
          const int ky = i >> 4, c2 = (i & 15) * 2;
          float ar0 = 0.f, ai0 = 0.f, ar1 = 0.f, ai1 = 0.f;
#pragma unroll 16
          for (int m = 0; m < NM2; ++m) {
            const int f = m < M ? m : G - 2 * M + m;
            const float2 t = ts[(f * r) & (G - 1)];
            const float4 v = __ldcg(reinterpret_cast<const float4*>(a.O + ((long long)m * M + ky) * 32 + c2));
            ar0 = fmaf(t.x, v.x, fmaf(-t.y, v.y, ar0));
            ai0 = fmaf(t.x, v.y, fmaf(t.y, v.x, ai0));
            ar1 = fmaf(t.x, v.z, fmaf(-t.y, v.w, ar1));
            ai1 = fmaf(t.x, v.w, fmaf(t.y, v.z, ai1));
          }
          const float sk = (ky ? 2.f : 1.f) / GG;
          gs[ky * 32 + c2] = make_float2(ar0 * sk, ai0 * sk);
          gs[ky * 32 + c2 + 1] = make_float2(ar1 * sk, ai1 * sk);
        }
        for (int i = tid; i < 1024; i += nt) ps[(i >> 5) * 33 + (i & 31)] = a.pw_w[l][i];
        if (p == L) {
          for (int i = tid; i < PW * 32; i += nt) q1s[(i >> 5) * 33 + (i & 31)] = a.p1_w[i];
          for (int i = tid; i < PW; i += nt) {
            b1s[i] = a.p1_b[i];
            q2s[i] = a.p2_w[i];
            q2s[128 + i] = a.p2_w[PW + i];
          }
        }
        __syncthreads();
        const float bc = a.pw_b[l][lane];
        const bool act = p < L;
        for (int y0 = warp * kC2rRows; y0 < G; y0 += nw * kC2rRows) {
          float acc[kC2rRows];
#pragma unroll
          for (int q = 0; q < kC2rRows; ++q) acc[q] = bc;
          for (int ky = 0; ky < M; ++ky) {
            const float2 g = gs[ky * 32 + lane];
#pragma unroll
            for (int q = 0; q < kC2rRows; ++q) {
              const float2 t = ts[(ky * (y0 + q)) & (G - 1)];
              acc[q] = fmaf(t.x, g.x, fmaf(-t.y, g.y, acc[q]));
            }
          }
#pragma unroll 8
          for (int i = 0; i < 32; ++i) {
            const float pc = ps[lane * 33 + i];
#pragma unroll
            for (int q = 0; q < kC2rRows; ++q) acc[q] = fmaf(pc, hs_old[min(y0 + q, G - 1) * 32 + i], acc[q]);
          }
#pragma unroll
          for (int q = 0; q < kC2rRows; ++q)
            if (y0 + q < G) hs_new[(y0 + q) * 32 + lane] = act ? gelu(acc[q]) : acc[q];
        }
      }
      __syncthreads();
      if (p < L) {
        for (int i = tid; i < G * 32; i += nt) a.h[row0 * 32 + i] = hs_new[i];
        for (int item = tid; item < M * 32; item += nt) {
          const int ky = item >> 5, c = item & 31;
          // four interleaved partial sums (independent FMA chains)
          float ar[4] = {0.f, 0.f, 0.f, 0.f}, ai[4] = {0.f, 0.f, 0.f, 0.f};
          for (int y = 0; y < G; y += 4) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const float2 t = ts[(ky * (y + u)) & (G - 1)];
              const float v = hs_new[(y + u) * 32 + c];
              ar[u] = fmaf(t.x, v, ar[u]);
              ai[u] = fmaf(-t.y, v, ai[u]);
            }
          }
          a.H1[((long long)r * M + ky) * 32 + c] = make_float2((ar[0] + ar[1]) + (ar[2] + ar[3]),
                                                               (ai[0] + ai[1]) + (ai[2] + ai[3]));
        }
      } else {
        const int nk = PW >> 5;
        for (int y = warp; y < G; y += nw) {
          const float hv = hs_new[y * 32 + lane];
          float uj[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) uj[k] = k < nk ? b1s[lane + 32 * k] : 0.f;
          for (int i = 0; i < 32; ++i) {
            const float hb = __shfl_sync(0xffffffffu, hv, i);
#pragma unroll
            for (int k = 0; k < 4; ++k)
              if (k < nk) uj[k] = fmaf(q1s[(lane + 32 * k) * 33 + i], hb, uj[k]);
          }
          float o0 = 0.f, o1 = 0.f;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (k < nk) {
              const float gv = gelu(uj[k]);
              o0 = fmaf(q2s[lane + 32 * k], gv, o0);
              o1 = fmaf(q2s[128 + lane + 32 * k], gv, o1);
            }
          }
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) {
            o0 += __shfl_xor_sync(0xffffffffu, o0, off);
            o1 += __shfl_xor_sync(0xffffffffu, o1, off);
          }
          if (lane == 0) {
            a.out[(row0 + y) * 2] = (o0 + a.p2_b[0]) * sc_out;
            a.out[(row0 + y) * 2 + 1] = (o1 + a.p2_b[1]) * sc_out;
          }
        }
      }
      __syncthreads();
    }
    if (p == L) break;
    grid.sync();
    // ---------------- column phase (layer p): x-DFT and mixing of one kept
    // ky for a group of kMixGroup kept kx, so that M * ceil(2M / kMixGroup)
    // blocks share the work; the x-synthesis runs in the next row phase.
    const int ngrp = (NM2 + kMixGroup - 1) / kMixGroup;
    for (int item = blockIdx.x; item < M * ngrp; item += gridDim.x) {
      const int ky = item / ngrp, m0 = (item % ngrp) * kMixGroup;
      float2* ins = reinterpret_cast<float2*>(region);   // [G][32]
      float2* part = ins + G * 32;                        // [2][kMixGroup][32]
      float2* h2s = part + 2 * kMixGroup * 32;            // [kMixGroup][32]
      for (int i = tid; i < G * 32; i += nt) ins[i] = __ldcg(a.H1 + ((long long)(i >> 5) * M + ky) * 32 + (i & 31));
      __syncthreads();
      // each output's sum over x in two halves (independent chains)
      for (int it = tid; it < 2 * kMixGroup * 32; it += nt) {
        const int half = it / (kMixGroup * 32), rem = it - half * kMixGroup * 32;
        const int mm = rem >> 5, c = rem & 31, m = m0 + mm;
        float ar[2] = {0.f, 0.f}, ai[2] = {0.f, 0.f};
        if (m < NM2) {
          const int f = m < M ? m : G - 2 * M + m;
          for (int x = half * (G >> 1); x < (half + 1) * (G >> 1); x += 2) {
#pragma unroll
            for (int u = 0; u < 2; ++u) {  // two interleaved partial sums
              const float2 t = ts[(f * (x + u)) & (G - 1)];
              const float2 v = ins[(x + u) * 32 + c];
              ar[u] = fmaf(t.x, v.x, fmaf(t.y, v.y, ar[u]));
              ai[u] = fmaf(t.x, v.y, fmaf(-t.y, v.x, ai[u]));
            }
          }
        }
        part[it] = make_float2(ar[0] + ar[1], ai[0] + ai[1]);
      }
      __syncthreads();
      for (int it = tid; it < kMixGroup * 32; it += nt) {
        const float2 u = part[it], v = part[kMixGroup * 32 + it];
        h2s[it] = make_float2(u.x + v.x, u.y + v.y);
      }
      __syncthreads();
      for (int it = tid; it < kMixGroup * 32; it += nt) {
        const int mm = it >> 5, o = it & 31, m = m0 + mm;
        if (m >= NM2) continue;
        const float2* wm = a.spec[p] + (long long)(m * M + ky) * 1024 + o;
        float ar = 0.f, ai = 0.f;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float2 v = h2s[mm * 32 + i];
          const float2 w = wm[i * 32];
          ar = fmaf(v.x, w.x, fmaf(-v.y, w.y, ar));
          ai = fmaf(v.x, w.y, fmaf(v.y, w.x, ai));
        }
        a.O[((long long)m * M + ky) * 32 + o] = make_float2(ar, ai);
      }
      __syncthreads();
    }
    grid.sync();
  }
}

// Host-side uniform numbers for the initial weights (splitmix64).
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

int wgrad_blocks(long long P) { return (int)std::min<long long>((P + kWgradChunk - 1) / kWgradChunk, 152 * 2); }

// Blocks per (sample, ky) of the x-DFT: at least enough output chunks for
// kXOut accumulators, and for a batch of one (only M blocks otherwise)
// enough to put about two blocks on every SM.
dim3 xdft_grid(int B, int M, int NO) {
  const int need = (NO + kXOut - 1) / kXOut;
  return dim3((unsigned)(B * M), (unsigned)std::max(need, std::min(NO, 304 / (B * M))));
}
// Rows of the y-transforms (B G of them) split in the same way.
dim3 row_grid(int B, int G, int most) {
  return dim3((unsigned)(B * G), (unsigned)std::max(1, std::min(most, 608 / (B * G))));
}
// Blocks of the projection kernels: at least 8 points per warp, so that
// each block's copy of the projection weights serves many points.
unsigned proj_blocks(long long P) { return (unsigned)std::min<long long>((P + 63) / 64, 152LL * 8); }

}  // namespace

void FnoLayout::build(const FnoShape& s) {
  long long o = 0;
  lift_w = o; o += kFnoWidth * kFnoIn;
  lift_b = o; o += kFnoWidth;
  spec.clear(); pw_w.clear(); pw_b.clear();
  for (int l = 0; l < s.layers; ++l) {
    spec.push_back(o); o += 2LL * (2 * s.modes) * s.modes * kFnoWidth * kFnoWidth;
    pw_w.push_back(o); o += kFnoWidth * kFnoWidth;
    pw_b.push_back(o); o += kFnoWidth;
  }
  p1_w = o; o += (long long)s.proj * kFnoWidth;
  p1_b = o; o += s.proj;
  p2_w = o; o += (long long)kFnoOut * s.proj;
  p2_b = o; o += kFnoOut;
  total = o;
}

bool FnoNet::init(int dev, const FnoShape& s, unsigned long long seed, std::string& err) {
  const int G = s.grid;
  if (G < 8 || G > 256 || (G & (G - 1))) { err = "grid must be a power of two in [8, 256]"; return false; }
  if (s.modes < 1 || s.modes > 32 || 2 * s.modes > G) { err = "modes must be in [1, 32] with 2 * modes <= grid"; return false; }
  if (s.layers < 1 || s.layers > 8) { err = "layers must be in [1, 8]"; return false; }
  if (s.proj < 32 || s.proj > 128 || s.proj % 32) { err = "proj_width must be 32, 64, 96 or 128"; return false; }
  device = dev;
  shape = s;
  lay.build(s);
  cudaError_t e = cudaSetDevice(dev);
  const size_t pb = (size_t)lay.total * sizeof(float);
  if (e == cudaSuccess) e = cudaMalloc(&params, pb);
  if (e == cudaSuccess) e = cudaMalloc(&grads, pb);
  if (e == cudaSuccess) e = cudaMalloc(&adam_m, pb);
  if (e == cudaSuccess) e = cudaMalloc(&adam_v, pb);
  if (e == cudaSuccess) e = cudaMalloc(&tw, (size_t)G * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&loss, sizeof(float));
  if (e != cudaSuccess) {
    err = std::string("device allocation: ") + cudaGetErrorString(e);
    release();
    return false;
  }
  // Initial weights: linear layers U(-1/sqrt(fan_in), 1/sqrt(fan_in)) for
  // weights and biases; spectral weights (1 / 32^2) U[0, 1) per part.
  std::vector<float> p((size_t)lay.total);
  Rng rng(seed);
  auto fill = [&](long long off, long long n, double lo, double hi) {
    for (long long i = 0; i < n; ++i) p[(size_t)(off + i)] = (float)(lo + (hi - lo) * rng.uniform());
  };
  const double bl = 1.0 / std::sqrt((double)kFnoIn), bw = 1.0 / std::sqrt((double)kFnoWidth),
               bp = 1.0 / std::sqrt((double)s.proj);
  fill(lay.lift_w, kFnoWidth * kFnoIn, -bl, bl);
  fill(lay.lift_b, kFnoWidth, -bl, bl);
  const long long nspec = 2LL * (2 * s.modes) * s.modes * kFnoWidth * kFnoWidth;
  for (int l = 0; l < s.layers; ++l) {
    fill(lay.spec[l], nspec, 0.0, 1.0 / (kFnoWidth * kFnoWidth));
    fill(lay.pw_w[l], kFnoWidth * kFnoWidth, -bw, bw);
    fill(lay.pw_b[l], kFnoWidth, -bw, bw);
  }
  fill(lay.p1_w, (long long)s.proj * kFnoWidth, -bw, bw);
  fill(lay.p1_b, s.proj, -bw, bw);
  fill(lay.p2_w, (long long)kFnoOut * s.proj, -bp, bp);
  fill(lay.p2_b, kFnoOut, -bp, bp);
  std::vector<float2> t(G);
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < G; ++k) t[k] = make_float2((float)std::cos(2 * pi * k / G), (float)std::sin(2 * pi * k / G));
  e = cudaMemcpy(params, p.data(), pb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(tw, t.data(), (size_t)G * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(adam_m, 0, pb);
  if (e == cudaSuccess) e = cudaMemset(adam_v, 0, pb);
  if (e == cudaSuccess) e = cudaMemset(grads, 0, pb);
  // The uploads and clears above run on the default stream; the net's
  // kernels may run on any other.
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    err = std::string("device upload: ") + cudaGetErrorString(e);
    release();
    return false;
  }
  adam_t = 0;
  return true;
}

void FnoNet::release() {
  for (float* p : h) cudaFree(p);
  for (float* p : z) cudaFree(p);
  for (float2* p : H2) cudaFree(p);
  h.clear(); z.clear(); H2.clear();
  cudaFree(H1); cudaFree(O); cudaFree(G1); cudaFree(u); cudaFree(out); cudaFree(dout); cudaFree(dz);
  cudaFree(dh0); cudaFree(dh1); cudaFree(du); cudaFree(sums);
  H1 = O = G1 = nullptr;
  u = out = dout = dz = dh0 = dh1 = du = sums = nullptr;
  cap = 0;
  ++generation;
  cudaFree(params); cudaFree(grads); cudaFree(adam_m); cudaFree(adam_v); cudaFree(tw); cudaFree(loss);
  params = grads = adam_m = adam_v = loss = nullptr;
  tw = nullptr;
}

cudaError_t FnoNet::ensure(int batch) {
  if (batch <= cap) return cudaSuccess;
  ++generation;
  for (float* p : h) cudaFree(p);
  for (float* p : z) cudaFree(p);
  for (float2* p : H2) cudaFree(p);
  h.clear(); z.clear(); H2.clear();
  cudaFree(H1); cudaFree(O); cudaFree(G1); cudaFree(u); cudaFree(out); cudaFree(dout); cudaFree(dz);
  cudaFree(dh0); cudaFree(dh1); cudaFree(du); cudaFree(sums);
  cap = 0;
  const int G = shape.grid, M = shape.modes, L = shape.layers;
  const long long P = (long long)batch * G * G;
  const size_t act = (size_t)P * kFnoWidth * sizeof(float);
  const size_t spec = (size_t)batch * 2 * M * M * kFnoWidth * sizeof(float2);
  const size_t ygrid = (size_t)batch * G * M * kFnoWidth * sizeof(float2);
  cudaError_t e = cudaSuccess;
  h.assign(L + 1, nullptr);
  z.assign(L, nullptr);
  H2.assign(L, nullptr);
  for (int l = 0; l <= L && e == cudaSuccess; ++l) e = cudaMalloc(&h[l], act);
  for (int l = 0; l < L && e == cudaSuccess; ++l) e = cudaMalloc(&z[l], act);
  for (int l = 0; l < L && e == cudaSuccess; ++l) e = cudaMalloc(&H2[l], spec);
  if (e == cudaSuccess) e = cudaMalloc(&H1, ygrid);
  if (e == cudaSuccess) e = cudaMalloc(&G1, ygrid);
  if (e == cudaSuccess) e = cudaMalloc(&O, spec);
  if (e == cudaSuccess) e = cudaMalloc(&u, (size_t)P * shape.proj * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&du, (size_t)P * shape.proj * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&out, (size_t)P * kFnoOut * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)P * kFnoOut * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dz, act);
  if (e == cudaSuccess) e = cudaMalloc(&dh0, act);
  if (e == cudaSuccess) e = cudaMalloc(&dh1, act);
  if (e == cudaSuccess) e = cudaMalloc(&sums, (size_t)batch * 2 * sizeof(float));
  if (e == cudaSuccess) cap = batch;
  return e;
}

cudaError_t FnoNet::forward(int B, const float* in, float* outp, const float* ssq, cudaStream_t s) {
  if (B == 1 && fused_ok()) {
    const cudaError_t e = forward1(in, outp, ssq, s);
    if (e == cudaSuccess) return e;
    cudaGetLastError();  // not launchable here: separate kernels
    fused = -1;
  }
  return forward_layers(B, in, outp, ssq, s);
}

bool FnoNet::fused_ok() {
  if (fused == 0) {
    int coop = 0, nsm = 0, per_sm = 0;
    const size_t smem = fwd1_smem_floats(shape.grid, shape.modes) * sizeof(float);
    fused = -1;
    if (shape.grid <= 128 && shape.layers <= 8 && shape.proj <= 128 &&
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) == cudaSuccess && coop &&
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) == cudaSuccess &&
        raise_smem_limit((const void*)forward1_kernel, (int)smem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, forward1_kernel, kF1Threads, smem) == cudaSuccess &&
        per_sm >= 1) {
      fused_blocks = nsm * per_sm;
      fused = 1;
    }
    cudaGetLastError();
  }
  return fused == 1;
}

cudaError_t FnoNet::forward1(const float* in, float* outp, const float* ssq, cudaStream_t s) {
  cudaError_t e = ensure(1);
  if (e != cudaSuccess) return e;
  Fwd1Args a = {};
  a.G = shape.grid;
  a.M = shape.modes;
  a.L = shape.layers;
  a.PW = shape.proj;
  a.in = in;
  a.ssq = ssq;
  a.out = outp;
  a.h = h[0];
  a.H1 = H1;
  a.G1 = G1;
  a.O = O;
  a.tw = tw;
  a.lift_w = params + lay.lift_w;
  a.lift_b = params + lay.lift_b;
  for (int l = 0; l < shape.layers; ++l) {
    a.spec[l] = reinterpret_cast<const float2*>(params + lay.spec[l]);
    a.pw_w[l] = params + lay.pw_w[l];
    a.pw_b[l] = params + lay.pw_b[l];
  }
  a.p1_w = params + lay.p1_w;
  a.p1_b = params + lay.p1_b;
  a.p2_w = params + lay.p2_w;
  a.p2_b = params + lay.p2_b;
  void* args[] = {&a};
  const size_t smem = fwd1_smem_floats(shape.grid, shape.modes) * sizeof(float);
  // one block per grid row and per column work item (a kept ky and a group of kMixGroup kept kx)
  const int col_items = shape.modes * ((2 * shape.modes + kMixGroup - 1) / kMixGroup);
  const int blocks = std::min(fused_blocks, std::max(shape.grid, col_items));
  launches = 1;
  return cudaLaunchCooperativeKernel((const void*)forward1_kernel, dim3((unsigned)blocks), dim3(kF1Threads), args,
                                     smem, s);
}

cudaError_t FnoNet::forward_layers(int B, const float* in, float* outp, const float* ssq, cudaStream_t s) {
  if (B < 1 || B > kFnoMaxBatch) return cudaErrorInvalidValue;
  cudaError_t e = ensure(B);
  if (e != cudaSuccess) return e;
  const int G = shape.grid, M = shape.modes, L = shape.layers, NM = 2 * M * M;
  const long long GG = (long long)G * G, P = B * GG;
  const float* w = params;
  launches = 0;
  lift_kernel<<<(unsigned)((P * kFnoWidth + 255) / 256), 256, 0, s>>>(P, (int)GG, in, w + lay.lift_w, w + lay.lift_b, ssq, h[0]);
  ++launches;
  const size_t sm_r2c = (size_t)G * 32 * sizeof(float) + (size_t)G * sizeof(float2);
  const size_t sm_c2r = (size_t)G * 32 * sizeof(float) + (size_t)M * 32 * sizeof(float2) + (size_t)G * sizeof(float2);
  const dim3 rg = row_grid(B, G, 2);
  const int r2c_threads = 32 * std::min(32, (M + (int)rg.y - 1) / (int)rg.y);
  for (int l = 0; l < L; ++l) {
    r2c_kernel<<<rg, r2c_threads, sm_r2c, s>>>(G, M, 0, h[l], nullptr, nullptr, tw, H1);
    xdft_kernel<<<xdft_grid(B, M, 2 * M), kXWarps * 32, 0, s>>>(G, M, 1, H1, tw, H2[l]);
    mix_kernel<<<(unsigned)NM, 256, (size_t)B * 32 * sizeof(float2), s>>>(B, NM, 0, H2[l], reinterpret_cast<const float2*>(w + lay.spec[l]), O);
    xdft_kernel<<<xdft_grid(B, M, G), kXWarps * 32, 0, s>>>(G, M, 0, O, tw, G1);
    c2r_kernel<<<row_grid(B, G, 4), 256, sm_c2r, s>>>(G, M, 1, G1, tw, h[l], w + lay.pw_w[l], w + lay.pw_b[l], z[l], h[l + 1], l + 1 < L ? 1 : 0);
    launches += 5;
  }
  const unsigned pblocks = proj_blocks(P);
  proj_kernel<<<pblocks, 256, 0, s>>>(P, shape.proj, (int)GG, h[L], w + lay.p1_w, w + lay.p1_b, w + lay.p2_w, w + lay.p2_b, ssq, ssq ? nullptr : u, outp);
  ++launches;
  return cudaGetLastError();
}

cudaError_t FnoNet::loss_grad(int B, const float* in, const float* target, cudaStream_t s) {
  if (B < 1 || B > kFnoMaxBatch) return cudaErrorInvalidValue;
  cudaError_t e = ensure(B);
  if (e == cudaSuccess) e = forward_layers(B, in, out, nullptr, s);  // keeps what the backward pass reads
  if (e != cudaSuccess) return e;
  const int G = shape.grid, M = shape.modes, L = shape.layers, NM = 2 * M * M, PW = shape.proj;
  const long long GG = (long long)G * G, P = B * GG;
  const float* w = params;
  float* gw = grads;
  zero_kernel<<<(unsigned)std::min<long long>((lay.total + 255) / 256, 152LL * 8), 256, 0, s>>>(lay.total, grads);
  zero_kernel<<<1, 256, 0, s>>>((long long)B * 2, sums);
  // Loss and its gradient with respect to the outputs.
  const long long n_per = GG * kFnoOut;
  loss_sums_kernel<<<dim3((unsigned)std::min<long long>((n_per + 255) / 256, 64), (unsigned)B), 256, 0, s>>>(n_per, out, target, sums);
  loss_grad_kernel<<<(unsigned)std::min<long long>((B * n_per + 255) / 256, 152LL * 8), 256, 0, s>>>(B, n_per, out, target, sums, dout, loss);
  // Projection.
  const unsigned pblocks = proj_blocks(P);
  const unsigned wb = (unsigned)wgrad_blocks(P);
  proj_bwd_kernel<<<pblocks, 256, 0, s>>>(P, PW, u, dout, w + lay.p1_w, w + lay.p2_w, du, dh0);
  wgrad_kernel<<<wb, 1024, 0, s>>>(P, kFnoOut, PW, dout, u, 1, gw + lay.p2_w, gw + lay.p2_b);
  wgrad_kernel<<<wb, 1024, 0, s>>>(P, PW, kFnoWidth, du, h[L], 0, gw + lay.p1_w, gw + lay.p1_b);
  // Fourier layers, last to first. dhA = dL/dh[l + 1] on entry.
  const size_t sm_r2c = (size_t)G * 32 * sizeof(float) + (size_t)G * sizeof(float2);
  const size_t sm_c2r = (size_t)G * 32 * sizeof(float) + (size_t)M * 32 * sizeof(float2) + (size_t)G * sizeof(float2);
  const dim3 rg = row_grid(B, G, 2);
  const int r2c_threads = 32 * std::min(32, (M + (int)rg.y - 1) / (int)rg.y);
  float* dhA = dh0;
  float* dhB = dh1;
  for (int l = L - 1; l >= 0; --l) {
    // dz = dL/dz[l] (GELU backward fused into the staging of the y-DFT
    // adjoint; the last layer has no activation), then dG1 = c2r^T dz.
    const float* dzl;
    if (l + 1 < L) {
      r2c_kernel<<<rg, r2c_threads, sm_r2c, s>>>(G, M, 1, dhA, z[l], dz, tw, H1);
      dzl = dz;
    } else {
      r2c_kernel<<<rg, r2c_threads, sm_r2c, s>>>(G, M, 1, dhA, nullptr, nullptr, tw, H1);
      dzl = dhA;
    }
    wgrad_kernel<<<wb, 1024, 0, s>>>(P, kFnoWidth, kFnoWidth, dzl, h[l], 0, gw + lay.pw_w[l], gw + lay.pw_b[l]);
    xdft_kernel<<<xdft_grid(B, M, 2 * M), kXWarps * 32, 0, s>>>(G, M, 1, H1, tw, O);  // dO = idft_x^T dG1
    mix_wgrad_kernel<<<(unsigned)NM, 256, (size_t)2 * B * 32 * sizeof(float2), s>>>(B, NM, H2[l], O, reinterpret_cast<float2*>(gw + lay.spec[l]));
    mix_kernel<<<(unsigned)NM, 256, (size_t)B * 32 * sizeof(float2), s>>>(B, NM, 1, O, reinterpret_cast<const float2*>(w + lay.spec[l]), H2[l]);  // dH2 (H2[l] no longer needed)
    xdft_kernel<<<xdft_grid(B, M, G), kXWarps * 32, 0, s>>>(G, M, 0, H2[l], tw, G1);  // dH1 = dft_x^T dH2
    // dh[l] = r2c^T dH1 + Wpw^T dz
    c2r_kernel<<<row_grid(B, G, 4), 256, sm_c2r, s>>>(G, M, 0, G1, tw, dzl, w + lay.pw_w[l], nullptr, nullptr, dhB, 0);
    std::swap(dhA, dhB);
  }
  wgrad_kernel<<<wb, 1024, 0, s>>>(P, kFnoWidth, kFnoIn, dhA, in, 0, gw + lay.lift_w, gw + lay.lift_b);
  return cudaGetLastError();
}

cudaError_t FnoNet::adam(float lr, float beta1, float beta2, float eps, cudaStream_t s) {
  ++adam_t;
  const float c1 = 1.f - (float)std::pow((double)beta1, adam_t);
  const float c2 = 1.f - (float)std::pow((double)beta2, adam_t);
  const long long n = lay.total;
  const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 8);
  adam_kernel<<<blocks, 256, 0, s>>>(n, params, grads, adam_m, adam_v, lr, beta1, beta2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t fno_make_batch(int G, int B, int nb, int S, const float2* F, const float2* PHI, const float* Q,
                           const float* kap, const int* sidx, const float2* coef, float* in, float* target, float* ssq,
                           cudaStream_t s) {
  if (B < 1 || nb < 1 || nb > 64 || S < 1) return cudaErrorInvalidValue;
  const int GG = G * G;
  zero_kernel<<<1, 256, 0, s>>>((long long)B, ssq);
  superpose_kernel<<<dim3((unsigned)std::min((GG + 255) / 256, 64), (unsigned)B), 256, 0, s>>>(GG, nb, S, F, PHI, sidx, coef, in, target, ssq);
  features_kernel<<<(unsigned)(((long long)B * GG + 255) / 256), 256, 0, s>>>(G, B, S, Q, kap, sidx, ssq, in, target);
  return cudaGetLastError();
}

}  // namespace lsg
