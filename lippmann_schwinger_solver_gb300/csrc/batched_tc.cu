// The FP32 operator applied to 64 right-hand sides at once on the
// tensor cores (tcgen05, sm_103a).
//
// With many right-hand sides every block of the DAFMM becomes a dense
// contraction: a node's output rows are  out[n][j] = sum_k A[n][k] x[idx[k]][j]
// for the 64 columns j of the block of right-hand sides. One MMA tile is
//
//   D[m][n] = sum_k' Xop[m][k'] Aop[n][k']      (M = 128, N = block rows)
//
// with the complex product written in real arithmetic: row m = j < 64 of
// Xop holds (Re x, Im x) of right-hand side j, row 64 + j holds (Im x,
// -Re x), and row n of Aop holds (Re A, -Im A) of the block row, so that
// D[j][n] = Re(A x)[n][j] and D[64 + j][n] = Im(A x)[n][j]. The operator
// operand is stored once per phase in the MMA's canonical shared-memory
// layout (K-major, no swizzle: 8-row core matrices of 16-byte K slices,
// 128 bytes apart along K, 1024 bytes apart along the rows), one stage of
// 16 complex columns after another, so that staging it is a linear copy.
//
// Precision: FP32 operands through TF32 tensor cores in three products,
// hi*hi + hi*lo + lo*hi with hi a value rounded to TF32 and lo the
// FP32 remainder (lo*lo, about 2^-22 relative, is dropped). The tensor
// core's FP32 accumulation is not round-to-nearest over long sums (measured:
// 3x the error of the CUDA-core FP32 form on blocks of ~1,000 columns), so
// each accumulator covers kChunkStages stages (128 real columns) and is then
// added to running FP32 sums (round-to-nearest) that are also kept in tensor
// memory, next to the two accumulator slots, which alternate so that the
// tensor core keeps working while a slot is read.
//
// Two kernels implement this: tc_ws_kernel (the default, described at its
// definition: one CTA per SM with loader, converter, MMA and epilogue warps
// fed by a per-CTA stage program) and tc_gemm_kernel (LS_TC_WS=0).
//
// Kernel structure (tc_gemm_kernel): a persistent grid of two CTAs per SM, 128 threads per CTA
// (four warps, one per 32-lane quarter of tensor memory). Blocks of the
// phase are dealt round-robin. Per block the K columns are walked in stages
// of 16 complex columns through two shared-memory buffers: all threads
// gather the 64-wide source rows (split hi/lo, two MMA rows per value) and
// copy the operator stage (split hi/lo), with the loads of the next two
// stages in flight; one thread issues the 12 MMAs of a stage (4 K-steps x 3
// products) and commits them to the buffer's mbarrier, which the threads
// wait on before they refill that buffer two stages later. The last stage
// of a chunk is also committed to its accumulator slot's mbarrier; before a
// slot is reused the four warps read it out of tensor memory (tcgen05.ld
// 32x32b, each warp its 32 lanes) and add it to the sums (tcgen05.st).
// After the last chunk they write, add to, or combine the sums into the
// destination, eight rows at a time with their loads batched. Every mbarrier wait is bounded; a wait that gives up sets
// the error flag, the CTA skips its remaining work and still frees its
// tensor memory.

#include <cuda_runtime.h>

#include <algorithm>
#include <queue>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "device.h"
#include "launch.h"

namespace lsg {

namespace {

constexpr int kTcThreads = 128;
constexpr int kStageCols = 16;                 // complex columns per stage (32 reals, 128 bytes per row)
constexpr int kRowGroupBytes = 8 * 128;        // stride between 8-row core-matrix groups (SBO)
constexpr int kXBytes = 128 * 128;             // one plane (hi or lo) of the 128-row operand
constexpr long long kWaitLimit = 20000000;     // mbarrier polls before a wait gives up
constexpr int kMaxRows = 64;                   // block rows per MMA tile (N <= 64; larger blocks are split)
constexpr int kChunkStages = 4;                // stages accumulated in tensor memory before promotion
constexpr int kSumCol = 2 * kMaxRows;          // tensor-memory columns of the running FP32 sums
constexpr int kTmemCols = 256;                 // two accumulator slots and the sums (a power of two)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading (K) and stride (row
// group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Shared-memory matrix descriptor of a K-major operand in the 128-byte
// swizzle layout: 128-byte rows, 8-row atoms of 1024 bytes (SBO), the
// 16-byte chunk c of row r stored at chunk c ^ (r & 7); descriptor version
// 1, layout type 2 (128-byte swizzle). A K-step starts 32 bytes further
// into the rows of the atom.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;               // LBO (unused by swizzled K-major operands)
  d |= (uint64_t)(1024 >> 4) << 32;     // SBO
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Float2 index of (row, complex column cc) of a stage plane in the 128-byte
// swizzle layout (one 128-byte row = the stage's 16 complex columns).
__host__ __device__ __forceinline__ int canon_sw128(int row, int cc) {
  return ((row >> 3) * 1024 + (row & 7) * 128 + ((((cc >> 1) ^ (row & 7))) << 4) + (cc & 1) * 8) >> 3;
}

// Float2 index of (row, complex column cc) inside one stage plane.
__host__ __device__ __forceinline__ int canon(int row, int cc) {
  return ((row & 7) * 16 + (row >> 3) * kRowGroupBytes + (cc >> 1) * 128 + (cc & 1) * 8) >> 3;
}

// v rounded to the nearest TF32 value (10 explicit mantissa bits; ties away
// from zero). Both parts of the split are rounded, so that the tensor
// core's truncation of its TF32 inputs changes neither: v - hi - lo is then
// below 2^-22 |v|.
__device__ __forceinline__ float tf32_rn(float v) {
  return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile("{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }" ::
                   "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, uint32_t parity, long long limit) {
  uint32_t done = 0;
  for (long long it = 0; it < limit && !done; ++it)
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
  return done != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) { return mbar_wait_n(bar, parity, kWaitLimit); }

}  // namespace

// One block of a phase in tensor-core form.
struct TcBlock {
  long long a_off;  // first float2 of the block's operator stages (stage s at a_off + s * npad * 16)
  int i_off;        // gather list: column k at idx[i_off + k]
  int o_off;        // output rows: row n at out[o_off + n]
  int rows;         // block rows (<= npad <= kMaxRows)
  int npad;         // rows padded to a multiple of 16 (MMA N)
  int K;            // complex columns
  int nst;          // stages of kStageCols columns
};

// One stage of a CTA's stage program (80 bytes): what the loader of
// tc_ws_kernel copies for it and how the stage sits in its block.
struct TcStage {
  int rows[16];  // gather source row of each column (ncols used)
  int a256;      // first float2 of the operator stage / 256
  int ncols;     // columns present (1..16)
  int npad;      // block rows padded to a multiple of 16
  int flags;     // 1: first stage of an accumulator chunk, 2: last stage of a chunk
};
static_assert(sizeof(TcStage) == 80, "stage record");

namespace {

// mode 0: dst rows = D; 1: dst rows += D; 2 (near field and output):
// y = P + s D + x with s = kappa^2 q of the row (find_phi) or 1.
__global__ void __launch_bounds__(kTcThreads, 2)
    tc_gemm_kernel(const TcBlock* __restrict__ blocks, int n_blocks, const float2* __restrict__ A,
                   const int* __restrict__ idx, const int* __restrict__ out, const float2* __restrict__ src,
                   float2* __restrict__ dst, int mode, const float2* __restrict__ P, const float* __restrict__ kq,
                   int find_phi, int npad_max, unsigned* __restrict__ err) {
  pdl_enter();
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bar[2];     // per stage buffer: its MMAs completed
  __shared__ uint64_t accbar[2];  // per accumulator slot: its chunk completed
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ int orows[kMaxRows];  // the current block's output rows
  const int t = threadIdx.x, warp = t >> 5;
  const int a_plane = npad_max * 128;               // bytes of one operator plane
  const int buf_bytes = 2 * kXBytes + 2 * a_plane;  // Xh, Xl, Ah, Al
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar[0])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar[1])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&accbar[0])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&accbar[1])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  // M = 128, N = npad (set per block), A and B K-major, TF32 inputs, FP32 accumulator.
  const uint32_t idesc_base = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(128 >> 4) << 24);
  // The gather mapping of a thread: 16-thread groups cover one 8-row x
  // 2-column core-matrix slice per step, so their shared stores hit 32
  // distinct banks; their loads are 2 x 64 contiguous bytes.
  const int l16 = t & 15, hw = t >> 4, j8 = l16 & 7, cpar = l16 >> 3;
  long long g = 0;   // stages issued by this CTA (buffer g & 1, use g >> 1)
  long long gc = 0;  // chunks issued by this CTA (accumulator slot gc & 1, use gc >> 1)
  // The running FP32 sums of a block live in tensor memory next to the two
  // accumulator slots (columns kSumCol + n, this thread's lane), which
  // leaves the registers to the loads in flight.
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  auto tld8 = [&](uint32_t col, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(lane_base + col));
  };
  // sums[n] (+)= the accumulator slot's column n, round-to-nearest FP32;
  // the first chunk of a block sets the sums.
  auto promote = [&](int slot, int npad, bool first) {
#pragma unroll
    for (int c0 = 0; c0 < kMaxRows; c0 += 8) {
      if (c0 < npad) {
        uint32_t r[8], q[8];
        tld8((uint32_t)(slot * kMaxRows + c0), r);
        if (!first) tld8((uint32_t)(kSumCol + c0), q);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (!first) {
#pragma unroll
          for (int i = 0; i < 8; ++i) r[i] = __float_as_uint(__uint_as_float(q[i]) + __uint_as_float(r[i]));
        }
        asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(
                         lane_base + (uint32_t)(kSumCol + c0)),
                     "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
                     : "memory");
      }
    }
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  };
  for (int b = blockIdx.x; b < n_blocks; b += gridDim.x) {
    const TcBlock blk = blocks[b];
    const uint32_t idesc = idesc_base | ((uint32_t)(blk.npad >> 3) << 17);
    const long long gc0 = gc;
    // Output rows of the block, loaded now so that they have arrived by the
    // epilogue (the barriers of the stage loop order the shared stores before
    // their reads there).
    if (t < blk.rows) orows[t] = __ldg(out + blk.o_off + t);
    const int nchunks = (blk.nst + kChunkStages - 1) / kChunkStages;
    // Loads of stage st: 8 gathered right-hand-side values and up to 4
    // operator vectors per thread. The loads of stages st + 1 and st + 2 are
    // in flight while stage st is stored (x0/a0: stage st, x1/a1: st + 1,
    // x2/a2: st + 2), and the gather indices are loaded a stage earlier
    // still (ix: stage st + 3), so the dependent index load is off the
    // critical path.
    float2 x0[8], x1[8], x2[8];
    float4 a0[4], a1[4], a2[4];
    int ix[8];  // gather sources of a stage not yet loaded (-1: past K)
    auto load_idx = [&](int st, int* ixp) {
      const int k0 = st * kStageCols;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int ci = hw * 8 + i;
        const int k = k0 + 2 * (ci >> 3) + cpar;
        ixp[i] = k < blk.K ? __ldg(idx + blk.i_off + k) : -1;
      }
    };
    auto load_stage = [&](int st, const int* ixp, float2* x, float4* a) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int ci = hw * 8 + i;
        const int jj = (ci & 7) * 8 + j8;
        x[i] = ixp[i] >= 0 ? ld_chain(src + (size_t)ixp[i] * 64 + jj) : make_float2(0.f, 0.f);
      }
      // npad rows x 16 complex columns in the canonical layout: npad * 8 <= 512 float4.
      const float4* As = reinterpret_cast<const float4*>(A + blk.a_off + (long long)st * blk.npad * kStageCols);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int u = t + q * kTcThreads;
        a[q] = u < blk.npad * 8 ? __ldcs(As + u) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    };
    if (blk.nst > 0) {
      load_idx(0, ix);
      load_stage(0, ix, x0, a0);
    }
    if (blk.nst > 1) {
      load_idx(1, ix);
      load_stage(1, ix, x1, a1);
    }
    if (blk.nst > 2) load_idx(2, ix);
    for (int st = 0; st < blk.nst; ++st, ++g) {
      const int buf = (int)(g & 1);
      const long long G = gc0 + st / kChunkStages;  // chunk of this stage
      const bool chunk_start = st % kChunkStages == 0;
      const bool chunk_end = st % kChunkStages == kChunkStages - 1 || st == blk.nst - 1;
      uint8_t* base = smem + buf * buf_bytes;
      float2* Xh = reinterpret_cast<float2*>(base);
      float2* Xl = reinterpret_cast<float2*>(base + kXBytes);
      float4* Ah = reinterpret_cast<float4*>(base + 2 * kXBytes);
      float4* Al = reinterpret_cast<float4*>(base + 2 * kXBytes + a_plane);
      if (st + 2 < blk.nst) load_stage(st + 2, ix, x2, a2);
      if (st + 3 < blk.nst) load_idx(st + 3, ix);
      if (g >= 2 && !mbar_wait(&bar[buf], (uint32_t)(((g >> 1) - 1) & 1))) {
        atomicOr(err, 1u);
        abort_flag = 1;
      }
      __syncthreads();
      if (abort_flag) break;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int ci = hw * 8 + i;
        const int jj = (ci & 7) * 8 + j8, cc = 2 * (ci >> 3) + cpar;
        const float2 v = x0[i];
        const float hx = tf32_rn(v.x), hy = tf32_rn(v.y);
        const float lx = tf32_rn(v.x - hx), ly = tf32_rn(v.y - hy);
        const int o_re = canon(jj, cc), o_im = canon(64 + jj, cc);
        Xh[o_re] = make_float2(hx, hy);
        Xl[o_re] = make_float2(lx, ly);
        Xh[o_im] = make_float2(hy, -hx);
        Xl[o_im] = make_float2(ly, -lx);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int u = t + q * kTcThreads;
        if (u < blk.npad * 8) {
          const float4 v = a0[q];
          const float4 h = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
          Ah[u] = h;
          Al[u] = make_float4(tf32_rn(v.x - h.x), tf32_rn(v.y - h.y), tf32_rn(v.z - h.z), tf32_rn(v.w - h.w));
        }
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        x0[i] = x1[i];
        x1[i] = x2[i];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a0[q] = a1[q];
        a1[q] = a2[q];
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      // Slot G & 1 still holds chunk G - 2 of this block: add it to the
      // registers before the slot is reused (its commit is the slot's latest).
      if (chunk_start && G - 2 >= gc0) {
        if (!mbar_wait(&accbar[G & 1], (uint32_t)(((G - 2) >> 1) & 1))) {
          atomicOr(err, 1u);
          abort_flag = 1;
        } else {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          promote((int)(G & 1), blk.npad, G - 2 == gc0);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (abort_flag) break;
      if (t == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t xh = smem_u32(Xh), xl = smem_u32(Xl), ah = smem_u32(Ah), al = smem_u32(Al);
        const uint32_t dt = tmem + (uint32_t)((G & 1) * kMaxRows);
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint32_t o = ks * 256;
          const uint64_t dxh = sdesc(xh + o, 128, kRowGroupBytes), dxl = sdesc(xl + o, 128, kRowGroupBytes);
          const uint64_t dah = sdesc(ah + o, 128, kRowGroupBytes), dal = sdesc(al + o, 128, kRowGroupBytes);
          mma_tf32(dt, dxh, dah, idesc, (!chunk_start || ks > 0) ? 1u : 0u);
          mma_tf32(dt, dxh, dal, idesc, 1u);
          mma_tf32(dt, dxl, dah, idesc, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&bar[buf]))
                     : "memory");
        if (chunk_end)
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&accbar[G & 1]))
                       : "memory");
      }
    }
    if (abort_flag) break;
    gc = gc0 + nchunks;
    // The last one or two chunks are still in tensor memory.
    for (long long G = (gc - 2 > gc0 ? gc - 2 : gc0); G < gc; ++G) {
      if (!mbar_wait(&accbar[G & 1], (uint32_t)((G >> 1) & 1))) {
        atomicOr(err, 1u);
        abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      promote((int)(G & 1), blk.npad, G == gc0);
    }
    __syncthreads();
    if (abort_flag) break;
    // Epilogue, eight rows at a time: their output indices and old values
    // are all loaded before any of them is written (the rows of a phase are
    // distinct), so a group costs one round trip, not eight.
    const int m = t, part = m >> 6, j = m & 63;
    float* dstf = reinterpret_cast<float*>(dst);
    for (int c0 = 0; c0 < blk.rows; c0 += 8) {
      uint32_t r[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};  // a block without columns sums to zero
      if (nchunks > 0) tld8((uint32_t)(kSumCol + c0), r);
      size_t e[8];
      float base[8], extra[8], scale[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int orow = c0 + i < blk.rows ? orows[c0 + i] : 0;
        e[i] = ((size_t)orow * 64 + j) * 2 + part;
        scale[i] = (mode == 2 && find_phi) ? __ldg(kq + orow) : 1.f;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        base[i] = extra[i] = 0.f;
        if (c0 + i < blk.rows) {
          if (mode == 1) {
            base[i] = ld_chain(dstf + e[i]);
          } else if (mode == 2) {
            base[i] = ld_chain(reinterpret_cast<const float*>(P) + e[i]);
            if (find_phi) extra[i] = ld_chain(reinterpret_cast<const float*>(src) + e[i]);
          }
        }
      }
      if (nchunks > 0) asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (c0 + i >= blk.rows) break;
        const float v = __uint_as_float(r[i]);
        // mode 0: v; mode 1: old + v; mode 2: P + s v, + x with find_phi
        if (mode == 0)
          dstf[e[i]] = v;
        else if (mode == 1)
          dstf[e[i]] = base[i] + v;
        else if (find_phi)
          dstf[e[i]] = base[i] + scale[i] * v + extra[i];
        else
          dstf[e[i]] = base[i] + v;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// Warp-specialized form of tc_gemm_kernel (same operands, accumulation
// order and epilogue modes), one CTA per SM in four roles:
//   - a loader warp streams the raw stages (the 16 gathered source rows of
//     64 right-hand sides, 512 bytes each, and the operator stage) into a
//     ring of kWsRaw shared-memory slots with per-lane cp.async (16 bytes a
//     lane per row, then the contiguous operator stage), each lane's copies
//     one arrival on the slot's `raw_full` mbarrier (small bulk copies of
//     single rows would queue on the copy engine one by one).
//     What it copies comes from the CTA's stage program (one
//     TcStage record per stage, built once per phase), itself streamed into
//     shared memory kProgChunk records at a time, kProgRing chunks ahead, so
//     no dependent global load sits on the loader's path;
//   - eight converter warps read a raw stage, split it into the TF32 hi/lo
//     planes of the MMA layout in one of kWsCan canonical slots, release
//     the raw slot (`raw_empty`) and arrive on the canonical slot's `full`;
//   - an MMA warp whose elected thread waits on `full`, issues the stage's
//     12 MMAs into the chunk's accumulator slot and commits them to the
//     canonical slot's `empty` and, at a chunk's end, to the accumulator
//     slot's `accfull`;
//   - four epilogue warps (one per 32-lane quarter of tensor memory) add
//     each finished chunk into the block's running FP32 sums, free the
//     accumulator slot (`accempty`), and after the block's last chunk
//     combine sums + last chunk with the destination. Their block records
//     are read 32 blocks ahead, their output rows copied (cp.async) two
//     blocks ahead.
// A stage's column count, padding and chunk flags travel with it: the
// loader writes them beside the raw slot, the converters beside the
// canonical slot. Chunks rotate over kWsAcc accumulator slots, so the
// tensor core runs up to six chunks ahead of the epilogue warps and no role
// waits for another at a block boundary. Every wait is bounded: one that
// gives up sets the error flag and the abort flag and every role leaves its
// loops; the loader waits (bounded) for its copies in flight and the MMA
// thread for its MMAs before the tensor memory is freed.
constexpr int kWsCan = 3;
constexpr int kWsRaw = 4;
constexpr int kWsTmemCols = 512;                   // all of an SM's tensor memory (one CTA per SM)
constexpr int kWsAcc = 7;                          // accumulator slots (columns 64 s .. 64 s + 63)
constexpr int kWsSumCol = kWsAcc * kMaxRows;       // the running sums (448 .. 511)
constexpr int kWsConv = 256;                       // converter threads (warps 0-7)
constexpr int kWsMmaWarp = 8, kWsLoadWarp = 9, kWsEpiWarp0 = 10;
constexpr int kWsEpi = 128;                        // epilogue threads (warps 10-13)
constexpr int kWsThreads = kWsConv + 64 + kWsEpi;
constexpr int kRowBytes = 64 * 8;                  // one gathered source row (64 complex FP32)
constexpr int kRawXBytes = kStageCols * kRowBytes;
constexpr int kProgChunk = 8, kProgRing = 4;       // stage records per program copy; copies in the ring
static_assert(kWsSumCol + kMaxRows <= kWsTmemCols, "tensor-memory columns");

__host__ __device__ constexpr int ws_can_bytes(int npad_max) { return kWsCan * (2 * kXBytes + 2 * npad_max * 128); }
__host__ __device__ constexpr int ws_raw_slot(int npad_max) { return kRawXBytes + npad_max * 128; }

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Named barrier 1 of the epilogue warps that also ORs a flag over them, so
// that every epilogue warp takes the same branch after it.
__device__ __forceinline__ bool epilogue_sync_or(bool v) {
  int r;
  asm volatile("{ .reg .pred p, q; setp.ne.s32 p, %1, 0; bar.red.or.pred q, 1, %2, p; selp.s32 %0, 1, 0, q; }"
               : "=r"(r)
               : "r"((int)v), "n"(kWsEpi)
               : "memory");
  return r != 0;
}

__global__ void __launch_bounds__(kWsThreads, 1)
    tc_ws_kernel(const TcBlock* __restrict__ blocks, const int* __restrict__ blk_list, const int* __restrict__ blk_off,
                 const TcStage* __restrict__ prog, const int* __restrict__ prog_off, const float2* __restrict__ A,
                 const int* __restrict__ out,
                 const float2* __restrict__ src, float2* __restrict__ dst, int mode, const float2* __restrict__ P,
                 const float* __restrict__ kq, int find_phi, int npad_max, unsigned* __restrict__ err) {
  pdl_enter();
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t full[kWsCan], empty[kWsCan], raw_full[kWsRaw], raw_empty[kWsRaw], prog_full[kProgRing];
  __shared__ uint64_t accfull[kWsAcc], accempty[kWsAcc], drained;
  __shared__ __align__(16) TcStage prog_ring[kProgRing][kProgChunk];
  __shared__ int raw_hdr[kWsRaw][3];    // ncols, npad, flags of the raw slot's stage
  __shared__ int can_hdr[kWsCan][2];    // npad, flags of the canonical slot's stage
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ int orows[4][kMaxRows];    // output rows of the epilogue's blocks k .. k + 2 (slot k & 3)
  __shared__ float oscale[2][kMaxRows]; // mode 2 with find_phi: kappa^2 q of the output row
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int a_plane = npad_max * 128;
  const int can_slot = 2 * kXBytes + 2 * a_plane;
  const int raw_slot = ws_raw_slot(npad_max);
  uint8_t* const raw_base = smem + ws_can_bytes(npad_max);
  const int s_begin = __ldg(prog_off + blockIdx.x), n_st = __ldg(prog_off + blockIdx.x + 1) - s_begin;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kWsTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    auto init = [](uint64_t* bar, int count) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
    };
    for (int i = 0; i < kWsCan; ++i) {
      init(&full[i], kWsConv / 32);
      init(&empty[i], 1);
    }
    for (int i = 0; i < kWsRaw; ++i) {
      init(&raw_full[i], 33);  // the loader's 32 lanes (their copies) + lane 0's header arrival
      init(&raw_empty[i], kWsConv / 32);
    }
    for (int i = 0; i < kProgRing; ++i) init(&prog_full[i], 1);
    for (int i = 0; i < kWsAcc; ++i) {
      init(&accfull[i], 1);
      init(&accempty[i], kWsEpi / 32);
    }
    init(&drained, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  auto fail = [&]() {
    atomicOr(err, 1u);
    abort_flag = 1;
  };

  if (warp == kWsLoadWarp) {
    // ---------------- loader warp
    auto fetch = [&](int q) {  // program chunk q into ring slot q % kProgRing
      const int first = q * kProgChunk;
      if (first >= n_st || lane != 0) return;
      const uint32_t bytes = (uint32_t)(min(kProgChunk, n_st - first) * (int)sizeof(TcStage));
      mbar_expect_tx(&prog_full[q % kProgRing], bytes);
      bulk_copy(prog_ring[q % kProgRing], prog + s_begin + first, bytes, &prog_full[q % kProgRing]);
    };
    for (int q = 0; q < kProgRing; ++q) fetch(q);
    int g = 0;
    for (; g < n_st; ++g) {
      const int q = g / kProgChunk, w = g % kProgChunk, rs = g % kWsRaw;
      const bool waited = (w != 0 || mbar_wait(&prog_full[q % kProgRing], (uint32_t)((q / kProgRing) & 1))) &&
                          (g < kWsRaw || mbar_wait(&raw_empty[rs], (uint32_t)(((g / kWsRaw) - 1) & 1)));
      if (!__all_sync(0xffffffffu, waited && !abort_flag)) {
        if (lane == 0 && !waited) fail();
        break;
      }
      const TcStage& rec = prog_ring[q % kProgRing][w];
      const int ncols = rec.ncols, npad = rec.npad, flags = rec.flags;
      const float4* As = reinterpret_cast<const float4*>(A + (long long)rec.a256 * 256);
      int rows[kStageCols];  // all read before the first copy is issued
#pragma unroll
      for (int c = 0; c < kStageCols; ++c) rows[c] = rec.rows[c];
      uint8_t* raw = raw_base + rs * raw_slot;
      // 16 bytes of each gathered row per lane, then the contiguous operator
      // stage in 16-byte pieces (cp.async through L2); the slot's mbarrier
      // counts each lane's copies
#pragma unroll
      for (int c = 0; c < kStageCols; ++c)
        if (c < ncols) cp_async16(raw + c * kRowBytes + 16 * lane, src + (size_t)rows[c] * 64 + 2 * lane);
      for (int u = lane; u < npad * 8; u += 32) cp_async16(raw + kRawXBytes + 16 * u, As + u);
      if (lane == 0) {
        raw_hdr[rs][0] = ncols;
        raw_hdr[rs][1] = npad;
        raw_hdr[rs][2] = flags;
      }
      asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(&raw_full[rs])) : "memory");
      if (lane == 0) mbar_arrive(&raw_full[rs]);  // publishes the stage's header
      if (w == kProgChunk - 1) {  // chunk q is read: its slot takes chunk q + kProgRing
        __syncwarp();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        fetch(q + kProgRing);
      }
    }
    // the copies of the last stages issued have landed before the shared
    // memory is released (after a normal run these phases are long complete)
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (lane == 0)
      for (int s = (g > kWsRaw ? g - kWsRaw : 0); s < g; ++s)
        if (!mbar_wait(&raw_full[s % kWsRaw], (uint32_t)((s / kWsRaw) & 1))) {
          fail();
          break;
        }
    __syncwarp();
  } else if (warp == kWsMmaWarp) {
    // ---------------- MMA warp: one elected thread issues and commits.
    if (lane == 0) {
      const uint32_t idesc_base = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(128 >> 4) << 24);
      int g = 0;
      long long G = -1;  // chunks started
      for (; g < n_st; ++g) {
        const int slot = g % kWsCan;
        if (!mbar_wait(&full[slot], (uint32_t)((g / kWsCan) & 1))) {
          fail();
          break;
        }
        const int npad = can_hdr[slot][0], flags = can_hdr[slot][1];
        const bool chunk_start = flags & 1, chunk_end = flags & 2;
        if (chunk_start) ++G;
        const int as = (int)(G % kWsAcc);
        if (chunk_start && G >= kWsAcc && !mbar_wait(&accempty[as], (uint32_t)(((G / kWsAcc) - 1) & 1))) {
          fail();
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t idesc = idesc_base | ((uint32_t)(npad >> 3) << 17);
        uint8_t* base = smem + slot * can_slot;
        const uint32_t xh = smem_u32(base), xl = smem_u32(base + kXBytes);
        const uint32_t ah = smem_u32(base + 2 * kXBytes), al = smem_u32(base + 2 * kXBytes + a_plane);
        const uint32_t dt = tmem + (uint32_t)(as * kMaxRows);
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint32_t o = ks * 256;
          const uint64_t dxh = sdesc_sw128(xh + 32 * ks), dxl = sdesc_sw128(xl + 32 * ks);
          const uint64_t dah = sdesc(ah + o, 128, kRowGroupBytes), dal = sdesc(al + o, 128, kRowGroupBytes);
          mma_tf32(dt, dxh, dah, idesc, (!chunk_start || ks > 0) ? 1u : 0u);
          mma_tf32(dt, dxh, dal, idesc, 1u);
          mma_tf32(dt, dxl, dah, idesc, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&empty[slot]))
                     : "memory");
        if (chunk_end)
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&accfull[as]))
                       : "memory");
      }
      // every MMA issued (g stages) has completed before the tensor memory is freed
      if (g > 0) {
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&drained))
                     : "memory");
        if (!mbar_wait(&drained, 0u)) fail();
      }
    }
    __syncwarp();
  } else if (warp < kWsMmaWarp) {
    // ---------------- converter warps
    // Thread (kk, m): source column kk of the stage, right-hand sides 2m,
    // 2m + 1, 2m + 32, 2m + 33. Eight consecutive lanes read 128
    // contiguous bytes of a raw row; the 16 lanes of a half-warp cover the
    // eight rows of a core matrix and both column parities, so the 8-byte
    // canonical stores are free of bank conflicts.
    const int m = (t & 7) | (((t >> 4) & 1) << 3);
    const int kk = ((t >> 5) << 1) | ((t >> 3) & 1);
    const int rot = (t >> 2) & 1;
    for (int g = 0; g < n_st; ++g) {
      const int rs = g % kWsRaw, cs = g % kWsCan;
      const bool waited = mbar_wait(&raw_full[rs], (uint32_t)((g / kWsRaw) & 1)) &&
                          (g < kWsCan || mbar_wait(&empty[cs], (uint32_t)(((g / kWsCan) - 1) & 1)));
      if (!__all_sync(0xffffffffu, waited && !abort_flag)) {
        if (lane == 0 && !waited) fail();
        break;
      }
      const int ncols = raw_hdr[rs][0], npad = raw_hdr[rs][1], flags = raw_hdr[rs][2];
      const uint8_t* raw = raw_base + rs * raw_slot;
      float4 x0 = make_float4(0.f, 0.f, 0.f, 0.f), x1 = x0, a[2];
      if (kk < ncols) {  // columns past the block's last are zero
        const float4* row = reinterpret_cast<const float4*>(raw + kk * kRowBytes);
        x0 = row[m];
        x1 = row[m + 16];
      }
      const float4* Ar = reinterpret_cast<const float4*>(raw + kRawXBytes);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int u = t + q * kWsConv;
        a[q] = u < npad * 8 ? Ar[u] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      uint8_t* base = smem + cs * can_slot;
      float2* Xh = reinterpret_cast<float2*>(base);
      float2* Xl = reinterpret_cast<float2*>(base + kXBytes);
      float4* Ah = reinterpret_cast<float4*>(base + 2 * kXBytes);
      float4* Al = reinterpret_cast<float4*>(base + 2 * kXBytes + a_plane);
      // value ii of the thread: right-hand side 2m + (ii & 1) + 32 (ii >> 1);
      // store i takes ii = i ^ rot
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int ii = i ^ rot;
        const float4 h2 = (ii & 2) ? x1 : x0;
        const float vx = (ii & 1) ? h2.z : h2.x, vy = (ii & 1) ? h2.w : h2.y;
        const int j = 2 * m + (ii & 1) + 32 * (ii >> 1);
        const float hx = tf32_rn(vx), hy = tf32_rn(vy);
        const float lx = tf32_rn(vx - hx), ly = tf32_rn(vy - hy);
        const int o_re = canon_sw128(j, kk), o_im = canon_sw128(64 + j, kk);
        Xh[o_re] = make_float2(hx, hy);
        Xl[o_re] = make_float2(lx, ly);
        Xh[o_im] = make_float2(hy, -hx);
        Xl[o_im] = make_float2(ly, -lx);
      }
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int u = t + q * kWsConv;
        if (u < npad * 8) {
          const float4 v = a[q];
          const float4 h = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
          Ah[u] = h;
          Al[u] = make_float4(tf32_rn(v.x - h.x), tf32_rn(v.y - h.y), tf32_rn(v.z - h.z), tf32_rn(v.w - h.w));
        }
      }
      if (t == 0) {  // read by the MMA thread after `full`
        can_hdr[cs][0] = npad;
        can_hdr[cs][1] = flags;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&full[cs]);
        mbar_arrive(&raw_empty[rs]);
      }
    }
  } else {
    // ---------------- epilogue warps
    const int e = t - kWsEpiWarp0 * 32;              // 0..127
    const int quarter = warp & 3;                    // tensor-memory lanes 32 quarter .. + 31
    const int mrow = quarter * 32 + lane, part = mrow >> 6, j = mrow & 63;
    const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
    auto tld16 = [&](uint32_t col, uint32_t* r) {
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(lane_base + col));
    };
    auto tst16 = [&](uint32_t col, const uint32_t* r) {
      asm volatile(
          "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
              lane_base + col),
          "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
          "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
          : "memory");
    };
    auto wait_chunk = [&](long long G) -> bool {  // warp-uniform: the loads after it are warp-collective
      const bool done = __all_sync(0xffffffffu, mbar_wait(&accfull[G % kWsAcc], (uint32_t)((G / kWsAcc) & 1)));
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      return done;
    };
    auto free_chunk = [&](long long G) {
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&accempty[G % kWsAcc]);
    };
    // Block k of this CTA is blocks[blk_list[blk_off[cta] + k]]. Its record
    // (rows, npad, nst, o_off) sits in lane k & 31 of a window of 32
    // records; the next window is loaded a window ahead.
    const int b_first = __ldg(blk_off + blockIdx.x), n_mine = __ldg(blk_off + blockIdx.x + 1) - b_first;
    auto load_rec = [&](int k) -> int4 {
      if (k >= n_mine) return make_int4(0, 0, 0, 0);
      const TcBlock* B = blocks + __ldg(blk_list + b_first + k);
      return make_int4(B->rows, B->npad, B->nst, B->o_off);
    };
    auto rec_of = [&](int k, const int4& cur, const int4& nxt, int base) -> int4 {  // warp-uniform k
      const int4 w = (k - base) < 32 ? cur : nxt;
      const int l = k & 31;
      return make_int4(__shfl_sync(0xffffffffu, w.x, l), __shfl_sync(0xffffffffu, w.y, l),
                       __shfl_sync(0xffffffffu, w.z, l), __shfl_sync(0xffffffffu, w.w, l));
    };
    // output rows of block k into orows[k & 3] (cp.async, one group per block)
    auto copy_rows = [&](int k, const int4& r) {
      if (k < n_mine && e < r.x) {
        const uint32_t d = smem_u32(&orows[k & 3][e]);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(out + r.w + e) : "memory");
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    int4 wcur = load_rec(lane), wnxt = load_rec(32 + lane);
    int wbase = 0;  // block of wcur's lane 0
    copy_rows(0, rec_of(0, wcur, wnxt, wbase));
    copy_rows(1, rec_of(1, wcur, wnxt, wbase));
    long long gc = 0;
    for (int k = 0; k < n_mine; ++k) {
      if (k - wbase == 32) {
        wcur = wnxt;
        wbase += 32;
        wnxt = load_rec(wbase + 32 + lane);
      }
      const int4 r = rec_of(k, wcur, wnxt, wbase);
      const int rows = r.x, npad = r.y, nst = r.z;
      copy_rows(k + 2, rec_of(k + 2, wcur, wnxt, wbase));
      asm volatile("cp.async.wait_group 2;" ::: "memory");  // this thread's rows of block k have landed
      const int ob = k & 3, sb = k & 1;
      const long long gc0 = gc;
      const int nchunks = (nst + kChunkStages - 1) / kChunkStages;
      gc = gc0 + nchunks;
      bool ok = true;
      // sums = chunk 0 + chunk 1 + ... (round-to-nearest FP32, in order), all but the last chunk
      for (long long G = gc0; G + 1 < gc; ++G) {
        if (!wait_chunk(G)) {
          ok = false;
          break;
        }
        const uint32_t acol = (uint32_t)((G % kWsAcc) * kMaxRows);
        for (int c0 = 0; c0 < npad; c0 += 16) {
          uint32_t ra[16], q[16];
          tld16(acol + c0, ra);
          if (G > gc0) tld16((uint32_t)(kWsSumCol + c0), q);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (G > gc0) {
#pragma unroll
            for (int i = 0; i < 16; ++i) ra[i] = __float_as_uint(__uint_as_float(q[i]) + __uint_as_float(ra[i]));
          }
          tst16((uint32_t)(kWsSumCol + c0), ra);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        free_chunk(G);
      }
      if (ok && nchunks > 0 && !wait_chunk(gc - 1)) ok = false;
      if (!ok && lane == 0) fail();
      if (mode == 2 && find_phi && e < rows) oscale[sb][e] = __ldg(kq + orows[ob][e]);
      // output rows visible; the same decision in every epilogue warp
      if (epilogue_sync_or(!ok || abort_flag)) break;
      // y = sums + last chunk, combined with the destination; all old values
      // of a 16-row group are loaded before any of them is written (the rows
      // of a phase are distinct)
      const uint32_t lcol = (uint32_t)(((gc - 1) % kWsAcc) * kMaxRows);
      float* dstf = reinterpret_cast<float*>(dst);
      for (int c0 = 0; c0 < rows; c0 += 16) {
        uint32_t ra[16], q[16];
        if (nchunks > 0) {
          tld16(lcol + c0, ra);
          if (nchunks > 1) tld16((uint32_t)(kWsSumCol + c0), q);
        }
        float basev[16], extra[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          basev[i] = extra[i] = 0.f;
          if (c0 + i < rows) {
            const size_t el = ((size_t)orows[ob][c0 + i] * 64 + j) * 2 + part;
            if (mode == 2) {
              basev[i] = ld_chain(reinterpret_cast<const float*>(P) + el);
              if (find_phi) extra[i] = ld_chain(reinterpret_cast<const float*>(src) + el);
            }
          }
        }
        if (nchunks > 0) asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          if (c0 + i < rows) {
            const size_t el = ((size_t)orows[ob][c0 + i] * 64 + j) * 2 + part;
            float v = 0.f;  // a block without columns sums to zero
            if (nchunks > 1)
              v = __uint_as_float(q[i]) + __uint_as_float(ra[i]);
            else if (nchunks == 1)
              v = __uint_as_float(ra[i]);
            // mode 0: v; mode 1: old + v (an L2 reduction: one FP32 add, no
            // round trip); mode 2: P + s v, + x with find_phi
            if (mode == 1)
              asm volatile("red.global.add.f32 [%0], %1;" ::"l"(dstf + el), "f"(v) : "memory");
            else
              dstf[el] = mode == 0 ? v
                                   : (find_phi ? basev[i] + oscale[sb][c0 + i] * v + extra[i] : basev[i] + v);
          }
        }
      }
      if (nchunks > 0) free_chunk(gc - 1);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");  // no copy into shared memory outlives the CTA
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kWsTmemCols));
}

// The bounded-wait path of the tensor-core kernels on its own: the CTA
// allocates its tensor memory, every thread waits on an mbarrier that
// nothing arrives on with the kernels' wait (`polls` polls), a wait that
// gives up sets the error flag as the kernels' do, and the tensor memory is
// freed before the CTA exits.
__global__ void tc_wait_probe_kernel(long long polls, unsigned* __restrict__ err) {
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  const int t = threadIdx.x;
  if (t < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tbase)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tm = tbase;
  if (!mbar_wait_n(&bar, 0u, polls)) atomicOr(err, 1u);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(kTmemCols));
}

// Stage program of a phase: the stages of block b in order, blocks dealt
// to the CTAs round-robin (CTA c: blocks c, c + grid, ...); one thread per
// stage record.
__global__ void tc_program_kernel(const int2* __restrict__ stage_of, int n, const TcBlock* __restrict__ blocks,
                                  const int* __restrict__ idx, TcStage* __restrict__ prog) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const TcBlock blk = blocks[stage_of[s].x];
    const int st = stage_of[s].y;
    TcStage r;
    r.ncols = min(kStageCols, blk.K - st * kStageCols);
    for (int c = 0; c < kStageCols; ++c) r.rows[c] = c < r.ncols ? idx[blk.i_off + st * kStageCols + c] : 0;
    r.a256 = (int)((blk.a_off + (long long)st * blk.npad * kStageCols) >> 8);
    r.npad = blk.npad;
    r.flags = (st % kChunkStages == 0 ? 1 : 0) | (st % kChunkStages == kChunkStages - 1 || st == blk.nst - 1 ? 2 : 0);
    prog[s] = r;
  }
}

// Far-field phase -> tensor-core form: one warp per tile writes its
// elements, conjugated, into the canonical stages of the part of its block
// that holds the row (tile_block: the block's first part; parts are
// consecutive, kMaxRows rows each).
__global__ void tc_build_far_kernel(const GemvTile* __restrict__ tiles, int n_tiles, const int* __restrict__ tile_block,
                                    const int* __restrict__ tile_row0, const TcBlock* __restrict__ blocks,
                                    const float2* __restrict__ A32, float2* __restrict__ Atc) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_tiles; w += nw) {
    const GemvTile tl = tiles[w];
    const int R = 32 >> tl.log2s, S = 1 << tl.log2s;
    const int r = lane % R, s = lane / R;
    if (r >= tl.rows) continue;
    const int row = tile_row0[w] + r;
    const TcBlock blk = blocks[tile_block[w] + row / kMaxRows];
    const int prow = row % kMaxRows;
    for (int q = 0; q < tl.qmax; ++q) {
      const int k = q * S + s;
      if (k >= blk.K) break;
      const float2 a = A32[tl.a_off + 32LL * q + lane];
      const int st = k / kStageCols, cc = k % kStageCols;
      Atc[blk.a_off + (long long)st * blk.npad * kStageCols + canon(prow, cc)] = make_float2(a.x, -a.y);
    }
  }
}

// Near field -> tensor-core form: the nine colleague blocks side by side
// (column k = q * rank + c), shared by every leaf; per leaf the gather list
// of its colleagues' points (a zero row of the source for a missing
// colleague) and its output rows.
__global__ void tc_build_near_kernel(int rank, int npad, const double2* __restrict__ nearB, float2* __restrict__ Atc) {
  const int K = 9 * rank;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rank * K; i += gridDim.x * blockDim.x) {
    const int row = i / K, k = i - row * K, q = k / rank, c = k - q * rank;
    const double2 v = nearB[((size_t)q * rank + row) * rank + c];
    const int st = k / kStageCols, cc = k % kStageCols;
    Atc[(long long)st * npad * kStageCols + canon(row, cc)] = make_float2((float)v.x, (float)-v.y);
  }
}

__global__ void tc_near_lists_kernel(int n_leaves, int rank, long long zero_row, const int* __restrict__ coll,
                                     int* __restrict__ idx, int* __restrict__ out, TcBlock* __restrict__ blocks,
                                     int npad, int nst) {
  const int K = 9 * rank;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)n_leaves * K;
       i += (long long)gridDim.x * blockDim.x) {
    const int leaf = (int)(i / K), k = (int)(i - (long long)leaf * K), q = k / rank, c = k - q * rank;
    const int nb = coll[leaf * 9 + q];
    idx[i] = nb >= 0 ? nb * rank + c : (int)zero_row;
    if (k < rank) out[(size_t)leaf * rank + k] = leaf * rank + k;
    if (k == 0) blocks[leaf] = TcBlock{0, leaf * K, leaf * rank, rank, npad, K, nst};
  }
}

__global__ void zero_f2_kernel(float2* __restrict__ p, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = make_float2(0.f, 0.f);
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side.

struct TcPhase {
  float2* A = nullptr;
  TcBlock* blocks = nullptr;
  const int* idx = nullptr;  // the FP32 phase's gather lists (near field: own)
  const int* out = nullptr;
  int n_blocks = 0;
  int npad_max = 16;
  int accumulate = 0;
  long long a_elems = 0;
  long long entries = 0;  // true complex entries
  TcStage* prog = nullptr;  // stage program of tc_ws_kernel (CTA c: prog[prog_off[c] .. prog_off[c + 1]))
  int* prog_off = nullptr;
  int* blk_list = nullptr;  // CTA c's blocks: blk_list[blk_off[c] .. blk_off[c + 1])
  int* blk_off = nullptr;
  int prog_grid = 0;
  long long prog_stages = 0;  // stages of the phase (all CTAs)
};

struct TcOperator {
  std::vector<TcPhase> up, down;
  TcPhase m2l, near;
  int* near_idx = nullptr;
  int* near_out = nullptr;
  unsigned* err = nullptr;
  int sms = 0;
  std::vector<void*> owned;
};

namespace {

int smem_for(int npad_max) { return 2 * (2 * kXBytes + 2 * npad_max * 128); }

template <class T>
cudaError_t dalloc(TcOperator& t, T** p, size_t n) {
  cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
  if (e == cudaSuccess) t.owned.push_back(*p);
  return e;
}

// Stage program of a phase whose blocks (nst per block on the host) and
// gather lists are on the device. The blocks are dealt to min(n_blocks, sms)
// CTAs longest first, each to the CTA with the least work so far (a block
// costs its stages plus about two stages of pipeline fill and epilogue);
// each CTA's stages are contiguous, in the order of its block list.
cudaError_t build_program(TcOperator& T, TcPhase& ph, const std::vector<int>& nst) {
  const int nb = ph.n_blocks;
  if (nb == 0) return cudaSuccess;
  const int grid = std::min(nb, T.sms);
  std::vector<int> order(nb);
  for (int b = 0; b < nb; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nst[a] > nst[b]; });
  std::priority_queue<std::pair<long long, int>, std::vector<std::pair<long long, int>>, std::greater<>> least;
  for (int c = 0; c < grid; ++c) least.push({0, c});
  std::vector<std::vector<int>> mine(grid);
  for (int b : order) {
    const auto [work, c] = least.top();
    least.pop();
    mine[c].push_back(b);
    least.push({work + nst[b] + 2, c});
  }
  std::vector<int> off(grid + 1, 0), boff(grid + 1, 0), list;
  std::vector<int2> stage_of;
  for (int c = 0; c < grid; ++c) {
    off[c] = (int)stage_of.size();
    boff[c] = (int)list.size();
    for (int b : mine[c]) {
      list.push_back(b);
      for (int st = 0; st < nst[b]; ++st) stage_of.push_back(make_int2(b, st));
    }
  }
  off[grid] = (int)stage_of.size();
  boff[grid] = (int)list.size();
  ph.prog_grid = grid;
  ph.prog_stages = (long long)stage_of.size();
  int2* d_of = nullptr;
  cudaError_t e = dalloc(T, &ph.prog, stage_of.size());
  if (e == cudaSuccess) e = dalloc(T, &ph.prog_off, off.size());
  if (e == cudaSuccess) e = dalloc(T, &ph.blk_list, list.size());
  if (e == cudaSuccess) e = dalloc(T, &ph.blk_off, boff.size());
  if (e == cudaSuccess) e = cudaMemcpy(ph.blk_list, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ph.blk_off, boff.data(), boff.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&d_of, std::max<size_t>(stage_of.size(), 1) * sizeof(int2));
  if (e == cudaSuccess) e = cudaMemcpy(ph.prog_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !stage_of.empty())
    e = cudaMemcpy(d_of, stage_of.data(), stage_of.size() * sizeof(int2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !stage_of.empty()) {
    tc_program_kernel<<<512, 256>>>(d_of, (int)stage_of.size(), ph.blocks, ph.idx, ph.prog);
    e = cudaDeviceSynchronize();
  }
  cudaFree(d_of);
  return e;
}

// Tensor-core form of one far-field phase from its tiles (host block
// structure, device FP32 tiles).
cudaError_t build_far(TcOperator& T, const GemvPhase& h, const DevPhase<float2>& d32, TcPhase& out, std::string& err) {
  out.idx = d32.idx;
  out.out = d32.out;
  out.accumulate = d32.accumulate;
  out.entries = d32.entries;
  const int nb = (int)h.blk_rows.size();
  out.n_blocks = 0;
  if (nb == 0 || d32.n_tiles == 0) return cudaSuccess;
  // Blocks of more than kMaxRows rows become several parts with the same
  // gather list.
  std::vector<TcBlock> blocks;
  std::vector<int> tile_block(h.tiles.size()), tile_row0(h.tiles.size());
  long long a = 0;
  for (int b = 0; b < nb; ++b) {
    const int t0 = h.blk_tile0[b], t1 = h.blk_tile0[b + 1];
    const int rows = h.blk_rows[b], K = h.blk_K[b];
    const int nst = (K + kStageCols - 1) / kStageCols;
    const int first = (int)blocks.size();
    for (int r0 = 0; r0 < rows; r0 += kMaxRows) {
      const int pr = std::min(kMaxRows, rows - r0);
      const int npad = std::max(16, (pr + 15) / 16 * 16);
      blocks.push_back(TcBlock{a, (int)h.tiles[t0].i_off, h.tiles[t0].row_base + r0, pr, npad, K, nst});
      out.npad_max = std::max(out.npad_max, npad);
      a += (long long)nst * npad * kStageCols;
    }
    int r0 = 0;
    for (int tt = t0; tt < t1; ++tt) {
      tile_block[tt] = first;
      tile_row0[tt] = r0;
      r0 += h.tiles[tt].rows;
    }
  }
  out.n_blocks = (int)blocks.size();
  out.a_elems = a;
  int *dtb = nullptr, *dtr = nullptr;
  cudaError_t e = dalloc(T, &out.A, (size_t)a);
  if (e == cudaSuccess) e = dalloc(T, &out.blocks, blocks.size());
  if (e == cudaSuccess) e = cudaMalloc(&dtb, tile_block.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&dtr, tile_row0.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(out.blocks, blocks.data(), blocks.size() * sizeof(TcBlock), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dtb, tile_block.data(), tile_block.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dtr, tile_row0.data(), tile_row0.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    zero_f2_kernel<<<1024, 256>>>(out.A, a);
    tc_build_far_kernel<<<1024, 256>>>(d32.tiles, d32.n_tiles, dtb, dtr, out.blocks, d32.A, out.A);
    e = cudaDeviceSynchronize();
  }
  cudaFree(dtb);
  cudaFree(dtr);
  if (e == cudaSuccess) {
    std::vector<int> nst(blocks.size());
    for (size_t b = 0; b < blocks.size(); ++b) nst[b] = blocks[b].nst;
    e = build_program(T, out, nst);
  }
  if (e != cudaSuccess) err = std::string("tensor-core form: ") + cudaGetErrorString(e);
  return e;
}

int ws_smem_for(int npad_max) { return ws_can_bytes(npad_max) + kWsRaw * ws_raw_slot(npad_max); }

// The warp-specialized kernel runs unless LS_TC_WS=0 selects the two-CTA
// kernel (read once).
bool use_ws() {
  static const bool ws = [] {
    const char* v = std::getenv("LS_TC_WS");
    return !(v && std::atoi(v) == 0);
  }();
  return ws;
}

cudaError_t launch_tc(const TcOperator& T, const TcPhase& ph, const float2* src, float2* dst, int mode,
                      const float2* P, const float* kq, int find_phi, cudaStream_t s) {
  if (ph.n_blocks == 0) return cudaSuccess;
  if (use_ws()) {  // one CTA per SM, the grid its stage program was dealt to
    return launch_pdl(tc_ws_kernel, ph.prog_grid, kWsThreads, (size_t)ws_smem_for(ph.npad_max), s,
                      (const TcBlock*)ph.blocks, (const int*)ph.blk_list, (const int*)ph.blk_off,
                      (const TcStage*)ph.prog, (const int*)ph.prog_off, (const float2*)ph.A, ph.out, src, dst, mode,
                      P, kq, find_phi, ph.npad_max, T.err);
  }
  const int grid = std::min(ph.n_blocks, 2 * T.sms);  // two CTAs per SM (96 KB shared memory, 128 TMEM columns each)
  return launch_pdl(tc_gemm_kernel, grid, kTcThreads, (size_t)smem_for(ph.npad_max), s, (const TcBlock*)ph.blocks,
                    ph.n_blocks, (const float2*)ph.A, ph.idx, ph.out, src, dst, mode, P, kq, find_phi, ph.npad_max,
                    T.err);
}

}  // namespace

void dev_free_tc(DevOperator& d) {
  if (!d.tc) return;
  for (void* p : d.tc->owned) cudaFree(p);
  delete d.tc;
  d.tc = nullptr;
}

bool dev_enable_tc(DevOperator& d, const HostOperator& h, std::string& err) {
  if (d.tc) return true;
  if (!d.has_f32) {
    err = "tensor-core form: the FP32 operator is not enabled";
    return false;
  }
  cudaSetDevice(d.device);
  TcOperator* T = new TcOperator();
  cudaDeviceGetAttribute(&T->sms, cudaDevAttrMultiProcessorCount, d.device);
  if (T->sms <= 0) T->sms = 148;
  cudaError_t e = dalloc(*T, &T->err, 1);
  if (e == cudaSuccess) e = cudaMemset(T->err, 0, sizeof(unsigned));
  T->up.resize(d.up32.size());
  for (size_t i = 0; i < d.up32.size() && e == cudaSuccess; ++i) e = build_far(*T, h.up[i], d.up32[i], T->up[i], err);
  if (e == cudaSuccess) e = build_far(*T, h.m2l, d.m2l32, T->m2l, err);
  T->down.resize(d.down32.size());
  for (size_t i = 0; i < d.down32.size() && e == cudaSuccess; ++i)
    e = build_far(*T, h.down[i], d.down32[i], T->down[i], err);
  if (e == cudaSuccess && d.generic_near) {
    // adaptive trees: the near phase is one more gather-GEMV phase
    e = build_far(*T, h.nearph, d.nearph32, T->near, err);
  } else if (e == cudaSuccess) {
    TcPhase& nr = T->near;
    const int K = 9 * d.rank;
    if (d.rank > kMaxRows) {
      err = "tensor-core form: more than 64 points per leaf";
      e = cudaErrorInvalidValue;
    }
    nr.npad_max = std::max(16, (d.rank + 15) / 16 * 16);
    const int nst = (K + kStageCols - 1) / kStageCols;
    nr.a_elems = (long long)nst * nr.npad_max * kStageCols;
    nr.n_blocks = d.n_leaves;
    nr.entries = 9LL * d.rank * d.rank;
    if (e == cudaSuccess) e = dalloc(*T, &nr.A, (size_t)nr.a_elems);
    if (e == cudaSuccess) e = dalloc(*T, &nr.blocks, (size_t)d.n_leaves);
    if (e == cudaSuccess) e = dalloc(*T, &T->near_idx, (size_t)d.n_leaves * K);
    if (e == cudaSuccess) e = dalloc(*T, &T->near_out, (size_t)d.N);
    if (e == cudaSuccess) {
      nr.idx = T->near_idx;
      nr.out = T->near_out;
      zero_f2_kernel<<<256, 256>>>(nr.A, nr.a_elems);
      tc_build_near_kernel<<<256, 256>>>(d.rank, nr.npad_max, d.nearB, nr.A);
      tc_near_lists_kernel<<<1024, 256>>>(d.n_leaves, d.rank, d.charges_len, d.colleague, T->near_idx, T->near_out,
                                          nr.blocks, nr.npad_max, nst);
      e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) e = build_program(*T, nr, std::vector<int>((size_t)d.n_leaves, nst));
  }
  int npad = std::max(T->m2l.npad_max, T->near.npad_max);
  for (auto& p : T->up) npad = std::max(npad, p.npad_max);
  for (auto& p : T->down) npad = std::max(npad, p.npad_max);
  if (e == cudaSuccess)
    e = raise_smem_limit((const void*)tc_gemm_kernel, smem_for(npad));
  if (e == cudaSuccess)
    e = raise_smem_limit((const void*)tc_ws_kernel, ws_smem_for(npad));
  if (e != cudaSuccess) {
    if (err.empty()) err = std::string("tensor-core form: ") + cudaGetErrorString(e);
    for (void* p : T->owned) cudaFree(p);
    delete T;
    return false;
  }
  d.tc = T;
  return true;
}

// y = A32 x for the 64 right-hand sides of a block stored rhs-minor
// (element (i, j) at 64 i + j). S and P are the block's charge and
// potential buffers (S with one extra zero row at charges_len, the gather
// target of missing near-field colleagues).
cudaError_t dev_matvec_f32_wide(DevOperator& d, const float2* x, float2* y, float2* S, float2* P, cudaStream_t s) {
  if (!d.tc) return cudaErrorInvalidValue;
  const TcOperator& T = *d.tc;
  cudaMemcpyAsync(S, x, (size_t)d.N * kTcRhs * sizeof(float2), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(P, 0, (size_t)d.pots_len * kTcRhs * sizeof(float2), s);
  cudaError_t e = cudaSuccess;
  for (const auto& ph : T.up)
    if (e == cudaSuccess) e = launch_tc(T, ph, S, S, 0, nullptr, nullptr, 0, s);
  if (e == cudaSuccess) e = launch_tc(T, T.m2l, S, P, 0, nullptr, nullptr, 0, s);
  for (const auto& ph : T.down)
    if (e == cudaSuccess) e = launch_tc(T, ph, P, P, 1, nullptr, nullptr, 0, s);
  if (d.generic_near) {  // adaptive trees: the near phase accumulates into P[0:N), which is y
    if (e == cudaSuccess) e = launch_tc(T, T.near, S, P, 1, nullptr, nullptr, 0, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(y, P, (size_t)d.N * kTcRhs * sizeof(float2), cudaMemcpyDeviceToDevice, s);
  } else if (e == cudaSuccess) {
    e = launch_tc(T, T.near, S, y, 2, P, d.kq32, d.find_phi, s);
  }
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t dev_tc_error(DevOperator& d, unsigned* flag) {
  *flag = 0;
  if (!d.tc) return cudaSuccess;
  return cudaMemcpy(flag, d.tc->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
}

cudaError_t dev_tc_wait_probe(int device, long long polls, unsigned* gave_up) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  unsigned* err = nullptr;
  if ((e = cudaMalloc(&err, sizeof(unsigned))) != cudaSuccess) return e;
  e = cudaMemset(err, 0, sizeof(unsigned));
  if (e == cudaSuccess) {
    tc_wait_probe_kernel<<<1, 128>>>(polls, err);
    e = cudaDeviceSynchronize();
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(gave_up, err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  cudaFree(err);
  return e;
}

long long dev_tc_stages(const DevOperator& d) {
  if (!d.tc) return 0;
  long long n = 0;
  auto add = [&](const TcPhase& p) {
    if (p.n_blocks) n += p.prog_stages;
  };
  for (auto& p : d.tc->up) add(p);
  add(d.tc->m2l);
  for (auto& p : d.tc->down) add(p);
  add(d.tc->near);
  return n;
}

long long dev_tc_operator_bytes(const DevOperator& d) {
  if (!d.tc) return 0;
  long long b = 0;
  for (auto& p : d.tc->up) b += p.a_elems * 8;
  for (auto& p : d.tc->down) b += p.a_elems * 8;
  return b + d.tc->m2l.a_elems * 8 + d.tc->near.a_elems * 8;
}

}  // namespace lsg
