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
#include <cstdint>
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

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done = 0;
  for (long long it = 0; it < kWaitLimit && !done; ++it)
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
  return done != 0;
}

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
  if (e != cudaSuccess) err = std::string("tensor-core form: ") + cudaGetErrorString(e);
  return e;
}

cudaError_t launch_tc(const TcOperator& T, const TcPhase& ph, const float2* src, float2* dst, int mode,
                      const float2* P, const float* kq, int find_phi, cudaStream_t s) {
  if (ph.n_blocks == 0) return cudaSuccess;
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
  }
  int need = 0;
  for (auto& p : T->up) need = std::max(need, smem_for(p.npad_max));
  for (auto& p : T->down) need = std::max(need, smem_for(p.npad_max));
  need = std::max(need, std::max(smem_for(T->m2l.npad_max), smem_for(T->near.npad_max)));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, need);
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

long long dev_tc_operator_bytes(const DevOperator& d) {
  if (!d.tc) return 0;
  long long b = 0;
  for (auto& p : d.tc->up) b += p.a_elems * 8;
  for (auto& p : d.tc->down) b += p.a_elems * 8;
  return b + d.tc->m2l.a_elems * 8 + d.tc->near.a_elems * 8;
}

}  // namespace lsg
