// The far-field part of the assembly on the GPU: the far-field entry table
// and the NCA skeleton search (ACA_only_nodes, GMRES/ACA.hpp:253-481) of
// every box of a level.
//
// Far-field entries. K(i, j) for a target i and a source node j of leaf l
// is (i/4) sum_n M[j mod rank][n] h_n(p_i - c_l) (G_FMM2DTree.hpp:603-658),
// scaled by kappa^2 q(p_i) (and + 1 on the diagonal) for the LS operator.
// On a uniform tree p_i - c_l takes few distinct values per coordinate: the
// x part is fl(gx_i - cx_l), a function of (x node of i, x column of i's
// leaf, x column of l), and likewise for y. The table holds, for every pair
// (distinct x value, distinct y value), the sums for all `rank` nodes of a
// leaf, so an entry is two index lookups and one load. Each key's Hankel
// vector follows the host's formulas (J_n, Y_n by the same recurrences from
// J_0, J_1, Y_0, Y_1; e^{i n theta} from sin and cos of n theta; the same
// operand order in every product and sum); the values differ from the
// host's only through CUDA's j0 / j1 / y0 / y1 / atan2 / sin / cos against
// libstdc++'s and glibc's, in the last bits. The file is compiled without
// FMA contraction, as the host's assembler is.
//
// NCA. One CTA per task (a box's outgoing or incoming block: rows, cols,
// tolerance; 128 threads on levels with few blocks, 32 on levels with many),
// tasks taken from an atomic counter. The steps are
// the host's aca_core in the same order: pivot search with ties to the
// lowest index, the rank-1 updates element by element in the same operand
// order, the norm estimate and the stopping rules. Norms and dot products
// are block reductions (another summation order than the host's loop), so
// a stopping decision taken within rounding of its threshold can differ. A
// task whose rank would pass the scratch's rank capacity is marked and the
// host redoes it. Every loop is bounded by the task's sizes; threads wait
// on nothing but the CTA's own barriers.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <string>
#include <vector>

#include "launch.h"
#include "ls_internal.h"

namespace lsg {

namespace {

constexpr int kSeriesG = 15;                 // FarFieldInteraction.hpp:55
constexpr int kTerms = 2 * kSeriesG + 1;
constexpr int kTableKeys = 128;              // keys (threads) per block of the table kernel
constexpr int kNcaRankCapG = 64;             // largest NcaTask::R the kernel takes
constexpr unsigned kFull = 0xffffffffu;

// J_n(x), Y_n(x), n = 0..15, x > 0, by the host's method: Y_n by forward
// recurrence from Y_0, Y_1; J_n by forward recurrence when x > 15, else by
// Miller's backward recurrence from order 2((15 + 20 + sqrt(60*15)) / 2),
// rescaled past 1e10 and normalised to the larger of J_0, J_1.
__device__ void bessel_jy_all(double x, double* J, double* Y) {
  const double j0v = j0(x), j1v = j1(x);
  Y[0] = y0(x);
  Y[1] = y1(x);
  for (int n = 1; n < kSeriesG; ++n) Y[n + 1] = (2.0 * n / x) * Y[n] - Y[n - 1];
  J[0] = j0v;
  J[1] = j1v;
  if (x > kSeriesG) {
    for (int n = 1; n < kSeriesG; ++n) J[n + 1] = (2.0 * n / x) * J[n] - J[n - 1];
    return;
  }
  const int base = kSeriesG > (int)x ? kSeriesG : (int)x;
  const int m = 2 * ((base + 20 + (int)sqrt(60.0 * base)) / 2);
  double F[kSeriesG + 1];
  double fp = 0.0, f = 1.0;
  for (int j = m; j > 0; --j) {
    const double fm = (2.0 * j / x) * f - fp;
    fp = f;
    f = fm;
    if (fabs(f) > 1e10) {
      f *= 1e-10;
      fp *= 1e-10;
      for (int i = j + 1; i <= kSeriesG; ++i) F[i] *= 1e-10;
    }
    if (j <= kSeriesG) F[j] = fp;
  }
  F[0] = f;
  const double s = fabs(j0v) >= fabs(j1v) ? j0v / F[0] : j1v / F[1];
  for (int i = 0; i <= kSeriesG; ++i) J[i] = F[i] * s;
}

// Table: S[(xi * ny + yi) * rank + node] = sum_n M[node][n] h_n(ux[xi], uy[yi]).
// Threads 0..kTableKeys-1 each form one key's Hankel vector in shared
// memory; then the block writes the sums of its keys, contiguous in S.
__global__ void __launch_bounds__(kTableKeys) far_table_kernel(const double* __restrict__ ux,
                                                               const double* __restrict__ uy, int ny, long long nkeys,
                                                               double kappa, const double2* __restrict__ M, int rank,
                                                               double2* __restrict__ S) {
  extern __shared__ double2 sm[];
  double2* sM = sm;                                  // rank x kTerms
  double2* sh = sm + (size_t)rank * kTerms;          // kTableKeys x kTerms
  for (int t = threadIdx.x; t < rank * kTerms; t += blockDim.x) sM[t] = M[t];
  const long long key0 = (long long)blockIdx.x * kTableKeys;
  const long long key = key0 + threadIdx.x;
  double2* h = sh + (size_t)threadIdx.x * kTerms;
  if (key < nkeys) {
    const double rx = ux[key / ny], ry = uy[key % ny];
    const double R2 = ry * ry + rx * rx;
    const double R = kappa * sqrt(R2);
    if (R > 0.0) {
      const double th = atan2(ry, rx);
      double J[kSeriesG + 1], Y[kSeriesG + 1];
      bessel_jy_all(R, J, Y);
      for (int n = -kSeriesG; n <= kSeriesG; ++n) {
        const int a = n < 0 ? -n : n;
        const bool neg = n < 0 && (a & 1);
        const double jn = neg ? -J[a] : J[a], yn = neg ? -Y[a] : Y[a];
        double s, c;
        sincos((double)n * th, &s, &c);
        h[n + kSeriesG] = make_double2(jn * c - yn * s, jn * s + yn * c);
      }
    } else {
      // Coincident points: never a far-field pair; the slot stays unused.
      for (int n = 0; n < kTerms; ++n) h[n] = make_double2(0.0, 0.0);
    }
  }
  __syncthreads();
  const long long nk = nkeys - key0 < kTableKeys ? nkeys - key0 : kTableKeys;
  for (long long o = threadIdx.x; o < nk * rank; o += blockDim.x) {
    const int kl = (int)(o / rank), node = (int)(o % rank);
    const double2* m = sM + (size_t)node * kTerms;
    const double2* hv = sh + (size_t)kl * kTerms;
    double sr = 0.0, si = 0.0;
    for (int n = 0; n < kTerms; ++n) {
      const double a = m[n].x, b = m[n].y, c = hv[n].x, d = hv[n].y;
      sr += a * c - b * d;
      si += a * d + b * c;
    }
    S[key0 * rank + o] = make_double2(sr, si);
  }
}

struct NcaGeomDev {
  const double2* S;
  const int *xid, *yid, *xrow, *yrow, *lcol, *lrow;
  const double* kq;
  int rank, ncol, ny, findPhi;
};

__device__ __forceinline__ double2 far_entry(const NcaGeomDev& g, int i, int j) {
  const int leaf = j / g.rank, node = j - leaf * g.rank;
  const int xi = g.xid[(size_t)g.xrow[i] * g.ncol + g.lcol[leaf]];
  const int yi = g.yid[(size_t)g.yrow[i] * g.ncol + g.lrow[leaf]];
  const double2 s = g.S[((size_t)xi * g.ny + yi) * g.rank + node];
  // s * (i/4), then the LS scaling (the host's entry()).
  double re = -(s.y * 0.25), im = s.x * 0.25;
  if (g.findPhi) {
    const double k = g.kq[i];
    re *= k;
    im *= k;
    if (i == j) re += 1.0;
  }
  return make_double2(re, im);
}

// Threads of one NCA block (a CTA of NT threads, 32 or 128): vectors are
// split over all of them; norms, dot products and the pivot search are
// block reductions.
template <int NT>
struct NcaShared {
  static constexpr int kWarps = NT / 32;
  double2 coef[kNcaRankCapG];  // coefficients of the current rank-1 updates
  double red[4][kWarps];       // per-warp partial sums
  int redi[kWarps];            // per-warp pivot candidates
  int task;
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Sums v[0..K) over the block; every thread gets the same bits (the warp
// sums are combined in warp order by each thread).
template <int K, int NT>
__device__ __forceinline__ void block_sum(double (&v)[K], NcaShared<NT>& sh) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < K; ++j) v[j] = warp_sum(v[j]);
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < K; ++j) sh.red[j][warp] = v[j];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < K; ++j) {
    double t = 0.0;
    for (int w = 0; w < NT / 32; ++w) t += sh.red[j][w];
    v[j] = t;
  }
  __syncthreads();
}

// First index of the largest |v| among the unused ones, 0 when all are used.
template <int NT>
__device__ int block_argmax(const double2* v, const unsigned char* used, int n, NcaShared<NT>& sh) {
  double best = -1.0;
  int bi = INT_MAX;
  for (int k = threadIdx.x; k < n; k += NT) {
    if (used[k]) continue;
    const double a = hypot(v[k].x, v[k].y);
    if (a > best) {
      best = a;
      bi = k;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(kFull, best, o);
    const int oi = __shfl_xor_sync(kFull, bi, o);
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh.red[0][warp] = best;
    sh.redi[warp] = bi;
  }
  __syncthreads();
  best = -1.0;
  bi = INT_MAX;
  for (int w = 0; w < NT / 32; ++w) {
    const double ob = sh.red[0][w];
    const int oi = sh.redi[w];
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  __syncthreads();
  return best < 0.0 ? 0 : bi;
}

__device__ __forceinline__ double cmag(double2 z) { return hypot(z.x, z.y); }

// Complex division by Smith's method (R. L. Smith, CACM 5(8), 1962).
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  const double r = b.x / b.y, den = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

// as_row: out[k] = K(rows[fixed], cols[k]), k < n2; else out[k] = K(rows[k], cols[fixed]), k < n1.
template <int NT>
__device__ __forceinline__ void fetch(const NcaGeomDev& g, const int* __restrict__ rows,
                                      const int* __restrict__ cols, int n1, int n2, bool as_row, int fixed,
                                      double2* __restrict__ out) {
  if (as_row) {
    const int i = rows[fixed];
#pragma unroll 4
    for (int k = threadIdx.x; k < n2; k += NT) out[k] = far_entry(g, i, cols[k]);
  } else {
    const int j = cols[fixed];
#pragma unroll 4
    for (int k = threadIdx.x; k < n1; k += NT) out[k] = far_entry(g, rows[k], j);
  }
}

// One NCA task by one block. The first vector fetched lives on domain D1
// (columns when the block has fewer rows than columns, rows otherwise),
// the second on D2; V holds the normalised D1 vectors, U the D2 ones.
// Every branch below depends only on values all threads hold alike.
template <int NT>
__device__ void aca_task(const NcaGeomDev& g, const NcaTask& tk, const int* idx, double eps, double2* scr,
                         unsigned char* used, int* piv, int* rank_out, int* status_out, NcaShared<NT>& sh) {
  const int tid = threadIdx.x;
  const int n1 = tk.n1, n2 = tk.n2, R = tk.R;
  const int* rows = idx + tk.idx_off;
  const int* cols = rows + n1;
  const bool rowfirst = n1 < n2;
  const int d1 = rowfirst ? n2 : n1, d2 = rowfirst ? n1 : n2;
  const int mn = n1 < n2 ? n1 : n2;
  double2* __restrict__ V = scr;                       // R x d1
  double2* __restrict__ U = V + (size_t)R * d1;        // R x d2
  double2* __restrict__ p = U + (size_t)R * d2;        // d1
  double2* __restrict__ q = p + d1;                    // d2
  unsigned char* used1 = used;
  unsigned char* used2 = used + d1;
  int* rb = piv + tk.out_off;
  int* cb = rb + R;
  int* list1 = rowfirst ? cb : rb;         // pivots on D1
  int* list2 = rowfirst ? rb : cb;         // pivots on D2
  for (int k = tid; k < d1 + d2; k += NT) used[k] = 0;
  __syncthreads();
  int i1 = 0, i2 = 0, l = 0;
  for (; l < d2; ++l) {
    i2 = l;
    __syncthreads();  // every thread has read p[i1] before p is refetched
    fetch<NT>(g, rows, cols, n1, n2, rowfirst, i2, p);
    __syncthreads();
    i1 = block_argmax(p, used1, d1, sh);
    if (cmag(p[i1]) > eps) break;
  }
  if (l == d2) {
    if (tid == 0) {
      *rank_out = 0;
      *status_out = 0;
    }
    return;
  }
  {
    const double2 pv = p[i1];
    for (int k = tid; k < d1; k += NT) V[k] = cdiv(p[k], pv);
  }
  fetch<NT>(g, rows, cols, n1, n2, !rowfirst, i1, q);
  __syncthreads();
  for (int k = tid; k < d2; k += NT) U[k] = q[k];
  if (tid == 0) {
    list1[0] = i1;
    list2[0] = i2;
    used1[i1] = 1;
    used2[i2] = 1;
  }
  __syncthreads();
  int rk = 1, status = 0;
  double nS = 0.0, prev = 1000.0;
  i2 = block_argmax(q, used2, d2, sh);
  while (cmag(p[i1]) > eps && cmag(q[i2]) > eps && fabs(prev - nS) >= eps * prev && rk < mn) {
    if (rk >= R) {
      status = 1;
      break;
    }
    __syncthreads();  // every thread has read p[i1] and q[i2] before they are refetched
    fetch<NT>(g, rows, cols, n1, n2, rowfirst, i2, p);
    // p[k] -= U[a][i2] V[a][k], a = 0..rk-1 in order (the host's sub_scaled
    // sequence for every element); the coefficients staged in shared memory.
    for (int a = tid; a < rk; a += NT) sh.coef[a] = U[(size_t)a * d2 + i2];
    __syncthreads();
    for (int k = tid; k < d1; k += NT) {
      double2 x = p[k];
#pragma unroll 4
      for (int a = 0; a < rk; ++a) {
        const double2 f = sh.coef[a], w = V[(size_t)a * d1 + k];
        x = make_double2(x.x - (f.x * w.x - f.y * w.y), x.y - (f.x * w.y + f.y * w.x));
      }
      p[k] = x;
    }
    __syncthreads();
    const int n_i1 = block_argmax(p, used1, d1, sh);
    double2* __restrict__ Vr = V + (size_t)rk * d1;
    {
      const double2 pv = p[n_i1];
      for (int k = tid; k < d1; k += NT) Vr[k] = cdiv(p[k], pv);
    }
    fetch<NT>(g, rows, cols, n1, n2, !rowfirst, n_i1, q);
    for (int a = tid; a < rk; a += NT) sh.coef[a] = V[(size_t)a * d1 + n_i1];
    __syncthreads();
    double2* __restrict__ Ur = U + (size_t)rk * d2;
    double nn[2] = {0.0, 0.0};
    for (int k = tid; k < d2; k += NT) {
      double2 x = q[k];
#pragma unroll 4
      for (int a = 0; a < rk; ++a) {
        const double2 f = sh.coef[a], w = U[(size_t)a * d2 + k];
        x = make_double2(x.x - (f.x * w.x - f.y * w.y), x.y - (f.x * w.y + f.y * w.x));
      }
      q[k] = x;
      Ur[k] = x;
      nn[0] += x.x * x.x + x.y * x.y;
    }
    for (int k = tid; k < d1; k += NT) nn[1] += Vr[k].x * Vr[k].x + Vr[k].y * Vr[k].y;
    block_sum<2>(nn, sh);  // also orders the writes of q, Ur before the reads below
    const double nu = sqrt(nn[0]), nv = sqrt(nn[1]);
    if (nu < 1e-8 || nv < 1e-8) break;
    i1 = n_i1;
    if (tid == 0) {
      list1[rk] = i1;
      list2[rk] = i2;
      used1[i1] = 1;
      used2[i2] = 1;
    }
    ++rk;
    if (rk != 2) prev = nS;
    nS = nS * nS + (nu * nv) * (nu * nv);
    for (int a = 0; a < rk; ++a) {
      // cu = sum conj(U[a]) Ur, cv = sum conj(V[a]) Vr
      double d4[4] = {0.0, 0.0, 0.0, 0.0};
      const double2* Ua = U + (size_t)a * d2;
      const double2* Va = V + (size_t)a * d1;
      for (int k = tid; k < d2; k += NT) {
        const double x = Ua[k].x, y = Ua[k].y, c = Ur[k].x, d = Ur[k].y;
        d4[0] += x * c + y * d;
        d4[1] += x * d - y * c;
      }
      for (int k = tid; k < d1; k += NT) {
        const double x = Va[k].x, y = Va[k].y, c = Vr[k].x, d = Vr[k].y;
        d4[2] += x * c + y * d;
        d4[3] += x * d - y * c;
      }
      block_sum<4>(d4, sh);
      const double prr = d4[0] * d4[2] - d4[1] * d4[3], pri = d4[0] * d4[3] + d4[1] * d4[2];
      nS += 2 * hypot(prr, pri);
    }
    nS = sqrt(nS);
    __syncthreads();
    i2 = block_argmax(q, used2, d2, sh);
  }
  if (tid == 0) {
    *rank_out = rk;
    *status_out = status;
  }
}

template <int NT>
__global__ void __launch_bounds__(NT) nca_kernel(NcaGeomDev g, const NcaTask* __restrict__ tasks, int ntasks,
                                                         const int* __restrict__ idx, double eps, int* next, int* piv,
                                                         int* ranks, int* status, double2* scratch,
                                                         long long blk_scr, unsigned char* flags,
                                                         long long blk_flags) {
  __shared__ NcaShared<NT> sh;
  double2* scr = scratch + (long long)blockIdx.x * blk_scr;
  unsigned char* used = flags + (long long)blockIdx.x * blk_flags;
  for (int iter = 0; iter <= ntasks; ++iter) {
    if (threadIdx.x == 0) sh.task = atomicAdd(next, 1);
    __syncthreads();
    const int t = sh.task;
    __syncthreads();
    if (t >= ntasks) break;
    aca_task<NT>(g, tasks[t], idx, eps, scr, used, piv, ranks + t, status + t, sh);
    __syncthreads();
  }
}

// Tiles of a phase from the far-field table (FillTile): one warp per tile,
// lane l writing column slot l of each 32-wide step, so a step is one
// contiguous 512-byte row.
__global__ void __launch_bounds__(256) table_fill_kernel(NcaGeomDev g, const FillTile* __restrict__ tiles,
                                                         long long ntiles, const int* __restrict__ rowpts,
                                                         const int* __restrict__ colpts, double2* __restrict__ A) {
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += nw) {
    const FillTile f = tiles[t];
    const int S = 1 << f.log2s, R = 32 >> f.log2s;
    const int sl = lane / R, r = lane - sl * R;
    const int i = r < f.rows ? rowpts[f.row_off + r] : 0;
    for (int q = 0; q < f.qmax; ++q) {
      const int k = q * S + sl;
      double2 v = make_double2(0.0, 0.0);
      if (r < f.rows && k < f.K) v = far_entry(g, i, colpts[f.col_off + k]);
      A[f.a_off + (long long)q * 32 + lane] = v;
    }
  }
}

template <class T>
bool upload(T** d, const std::vector<T>& h, cudaStream_t s) {
  *d = nullptr;
  if (h.empty()) return true;
  return cudaMallocAsync(reinterpret_cast<void**>(d), sizeof(T) * h.size(), s) == cudaSuccess &&
         cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s) == cudaSuccess;
}

template <class T>
bool alloc(T** d, size_t n, cudaStream_t s) {
  *d = nullptr;
  return cudaMallocAsync(reinterpret_cast<void**>(d), sizeof(T) * std::max<size_t>(n, 1), s) == cudaSuccess;
}

}  // namespace

// Device state of one assembly. Everything runs on a stream of its own with
// stream-ordered allocations, so an assembly on a host thread overlaps GPU
// work that other streams of the process (a solve) have in flight.
struct GpuFar {
  int device = -1;
  cudaStream_t stream = nullptr;
  NcaGeomDev g{};
  double2* S = nullptr;
  int *xid = nullptr, *yid = nullptr, *xrow = nullptr, *yrow = nullptr, *lcol = nullptr, *lrow = nullptr;
  double* kq = nullptr;
  ~GpuFar() {
    if (stream) {
      for (void* p : {(void*)S, (void*)xid, (void*)yid, (void*)xrow, (void*)yrow, (void*)lcol, (void*)lrow, (void*)kq})
        if (p) cudaFreeAsync(p, stream);
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    cudaGetLastError();
  }
};

GpuFar* gpu_far_open(int device, const FarTables& t, cd* S_host) {
  const long long nx = (long long)t.ux.size(), ny = (long long)t.uy.size();
  const long long nkeys = nx * ny;
  if (device < 0 || !S_host || nkeys <= 0 || t.rank < 1 || t.rank > 64 || (int)t.M.size() != t.rank * kTerms)
    return nullptr;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  GpuFar* f = new GpuFar();
  f->device = device;
  if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) {
    f->stream = nullptr;
    delete f;
    return nullptr;
  }
  cudaStream_t s = f->stream;
  const size_t sbytes = sizeof(double2) * (size_t)nkeys * t.rank;
  double *dux = nullptr, *duy = nullptr;
  double2* dM = nullptr;
  std::vector<double2> Mh(t.M.size());
  for (size_t i = 0; i < Mh.size(); ++i) Mh[i] = make_double2(t.M[i].real(), t.M[i].imag());
  const size_t smem = sizeof(double2) * ((size_t)t.rank * kTerms + (size_t)kTableKeys * kTerms);
  bool ok = upload(&dux, t.ux, s) && upload(&duy, t.uy, s) && upload(&dM, Mh, s) &&
            alloc(&f->S, (size_t)nkeys * t.rank, s) &&
            raise_smem_limit((const void*)far_table_kernel, (int)smem) == cudaSuccess;
  if (ok) {
    const long long blocks = (nkeys + kTableKeys - 1) / kTableKeys;
    far_table_kernel<<<(unsigned)blocks, kTableKeys, smem, s>>>(dux, duy, (int)ny, nkeys, t.kappa, dM, t.rank, f->S);
    static_assert(sizeof(cd) == sizeof(double2), "complex layout");
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(S_host, f->S, sbytes, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  }
  ok = ok && upload(&f->xid, t.xid, s) && upload(&f->yid, t.yid, s) && upload(&f->xrow, t.xrow, s) &&
       upload(&f->yrow, t.yrow, s) && upload(&f->lcol, t.lcol, s) && upload(&f->lrow, t.lrow, s) &&
       upload(&f->kq, t.kq, s);
  for (void* p : {(void*)dux, (void*)duy, (void*)dM})
    if (p) cudaFreeAsync(p, s);
  ok = cudaStreamSynchronize(s) == cudaSuccess && ok;
  if (!ok) {
    cudaGetLastError();
    delete f;
    return nullptr;
  }
  f->g = NcaGeomDev{f->S, f->xid, f->yid, f->xrow, f->yrow, f->lcol, f->lrow, f->kq, t.rank, t.ncol, (int)ny, t.findPhi};
  return f;
}

bool gpu_far_nca(GpuFar* f, const std::vector<NcaTask>& tasks, const std::vector<int>& idx, double eps,
                 std::vector<int>& ranks, std::vector<int>& piv, std::vector<int>& status) {
  if (!f || tasks.empty()) return f != nullptr;
  if (cudaSetDevice(f->device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaStream_t s = f->stream;
  const int nt = (int)tasks.size();
  long long blk_scr = 0, blk_flags = 0, npiv = 0;
  for (const NcaTask& t : tasks) {
    if (t.R < 1 || t.R > kNcaRankCapG) return false;
    const long long d = (long long)t.n1 + t.n2;
    blk_scr = std::max(blk_scr, (long long)t.R * d + d);
    blk_flags = std::max(blk_flags, d);
    npiv = std::max(npiv, (long long)t.out_off + 2LL * t.R);
  }
  blk_flags = (blk_flags + 15) / 16 * 16;
  // Threads per block: 128 when the level's blocks fill the GPU's CTAs of
  // 128 at most twice (few large blocks: the latency of each matters), else
  // 32 (many blocks: more of them in flight). CTAs: one per task up to the
  // resident ones (CTAs beyond those would find the task counter
  // exhausted) and an 8 GB scratch.
  int sms = 0, per128 = 0, per32 = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, f->device);
  sms = std::max(sms, 1);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per128, nca_kernel<128>, 128, 0) != cudaSuccess) per128 = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per32, nca_kernel<32>, 32, 0) != cudaSuccess) per32 = 1;
  const bool wide = nt <= 2LL * sms * std::max(per128, 1);
  long long blocks = std::min<long long>(nt, (long long)sms * std::max(wide ? per128 : per32, 1));
  const long long budget = 8LL << 30;
  blocks = std::max(1LL, std::min(blocks, budget / std::max(1LL, blk_scr * (long long)sizeof(double2))));
  NcaTask* dt = nullptr;
  int *didx = nullptr, *dnext = nullptr, *dpiv = nullptr, *drank = nullptr, *dstat = nullptr;
  double2* dscr = nullptr;
  unsigned char* dflags = nullptr;
  bool ok = upload(&dt, tasks, s) && upload(&didx, idx, s) && alloc(&dnext, 1, s) &&
            cudaMemsetAsync(dnext, 0, sizeof(int), s) == cudaSuccess && alloc(&dpiv, (size_t)npiv, s) &&
            alloc(&drank, (size_t)nt, s) && alloc(&dstat, (size_t)nt, s) &&
            alloc(&dscr, (size_t)(blocks * blk_scr), s) && alloc(&dflags, (size_t)(blocks * blk_flags), s);
  if (ok) {
    if (wide)
      nca_kernel<128><<<(unsigned)blocks, 128, 0, s>>>(f->g, dt, nt, didx, eps, dnext, dpiv, drank, dstat, dscr,
                                                       blk_scr, dflags, blk_flags);
    else
      nca_kernel<32><<<(unsigned)blocks, 32, 0, s>>>(f->g, dt, nt, didx, eps, dnext, dpiv, drank, dstat, dscr,
                                                     blk_scr, dflags, blk_flags);
    ok = cudaGetLastError() == cudaSuccess;
  }
  if (ok) {
    ranks.resize(nt);
    status.resize(nt);
    piv.resize((size_t)std::max(1LL, npiv));
    ok = cudaMemcpyAsync(ranks.data(), drank, sizeof(int) * nt, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
         cudaMemcpyAsync(status.data(), dstat, sizeof(int) * nt, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
         cudaMemcpyAsync(piv.data(), dpiv, sizeof(int) * npiv, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  }
  for (void* p : {(void*)dt, (void*)didx, (void*)dnext, (void*)dpiv, (void*)drank, (void*)dstat, (void*)dscr,
                  (void*)dflags})
    if (p) cudaFreeAsync(p, s);
  ok = cudaStreamSynchronize(s) == cudaSuccess && ok;
  cudaGetLastError();
  return ok;
}

void gpu_far_close(GpuFar* f) { delete f; }

void* gpu_far_fill(GpuFar* f, const std::vector<FillTile>& tiles, const std::vector<int>& rowpts,
                   const std::vector<int>& colpts, long long elems) {
  if (!f || tiles.empty() || elems <= 0) return nullptr;
  // Every tile inside A and its point lists (the kernel does not check).
  for (const FillTile& t : tiles) {
    const int R = 32 >> t.log2s;
    if (t.log2s < 0 || t.log2s > 5 || t.rows < 1 || t.rows > R || t.K < 1 || t.qmax < 1 ||
        t.qmax != (t.K + (1 << t.log2s) - 1) >> t.log2s || t.a_off < 0 || t.a_off + 32LL * t.qmax > elems ||
        t.row_off < 0 || t.row_off + t.rows > (long long)rowpts.size() || t.col_off < 0 ||
        t.col_off + t.K > (long long)colpts.size())
      return nullptr;
  }
  if (cudaSetDevice(f->device) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  cudaStream_t s = f->stream;
  double2* A = nullptr;
  if (cudaMalloc(&A, sizeof(double2) * (size_t)elems) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  FillTile* dt = nullptr;
  int *dr = nullptr, *dc = nullptr;
  bool ok = upload(&dt, tiles, s) && upload(&dr, rowpts, s) && upload(&dc, colpts, s);
  if (ok) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, f->device);
    const long long nt = (long long)tiles.size();
    const long long blocks = std::max(1LL, std::min((nt + 7) / 8, (long long)std::max(sms, 1) * 16));
    table_fill_kernel<<<(unsigned)blocks, 256, 0, s>>>(f->g, dt, nt, dr, dc, A);
    ok = cudaGetLastError() == cudaSuccess;
  }
  for (void* p : {(void*)dt, (void*)dr, (void*)dc})
    if (p) cudaFreeAsync(p, s);
  ok = cudaStreamSynchronize(s) == cudaSuccess && ok;
  if (!ok) {
    cudaFree(A);
    cudaGetLastError();
    return nullptr;
  }
  return A;
}

void gpu_far_free(void* p) {
  if (p) cudaFree(p);
}

}  // namespace lsg
